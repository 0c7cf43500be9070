"""Generates the fixtures that tie the render path to the reference's own scene and output:

* tests/golden/scenes/cbox.json — the reference's scene asset (Asset/cbox.json), byte for byte:
  the smallpt-style Cornell box (two spheres, a cube, a quad light, a thin-lens camera, PSSMLT at
  1024x768) the reference's JSON loader (Extensions/Scene/Loader.fs:241-281) was written for;
* tests/golden/cbox_samples.npz — the two sample images shipped with the reference ("Sample - Path
  Tracing.png", "Sample - Primary Sample Space Metropolis Light Transport.png", 1024x768 RGBA8,
  tone-mapped with ACES by Film.Save, Base/Film.fs:21-30,55-66), reduced to the means of their
  16x16 blocks (48 x 64 x 3, 8-bit units).  Their render settings were not recorded, so they pin
  the renders only coarsely (block means, a PSNR bound).

The reference is read from the directory given (default: the checkout next to this repository);
the GPU machines never need it.

    python tests/golden/make_cbox_fixture.py [/path/to/reference]
"""
from __future__ import annotations

import struct
import sys
import zlib
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
BLOCK = 16
SAMPLES = {"pt": "Sample - Path Tracing.png",
           "pssmlt": "Sample - Primary Sample Space Metropolis Light Transport.png"}


def decode_png(data: bytes) -> np.ndarray:
    """8-bit RGB/RGBA, non-interlaced PNG -> (H, W, C) uint8 (the PNG specification's filters)."""
    assert data[:8] == b"\x89PNG\r\n\x1a\n"
    i, idat, hdr = 8, b"", None
    while i < len(data):
        n, = struct.unpack(">I", data[i:i + 4])
        kind, body = data[i + 4:i + 8], data[i + 8:i + 8 + n]
        if kind == b"IHDR":
            hdr = struct.unpack(">IIBBBBB", body)
        elif kind == b"IDAT":
            idat += body
        i += 12 + n
    w, h, depth, ctype, _, _, interlace = hdr
    assert depth == 8 and ctype in (2, 6) and interlace == 0
    ch = 3 if ctype == 2 else 4
    raw = np.frombuffer(zlib.decompress(idat), np.uint8).reshape(h, 1 + w * ch)
    out = np.zeros((h, w * ch), np.int32)
    prev = np.zeros(w * ch, np.int32)
    for y in range(h):
        f, line = raw[y, 0], raw[y, 1:].astype(np.int32)
        cur = np.zeros(w * ch, np.int32)
        if f == 0:
            cur = line
        elif f == 2:
            cur = (line + prev) & 255
        else:
            for x in range(w * ch):
                a = cur[x - ch] if x >= ch else 0
                b = prev[x]
                c = prev[x - ch] if x >= ch else 0
                if f == 1:
                    p = a
                elif f == 3:
                    p = (a + b) // 2
                else:  # Paeth
                    pa, pb, pc = abs(b - c), abs(a - c), abs(a + b - 2 * c)
                    p = a if pa <= pb and pa <= pc else (b if pb <= pc else c)
                cur[x] = (line[x] + p) & 255
        out[y] = cur
        prev = cur
    return out.reshape(h, w, ch).astype(np.uint8)


def block_means(rgb: np.ndarray) -> np.ndarray:
    h, w = rgb.shape[:2]
    x = rgb[:, :, :3].astype(np.float64).reshape(h // BLOCK, BLOCK, w // BLOCK, BLOCK, 3)
    return x.mean((1, 3)).astype(np.float32)


def main():
    ref = Path(sys.argv[1]) if len(sys.argv) > 1 else HERE.parents[2] / "reference"
    (HERE / "scenes").mkdir(exist_ok=True)
    (HERE / "scenes" / "cbox.json").write_bytes((ref / "Asset" / "cbox.json").read_bytes())
    out = {}
    for k, name in SAMPLES.items():
        img = decode_png((ref / name).read_bytes())
        out[k] = block_means(img)
        print(k, img.shape, out[k].shape, float(out[k].mean()))
    np.savez_compressed(HERE / "cbox_samples.npz", **out)


if __name__ == "__main__":
    main()
