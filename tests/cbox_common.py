"""The reference's own scene and sample images as test fixtures (made by
tests/golden/make_cbox_fixture.py): the scene file loaded unchanged through the JSON loader, and
the 16x16 block means of the two 1024x768 sample images the reference ships (ACES tone-mapped,
8-bit; render settings not recorded)."""
from pathlib import Path

import numpy as np

GOLDEN = Path(__file__).resolve().parent / "golden"
CBOX = GOLDEN / "scenes" / "cbox.json"
BLOCK = 16
# PSNR of 16x16 block means (8-bit units) a render of cbox.json must reach against the reference's
# sample images.  Measured with the oracle's path tracer against the path-tracing sample: 33.9 dB
# at 8 spp, 35.1 dB at 16 spp (tone-mapping a noisier image costs PSNR); at 8 spp the same render
# with the cube's and sphere's rotations read as degrees instead of radians gives 29.1 dB, with
# the light's emission 50 instead of 60 gives 23.3 dB.  Renders checked against it use >= 16 spp.
PSNR_MIN = 33.0


def samples():
    d = np.load(GOLDEN / "cbox_samples.npz")
    return {"pt": d["pt"], "pssmlt": d["pssmlt"]}


def block_means(rgba: np.ndarray) -> np.ndarray:
    h, w = rgba.shape[:2]
    x = rgba[:, :, :3].astype(np.float64).reshape(h // BLOCK, BLOCK, w // BLOCK, BLOCK, 3)
    return x.mean((1, 3))


def psnr(a: np.ndarray, b: np.ndarray) -> float:
    return float(10 * np.log10(255.0 ** 2 / ((a - b) ** 2).mean()))
