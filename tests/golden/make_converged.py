"""Generates tests/golden/converged.npz: converged oracle images of small crops, the reference
the device images are checked against (tests/test_gpu_converged.py).

Each crop is rendered by the oracle (the CPU restatement of PathTracingIntegrator.Li,
Extensions/Integrator/PathTracing.fs:14-81, with ProgressiveIntegrator's per-pixel seeds,
Base/Integrator.fs:22-44) at 65,536 samples per pixel: 16 independent ranges of 4,096 samples
(frame ids 100000..100015, far from any frame a test renders), averaged in FP64 (a range whose
pixel is NaN is left out of that pixel's mean).  Beside each image ("<key>:var") the per-sample
variance of every pixel, estimated from the spread of the 16 range means.

    python tests/golden/make_converged.py [--threads N]
"""
from __future__ import annotations

import argparse
import os
import sys
import time
from concurrent.futures import ThreadPoolExecutor
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
sys.path.insert(0, str(HERE.parent.parent))

from barnacle_gb300 import Bundle, capi  # noqa: E402
from oracle import pyoracle  # noqa: E402

CONVERGED, RANGES, FRAME0 = 65536, 16, 100000
# (workload, view index, crop (x0, y0, x1, y1) in the render's pixel coordinates, y up)
# "cbox" is the reference's own scene (tests/golden/scenes/cbox.json) rendered with the path tracer
CASES = [
    ("cbox", 0, (330, 252, 346, 268)),
    ("cbox", 0, (680, 152, 696, 168)),
    ("cbox", 0, (100, 452, 116, 468)),
    ("cornell", 0, (96, 120, 112, 136)),
    ("cornell-objects", 0, (240, 260, 252, 272)),
    ("instances", 4, (150, 134, 166, 150)),
    ("instances", 7, (300, 224, 316, 240)),
    ("instances", 1, (220, 164, 236, 180)),
]


def key(name, vi, crop):
    return f"{name}:{vi}:{crop[0]},{crop[1]},{crop[2]},{crop[3]}"


def crop_of(img, v, crop):
    x0, y0, x1, y1 = crop
    return img[v.height - y1:v.height - y0, x0:x1]  # Film.Pixels rows are flipped


def load(name):
    """The workload's bundle and its path-tracing render settings."""
    if name == "cbox":
        b = Bundle.load_json(str(HERE / "scenes" / "cbox.json"))
    else:
        b = Bundle.generate(name, 1)
    r = b.render
    r.integrator = capi.BN_INTEGRATOR_PATH
    return b, r


def converged(o, r, v, crop, threads):
    def one(f):
        rr = capi.bn_render_desc.from_buffer_copy(r)
        rr.spp = CONVERGED // RANGES
        rr.frame_id = f
        return crop_of(o.render_pt(rr, v, crop=crop, threads=1)[0], v, crop)
    with ThreadPoolExecutor(max_workers=threads) as ex:
        frames = np.stack(list(ex.map(one, range(FRAME0, FRAME0 + RANGES)))).astype(np.float64)
    # a path can end in NaN as in the reference (e.g. a PBR sample at a grazing wo with wo.z = 0
    # exactly: G = 0 and |wo.z| = 0 make specularBSDF 0/0, PBR.fs:47); such a range's pixel is left
    # out of that pixel's mean, as a NaN pixel of the reference's film carries no radiance.
    # The variance of one sample is estimated from the spread of the range means (4,096 samples
    # each, so rare bright paths are represented in every range).
    per_sample_var = np.nanvar(frames, 0, ddof=1) * (CONVERGED // RANGES)
    return np.nanmean(frames, 0), per_sample_var


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--threads", type=int, default=os.cpu_count() or 4)
    ap.add_argument("--only", default="", help="recompute only the cases of this workload, keep the others")
    args = ap.parse_args()
    path = HERE / "converged.npz"
    out = dict(np.load(path)) if args.only and path.exists() else {}
    for name, vi, crop in CASES:
        if args.only and name != args.only:
            continue
        b, r = load(name)
        o = pyoracle.Scene(b.scene)
        t0 = time.time()
        img, var = converged(o, r, b.views[vi], crop, args.threads)
        out[key(name, vi, crop)] = img
        out[key(name, vi, crop) + ":var"] = var
        print(f"{key(name, vi, crop)}: mean {img.mean():.4f}, {time.time() - t0:.1f} s", flush=True)
    np.savez_compressed(path, **out)


if __name__ == "__main__":
    main()
