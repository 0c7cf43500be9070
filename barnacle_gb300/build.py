"""Builds libbarnacle_gb300.so in-tree with nvcc for sm_103a (no cmake, no torch).

Host C++ (scene preparation, BVH builder, loaders) is compiled by g++ with -ffp-contract=off:
the builder and the instance bounds must produce the reference's float bits, so no multiply-add
may be fused behind the code's back.  Device code is compiled for sm_103a only; the kernels spell
out every non-fused operation with __fadd_rn/__fmul_rn, so nvcc's default --fmad=true is kept.
Translation units compile in parallel; an object is rebuilt when any source or header is newer.
"""
from __future__ import annotations

import os
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor
from pathlib import Path

PKG = Path(__file__).resolve().parent
CSRC = PKG / "csrc"
BUILD = PKG / "_build"
LIB = PKG / "_lib" / "libbarnacle_gb300.so"
ROOT = PKG.parent

NVCC = os.environ.get("NVCC", "nvcc")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
CXXFLAGS = ["-O2", "-std=c++17", "-fPIC", "-ffp-contract=off", "-Wall", "-Wno-unused-function"]
NVFLAGS = ARCH + ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC", "-Xcompiler", "-ffp-contract=off",
                  "--expt-relaxed-constexpr", "-Xptxas", "-warn-spills"]


def _sources() -> list[Path]:
    return sorted(p for p in CSRC.rglob("*") if p.suffix in (".cu", ".cpp"))


def _headers() -> list[Path]:
    hs = [p for p in CSRC.rglob("*") if p.suffix in (".h", ".hpp", ".cuh")]
    hs.append(ROOT / "include" / "barnacle_gpu.h")
    return hs


def _compile(src: Path, newest_header: float, verbose: bool) -> Path:
    obj = BUILD / (src.relative_to(CSRC).as_posix().replace("/", "__") + ".o")
    if obj.exists() and obj.stat().st_mtime >= max(src.stat().st_mtime, newest_header):
        return obj
    if src.suffix == ".cpp":
        cmd = ["g++", *CXXFLAGS, "-I", str(ROOT / "include"), "-c", str(src), "-o", str(obj)]
    else:
        cmd = [NVCC, *NVFLAGS, "-I", str(ROOT / "include"), "-c", str(src), "-o", str(obj)]
    if verbose:
        print(" ".join(cmd), flush=True)
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"compile failed: {src}\n{r.stdout}\n{r.stderr}")
    if r.stderr.strip() and verbose:
        print(r.stderr, file=sys.stderr)
    return obj


def build(verbose: bool = False, jobs: int | None = None) -> Path:
    BUILD.mkdir(parents=True, exist_ok=True)
    LIB.parent.mkdir(parents=True, exist_ok=True)
    srcs = _sources()
    newest_header = max(h.stat().st_mtime for h in _headers())
    jobs = jobs or min(len(srcs), os.cpu_count() or 4)
    with ThreadPoolExecutor(max_workers=jobs) as ex:
        objs = list(ex.map(lambda s: _compile(s, newest_header, verbose), srcs))
    if LIB.exists() and LIB.stat().st_mtime >= max(o.stat().st_mtime for o in objs):
        return LIB
    tmp = LIB.with_suffix(".so.tmp")
    cmd = [NVCC, *ARCH, "-shared", "-o", str(tmp), *map(str, objs), "-lpthread"]
    if verbose:
        print(" ".join(cmd), flush=True)
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"link failed\n{r.stdout}\n{r.stderr}")
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(verbose="-v" in sys.argv))
