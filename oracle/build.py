"""ORACLE build (test infrastructure only): compiles the CPU restatement into
oracle/_build/libbarnacle_oracle.so with g++ -ffp-contract=off.

The reference itself is F# on .NET 9 and cannot be built here (no dotnet SDK), so there is no
oracle/_ref build; the restatement is the oracle.
"""
from __future__ import annotations

import subprocess
import sys
from pathlib import Path

HERE = Path(__file__).resolve().parent
SRC = HERE / "src"
OUT = HERE / "_build" / "libbarnacle_oracle.so"


HOST_SRC = HERE.parent / "barnacle_gb300" / "csrc" / "host"
SCENES = HERE / "_build" / "libbarnacle_scenes.so"


def build_scenes(verbose: bool = False) -> Path:
    """The library's host-side scene code alone (procedural workloads, JSON loader, BVH builder),
    without any CUDA: the CPU arms of the benchmark build their scenes with it and so load nothing
    of the GPU library."""
    OUT.parent.mkdir(parents=True, exist_ok=True)
    srcs = sorted(HOST_SRC.glob("*.cpp"))
    deps = srcs + sorted(HOST_SRC.glob("*.hpp")) + [HERE.parent / "include" / "barnacle_gpu.h"]
    if SCENES.exists() and SCENES.stat().st_mtime >= max(p.stat().st_mtime for p in deps):
        return SCENES
    tmp = SCENES.with_suffix(".so.tmp")
    cmd = ["g++", "-O2", "-std=c++17", "-fPIC", "-shared", "-pthread", "-ffp-contract=off",
           "-I", str(HERE.parent / "include"), *map(str, srcs), "-o", str(tmp)]
    if verbose:
        print(" ".join(cmd), flush=True)
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"scene library build failed\n{r.stdout}\n{r.stderr}")
    tmp.replace(SCENES)
    return SCENES


def build(verbose: bool = False) -> Path:
    OUT.parent.mkdir(parents=True, exist_ok=True)
    srcs = sorted(SRC.glob("*.cpp"))
    deps = srcs + sorted(SRC.glob("*.h*")) + [HERE.parent / "include" / "barnacle_gpu.h"]
    if OUT.exists() and OUT.stat().st_mtime >= max(p.stat().st_mtime for p in deps):
        build_scenes(verbose)
        return OUT
    tmp = OUT.with_suffix(".so.tmp")
    cmd = ["g++", "-O2", "-std=c++17", "-fPIC", "-shared", "-pthread", "-ffp-contract=off", "-fno-fast-math",
           "-I", str(HERE.parent / "include"), *map(str, srcs), "-o", str(tmp)]
    if verbose:
        print(" ".join(cmd), flush=True)
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"oracle build failed\n{r.stdout}\n{r.stderr}")
    tmp.replace(OUT)
    build_scenes(verbose)
    return OUT


if __name__ == "__main__":
    print(build(verbose="-v" in sys.argv))
