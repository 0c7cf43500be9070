"""Benchmark of the render call on the 1,024-instance, 16-view workload.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--mode wavefront|megakernel]
                  [--impl reference] [--spp-per-step S] [--workload instances|cornell]

A step renders every one of the 16 views (256x240 ... 1920x1080, 14.66 M pixels) at the
workload's 64 samples per pixel in ONE launch (938 M paths), max depth 12, Russian roulette from
depth 3, the alias-table light sampler over the 64 emissive triangles.  The scene (630 k unique /
163 M instanced triangles, 1,089 instances) is resident in HBM; L2 is flushed (a 512 MiB write)
before every timed step.  --workload cornell times the Cornell box instead (256x256, one 64-spp
render per step, depth 8).

value  = paths / device time (CUDA events on the library's stream around its kernels).
e2e    = the same metric through bn_render with a host output buffer: the views' descriptors
         go host->device and the FP32 film comes back device->host inside the timed region.
compare: the plain megakernel in the reference's order (trace every shadow ray, then evaluate),
         the megakernel that traces only shadow rays that can change the radiance (the test the
         wavefront applies), and the wavefront with the watertight triangle test; each timed the
         same way on the same step (fewer steps: --compare-steps).
roofline: the dominant kernel's algorithmic bytes (32 per BVH node tested, 48 per triangle
         tested, 152 per instance visited, counted by an instrumented run of the same step) over
         its event-timed duration, against the measured HBM copy bandwidth; traffic = DRAM bytes
         per ray from an ncu capture (profiles/roofline_<workload>.json) x the step's rays.
--impl reference: the CPU restatement of the reference path (the F# renderer cannot be built
         here) on all host cores; each step renders two 16x16 tiles of every view (tile positions
         stratified over a 4x4 grid per view, different cells every step) at the step's spp.
Multi-GPU (torchrun): every rank renders the full workload (replicas, weak scaling).
"""
from __future__ import annotations

import argparse
import ctypes as C
import json
import os
import statistics
import subprocess
import sys
import threading
import time
from concurrent.futures import ThreadPoolExecutor
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

METRIC = "paths/sec at equal image RMSE: batched wavefront vs plain megakernel; adjoint/fwd"
# name -> (description, samples per pixel per step (the workload's spp in one launch), CPU tiles
# per view per step)
WORKLOADS = {
    "instances": ("instances: 1024 instances of 4 displaced icospheres (20k/82k/200k/328k tris) + 64 emissive "
                  "triangles, 16 views 256x240..1920x1080, 64 spp in one launch, depth 12, rr 3", 64, 2),
    "cornell": ("cornell: procedural Cornell box (24 triangles, two rotated boxes, ceiling light), 256x256, "
                "64 spp, depth 8", 64, 16),
}
TILE = 16


def bytes_per_unit():
    return {"node": 32, "triangle": 48, "instance": 152}


def measured_peak_gbs():
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        try:
            return float(json.loads(p.read_text())["hbm_gbs"]), "measured"
        except Exception:
            pass
    return 6800.0, "fallback"


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled every 200 ms during the timed region."""

    FIELDS = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.hw_slowdown,"
              "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
              "clocks_event_reasons.sw_power_cap")

    def __init__(self, index: int):
        self.index = index
        self.rows = []
        self.proc = None

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.index), f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits",
                 "-lms", "200"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
        except FileNotFoundError:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            parts = [p.strip() for p in line.split(",")]
            if len(parts) == 7:
                self.rows.append(parts)

    def __exit__(self, *exc):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self):
        if not self.rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}
        sm = [float(r[0]) for r in self.rows if r[0].replace(".", "").isdigit()]
        mx = [float(r[1]) for r in self.rows if r[1].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[k] for r in self.rows for k in range(4) if r[3 + k].lower() == "active"})
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": reasons, "samples": len(self.rows)}


def dist_setup():
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    dist = None
    if world > 1:
        import torch
        import torch.distributed as dist
        backend = "nccl" if torch.cuda.is_available() else "gloo"
        if backend == "nccl":
            torch.cuda.set_device(local)
        dist.init_process_group(backend)
    return world, rank, local, dist


def barrier(dist):
    if dist is not None:
        dist.barrier()


def max_over_ranks(dist, x: float) -> float:
    if dist is None:
        return x
    import torch
    dev = "cuda" if torch.cuda.is_available() and dist.get_backend() == "nccl" else "cpu"
    t = torch.tensor([x], dtype=torch.float64, device=dev)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def workload_config(args, views, world):
    """The configuration both arms report (the GPU arm and --impl reference): the same workload."""
    return {"workload": WORKLOADS[args.workload][0], "views": len(views),
            "pixels_per_step": int(sum(v.width * v.height for v in views)), "spp_per_step": args.spp_per_step,
            "paths_per_step": int(sum(v.width * v.height for v in views)) * args.spp_per_step,
            "parallelism": "replicas" if world > 1 else "single",
            "l2": "GPU arm: flushed before every timed step (512 MiB write)"}


def cpu_tiles(views, step, per_view):
    """Tiles of one CPU step: per view, per_view 16x16 tiles at cells of a 4x4 grid over the view,
    a different cell every step (the cells of all views are covered every 16 steps)."""
    out = []
    for vi, v in enumerate(views):
        for j in range(per_view):
            c = (step * per_view + j + 5 * vi) % 16
            cx, cy = c % 4, c // 4
            x0 = min(max(0, int((cx + 0.5) * v.width / 4) - TILE // 2), v.width - TILE)
            y0 = min(max(0, int((cy + 0.5) * v.height / 4) - TILE // 2), v.height - TILE)
            out.append((vi, (x0, y0, x0 + TILE, y0 + TILE)))
    return out


def cpu_sample_render(osc, render, spp, views, tiles, threads):
    """Times the oracle (CPU restatement) on the given tiles, one tile per host thread at a time;
    returns (paths, seconds)."""
    r = render
    r.spp = spp

    def one(t):
        vi, crop = t
        osc.render_pt(r, views[vi], crop=crop, threads=1)

    t0 = time.perf_counter()
    with ThreadPoolExecutor(max_workers=threads) as ex:
        list(ex.map(one, tiles))
    secs = time.perf_counter() - t0
    paths = sum((c[2] - c[0]) * (c[3] - c[1]) for _, c in tiles) * spp
    return paths, secs


def run_extras(ctx, args, torch, flush):
    """The other parts of the metric, each on its own workload (device-timed, L2 flushed first):
    the Cornell box (256^2, 64 spp, depth 8) against the CPU path on this host; PSSMLT (1024^2,
    2^20 bootstrap paths, 65,536 chains, 16 mutations per pixel, Kelemen(1/1024, 1/64), depth 16);
    adjoint / forward cost on the 32-slot material workload (256^2, 16 spp, depth 8)."""
    from barnacle_gb300 import Bundle, capi
    from barnacle_gb300.inverse import MaterialProblem
    from oracle import pyoracle

    out = {}
    # Cornell box: plain megakernel vs the CPU restatement (same workload, bounded CPU sample)
    c0 = Bundle.generate("cornell", 1)
    c0.scene.contents.bvh_width = args.bvh_width
    ctx.upload(c0)
    r0 = c0.render
    r0.mode = capi.BN_MODE_MEGAKERNEL
    v0 = c0.views
    for k in range(3):
        r0.frame_id = k
        ctx.render(r0, v0, to_host=False)
    ms = []
    for k in range(3):
        flush.zero_()
        torch.cuda.synchronize()
        r0.frame_id = 10 + k
        ctx.render(r0, v0, to_host=False)
        ms.append(ctx.stats().last_kernel_ms)
    paths0 = v0[0].width * v0[0].height * r0.spp
    gpu0 = paths0 / (min(ms) / 1000.0)
    threads = os.cpu_count() or 1
    tiles = [t for k in range(2) for t in cpu_tiles(v0, k, 16)]
    pc, sc = cpu_sample_render(pyoracle.Scene(c0.scene), c0.render, 64, v0, tiles, threads)
    out["cornell"] = {"gpu_paths_per_s": gpu0, "gpu_ms": min(ms), "cpu_paths_per_s": pc / sc, "cpu_cores": threads,
                      "cpu_sample": f"{len(tiles)} 16x16 tiles x 64 spp (every cell of a 4x4 grid, twice)",
                      "gpu_over_cpu": gpu0 / (pc / sc)}
    # PSSMLT: the chains one thread each in lockstep, and compacted every bounce in the wavefront
    c3 = Bundle.generate("pssmlt", 1)
    ctx.upload(c3)
    out["pssmlt"] = {}
    for name, mode in (("lockstep", capi.BN_MODE_MEGAKERNEL), ("wavefront", capi.BN_MODE_WAVEFRONT)):
        r3 = c3.render
        r3.mode = mode
        r3.frame_id = 0
        ctx.render(r3, c3.views, to_host=False)
        flush.zero_()
        torch.cuda.synchronize()
        ctx.reset_stats()
        r3.frame_id = 1
        ctx.render(r3, c3.views, to_host=False)
        st = ctx.stats()
        out["pssmlt"][name] = {"ms": st.last_kernel_ms, "chain_ms": st.last_dominant_ms,
                               "proposals_per_s": st.proposed / (st.last_dominant_ms / 1000.0),
                               "paths_per_s": st.paths / (st.last_kernel_ms / 1000.0),
                               "acceptance": st.accepted / max(1, st.proposed), "b": st.bootstrap_b,
                               "launches": st.last_launches}
    out["pssmlt"]["workload"] = ("cornell-objects scene at 1024^2, 2^20 bootstrap paths, 65,536 chains, 16 mutations "
                                 "per pixel, Kelemen(1/1024, 1/64), p_large 0.3, depth 16")
    # adjoint / forward
    c4 = Bundle.generate("materials", 1)
    pb = MaterialProblem(ctx, c4, width=256, height=256, spp=16, max_depth=8)
    target = pb.render(c4.slot_params(), spp=16, frame=1)
    theta = pb.random_params(2)
    fwd, bwd = [], []
    for k in range(3):
        flush.zero_()
        torch.cuda.synchronize()
        pb.render(theta, frame=2 + k)
        fwd.append(ctx.stats().last_kernel_ms)
        flush.zero_()
        torch.cuda.synchronize()
        pb.loss_and_grad(theta, target, frame=2 + k)
        bwd.append(ctx.stats().last_kernel_ms)
    out["adjoint"] = {"forward_ms": min(fwd), "backward_ms": min(bwd), "backward_over_forward": min(bwd) / min(fwd),
                      "workload": "materials 256^2 x 16 spp, depth 8, 32 slots (forward + loss + replay)"}
    # the inverse-material task: 200 Adam steps at lr 1e-2 from random parameters against a
    # 1,024-spp target of the ground-truth parameters (256^2, 16 spp per step, depth 8)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    gt = c4.slot_params()
    target = pb.render(gt, spp=1024, frame=9000)
    x0 = pb.random_params(7)
    x, losses = pb.adam(x0, target, steps=200, lr=1e-2)
    wall = time.perf_counter() - t0
    names = ["albedo_r", "albedo_g", "albedo_b", "roughness", "metallic", "emission_scale"]

    def err(p):
        d = (p - gt).reshape(-1, 6)
        rows = np.arange(len(d))
        e = {n: float(np.sqrt((d[:, k] ** 2).mean())) for k, n in enumerate(names[:5])}
        em = rows >= c4.emissive_slot_base
        e["emission_scale"] = float(np.sqrt((d[em, 5] ** 2).mean())) if em.any() else 0.0
        e["all"] = float(np.sqrt((d[:, :5] ** 2).mean()))
        return e

    fin = [v for v in losses if np.isfinite(v)]
    out["inverse"] = {"steps": 200, "lr": 1e-2, "target_spp": 1024, "step_spp": 16, "wall_s": wall,
                      "skipped_nan_steps": len(losses) - len(fin),
                      "loss_first": fin[0] if fin else None, "loss_last": fin[-1] if fin else None,
                      "loss_mean_last_20": float(np.mean(fin[-20:])) if fin else None,
                      "loss_curve": [losses[k] for k in range(0, 200, 20)] + [losses[-1]],
                      "param_rmse_initial": err(x0), "param_rmse_final": err(x),
                      "workload": "materials: 32 slots, 4 emissive, 256^2, depth 8"}
    return out


def run_reference(args, world, rank, dist):
    """--impl reference: the CPU restatement on all host threads, a bounded sample per step."""
    if rank != 0:
        return
    from barnacle_gb300 import Bundle
    from oracle import pyoracle

    # the scene from the host code alone (no GPU library is loaded by this arm)
    b = Bundle.generate(args.workload, 1, lib=pyoracle.scenes_library())
    views = select_views(b.views, args.views)
    osc = pyoracle.Scene(b.scene)
    threads = os.cpu_count() or 1
    per_view = WORKLOADS[args.workload][2]
    for k in range(args.warmup):
        cpu_sample_render(osc, b.render, args.spp_per_step, views, cpu_tiles(views, k, per_view), threads)
    paths, secs = 0, 0.0
    for k in range(args.steps):
        p, s = cpu_sample_render(osc, b.render, args.spp_per_step, views,
                                 cpu_tiles(views, args.warmup + k, per_view), threads)
        paths += p
        secs += s
    value = paths / secs
    ntiles = len(views) * per_view
    line = {"metric": METRIC, "value": value, "unit": "paths/s", "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": 1000 * secs / args.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded procedural scene)",
            "impl": "reference",
            "config": workload_config(args, views, world),
            "cpu_baseline": {"value": value, "unit": "paths/s", "cores": threads, "kind": "port",
                             "sample": f"per step {ntiles} 16x16 tiles ({per_view} per view, stratified over a 4x4 "
                                       f"grid per view, a different cell each step) x {args.spp_per_step} spp "
                                       f"(the F# reference cannot be built: no .NET SDK)"},
            "e2e": {"value": value, "unit": "paths/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def profile_figures(workload):
    """The ncu figures committed under profiles/roofline_<workload>.json: DRAM bytes per traced ray
    of the render's kernels and the L2 side of the dominant kernel, each with its source."""
    prof = ROOT / "profiles" / f"roofline_{workload}.json"
    if not prof.exists():
        return None
    return json.loads(prof.read_text())


def select_views(views, n):
    return views if n <= 0 else views[:n]


def run_profile_case(ctx, case, mode):
    """Small cases of the kernels outside the headline loop, for ncu (a few launches each, inputs
    of tens of MB): PSSMLT chains at 256^2 (65,536 chains, 16 mutations per pixel, depth 16) and
    the path-replay adjoint at 128^2 (16 spp, depth 8, 32 slots)."""
    from barnacle_gb300 import Bundle, capi
    from barnacle_gb300.inverse import MaterialProblem
    if case == "pssmlt":
        b = Bundle.generate("pssmlt", 1)
        ctx.upload(b)
        v = b.views[0]
        v.width, v.height = 256, 256
        r = b.render
        r.mode = capi.BN_MODE_WAVEFRONT if mode == "wavefront" else capi.BN_MODE_MEGAKERNEL
        if mode == "wavefront":
            r.flags |= capi.BN_RENDER_NO_GRAPH
        r.n_bootstrap = 1 << 18
        for f in range(2):
            r.frame_id = f
            ctx.render(r, v, to_host=False)
            st = ctx.stats()
            print(json.dumps({"case": case, "mode": mode, "frame": f, "ms": st.last_kernel_ms,
                              "chain_ms": st.last_dominant_ms}), flush=True)
    else:
        b = Bundle.generate("materials", 1)
        pb = MaterialProblem(ctx, b, width=128, height=128, spp=16, max_depth=8)
        target = pb.render(b.slot_params(), spp=16, frame=1)
        theta = pb.random_params(2)
        for f in range(2):
            pb.loss_and_grad(theta, target, frame=2 + f)
            print(json.dumps({"case": case, "frame": f, "ms": ctx.stats().last_kernel_ms}), flush=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=4)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--mode", default="wavefront", choices=["megakernel", "wavefront"])
    ap.add_argument("--no-compare", action="store_true", help="skip timing the other render forms")
    ap.add_argument("--compare-steps", type=int, default=2, help="timed steps of each comparison form (1 warm-up)")
    ap.add_argument("--workload", default="instances", choices=sorted(WORKLOADS))
    ap.add_argument("--views", type=int, default=0, help="render only the first N views (0 = all; small cases)")
    ap.add_argument("--spp-per-step", type=int, default=0, help="0 = the workload's spp (64) in one launch")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-extras", action="store_true",
                    help="skip the Cornell-box CPU ratio, PSSMLT and adjoint/forward measurements")
    ap.add_argument("--no-count", action="store_true", help="skip the instrumented visit-counting render")
    ap.add_argument("--pool", type=int, default=0, help="wavefront path slots (0 = autotuned)")
    ap.add_argument("--cap", type=int, default=0, help="wavefront blocks per SM cap (0 = autotuned)")
    ap.add_argument("--bvh-width", type=int, default=0, choices=[0, 2, 4],
                    help="BVH walk: 0 = auto (wide records for BVHs of 1,024+ nodes), 2 = binary, 4 = wide")
    ap.add_argument("--profile-case", choices=["pssmlt", "adjoint"], default=None,
                    help="run only a small case of the PSSMLT chains or the adjoint (for ncu) and exit")
    ap.add_argument("--no-graph", action="store_true",
                    help="wavefront bounce loop driven from the host (ncu cannot profile kernels inside a "
                         "graph with a conditional node)")
    args = ap.parse_args()
    if args.spp_per_step <= 0:
        args.spp_per_step = WORKLOADS[args.workload][1]
    world, rank, local, dist = dist_setup()
    if args.impl == "reference":
        run_reference(args, world, rank, dist)
        return
    import torch

    from barnacle_gb300 import Bundle, Context, capi

    dev = local if world > 1 else 0
    ctx = Context(dev)
    if args.profile_case:
        run_profile_case(ctx, args.profile_case, args.mode)
        ctx.close()
        return
    b = Bundle.generate(args.workload, 1)
    b.scene.contents.bvh_width = args.bvh_width
    ctx.upload(b)
    views = select_views(b.views, args.views)
    r = b.render
    r.spp = args.spp_per_step
    if args.no_graph:
        r.flags |= capi.BN_RENDER_NO_GRAPH
    r.queue_capacity = args.pool
    r.block_size = args.cap
    pixels = sum(v.width * v.height for v in views)
    paths_per_step = pixels * r.spp
    torch.cuda.set_device(dev)
    flush = torch.empty(512 * 1024 * 1024, dtype=torch.uint8, device=f"cuda:{dev}")

    primary = capi.BN_MODE_WAVEFRONT if args.mode == "wavefront" else capi.BN_MODE_MEGAKERNEL
    # algorithmic bytes per launch of the dominant kernel: an instrumented run of one step in the
    # timed form (the wavefront does not trace shadow rays that cannot change the radiance, so its
    # rays are counted on its own walk), visits counted in the reference's binary traversal order
    st = None
    if not args.no_count:
        rc = capi.bn_render_desc.from_buffer_copy(r)
        rc.flags |= capi.BN_RENDER_COUNT
        rc.mode = primary
        rc.frame_id = 100
        ctx.reset_stats()
        ctx.render(rc, views, to_host=False)
        st = ctx.stats()
    bpu = bytes_per_unit()
    alg_bytes = (bpu["node"] * st.nodes_visited + bpu["triangle"] * st.tris_tested +
                 bpu["instance"] * st.instances_visited) if st else 0
    rays_per_step = st.rays if st else 0

    def timed(mode, flags, frame_base, steps, warmup):
        rr = capi.bn_render_desc.from_buffer_copy(r)
        rr.mode = mode
        rr.flags |= flags
        for w in range(warmup):
            rr.frame_id = frame_base + w
            ctx.render(rr, views, to_host=False)
        barrier(dist)
        torch.cuda.synchronize()
        dev_ms, dom_ms, launches = 0.0, 0.0, 0
        t0 = time.perf_counter()
        for k in range(steps):
            flush.zero_()
            torch.cuda.synchronize()
            rr.frame_id = frame_base + 100 + k
            ctx.render(rr, views, to_host=False)
            s = ctx.stats()
            dev_ms += s.last_kernel_ms
            dom_ms += s.last_dominant_ms
            launches += s.last_launches
        torch.cuda.synchronize()
        wall = time.perf_counter() - t0
        barrier(dist)
        return max_over_ranks(dist, dev_ms / 1000.0), dom_ms, launches, wall

    with ClockSampler(dev) as clk:
        dev_s, dom_ms, launches, wall = timed(primary, 0, 0, args.steps, args.warmup)

    compare = None
    if not args.no_compare:
        cs = max(1, args.compare_steps)
        legs = [("megakernel", capi.BN_MODE_MEGAKERNEL, 0),
                ("megakernel_cull", capi.BN_MODE_MEGAKERNEL, capi.BN_RENDER_CULL_SHADOW),
                ("wavefront_watertight", capi.BN_MODE_WAVEFRONT, capi.BN_RENDER_WATERTIGHT)]
        if primary == capi.BN_MODE_MEGAKERNEL:
            legs = [("wavefront", capi.BN_MODE_WAVEFRONT, 0)] + legs[1:]
        compare = {"steps": cs, "warmup": 1}
        for k, (name, mode, flags) in enumerate(legs):
            s, _, _, _ = timed(mode, flags, 1000 * (k + 1), cs, 1)
            compare[name] = {"paths_per_s": world * paths_per_step * cs / s, "ms_per_step": 1000 * s / cs}
        this = world * paths_per_step * args.steps / dev_s
        for name in ("megakernel", "megakernel_cull"):
            if name in compare:
                compare[f"ratio_over_{name}"] = this / compare[name]["paths_per_s"]
        compare["equal_rmse"] = ("same per-path estimator and random streams in every form (images equal to float "
                                 "summation order, tests/test_gpu_wavefront.py; watertight differs from "
                                 "Moller-Trumbore only where a ray grazes an edge)")

    # end to end through the C-ABI with a host film (pinned): descriptors in, film out, every step
    rr = capi.bn_render_desc.from_buffer_copy(r)
    rr.mode = primary
    film = torch.empty(pixels * 3, dtype=torch.float32).pin_memory().numpy()
    view_arr = (capi.bn_view * len(views))(*views)
    e2e_steps = max(1, min(args.steps, 4))
    barrier(dist)
    t0 = time.perf_counter()
    for k in range(e2e_steps):
        rr.frame_id = 200 + k
        rcode = ctx.lib.bn_render(ctx._h, C.byref(rr), view_arr, len(views), capi.ptr(film))
        if rcode:
            raise RuntimeError(ctx.error())
        float(film[0])  # the step's result is on the host
    e2e_s = max_over_ranks(dist, time.perf_counter() - t0)

    peak, peak_kind = measured_peak_gbs()
    dom_launch_s = dom_ms / 1000.0 / args.steps
    achieved = alg_bytes / dom_launch_s / 1e9
    prof = profile_figures(args.workload) or {}
    traffic = None
    tr = prof.get("traffic", {}).get(args.mode)
    if tr and rays_per_step:
        traffic = {"bytes_per_launch": int(tr["dram_bytes_per_ray"] * rays_per_step),
                   "dram_bytes_per_ray": tr["dram_bytes_per_ray"], "source": tr["source"]}

    cpu = None
    if rank == 0 and not args.no_cpu_baseline:
        from oracle import pyoracle
        threads = os.cpu_count() or 1
        per_view = WORKLOADS[args.workload][2]
        tiles = [t for k in range(8) for t in cpu_tiles(views, k, per_view)]
        p, s = cpu_sample_render(pyoracle.Scene(b.scene), b.render, args.spp_per_step, views, tiles, threads)
        cpu = {"value": p / s, "unit": "paths/s", "cores": threads, "kind": "port",
               "sample": f"{len(tiles)} 16x16 tiles ({8 * per_view} per view, stratified over a 4x4 grid per view) "
                         f"x {args.spp_per_step} spp (oracle: CPU restatement of the F# path; the F# renderer "
                         "cannot be built here)"}

    extras = None
    if rank == 0 and not args.no_extras:
        extras = run_extras(ctx, args, torch, flush)

    if rank == 0:
        value = world * paths_per_step * args.steps / dev_s
        line = {
            "metric": METRIC, "value": value, "unit": "paths/s", "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": 1000 * dev_s / args.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded procedural scene)",
            "config": workload_config(args, views, world),
            "form": {"mode": args.mode, "bvh_width": {0: "auto", 2: "binary", 4: "wide"}[args.bvh_width],
                     "triangle_test": "watertight" if r.flags & capi.BN_RENDER_WATERTIGHT else "moller-trumbore",
                     "graph": not args.no_graph},
            "rays": {"per_step": int(rays_per_step),
                     "per_ray": None if not st else {
                         "nodes": st.nodes_visited / max(1, st.rays), "triangles": st.tris_tested / max(1, st.rays),
                         "instances": st.instances_visited / max(1, st.rays)}},
            "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                         "frac": achieved / peak, "traffic": None if traffic is None else traffic["bytes_per_launch"],
                         "traffic_source": None if traffic is None else traffic["source"], "peak_kind": peak_kind,
                         "kernel": "k_pt_mega" if args.mode == "megakernel" else
                                   "wavefront bounce loop (regen+sort+extend+shade+shadow, one graph launch)",
                         "alg_bytes_per_launch": int(alg_bytes), "l2": prof.get("l2", {}).get(args.mode)},
            "cpu_baseline": cpu,
            "e2e": {"value": world * paths_per_step * e2e_steps / e2e_s, "unit": "paths/s", "steps": e2e_steps,
                    "h2d_bytes_per_step": C.sizeof(capi.bn_view) * len(views),
                    "d2h_bytes_per_step": pixels * 3 * 4},
            "gpu_launches": launches,
            "clocks": clk.summary(),
            "mrays_per_s": world * rays_per_step * args.steps / dev_s / 1e6,
            "compare": compare,
            "wall_s": wall,
            "extras": extras,
        }
        print(json.dumps(line), flush=True)
    ctx.close()
    if dist is not None:
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
