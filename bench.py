"""Benchmark of the render call on the 1,024-instance, 16-view workload.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--mode wavefront|megakernel]
                  [--impl reference] [--spp-per-step S] [--workload instances|cornell]

A step renders every one of the 16 views (256x240 ... 1920x1080, ~13 M pixels) at S samples per
pixel (the workload's 64 spp = 64 / S steps), max depth 12, Russian roulette from depth 3, the
alias-table light sampler over the 64 emissive triangles.  The scene (630 k unique / 163 M
instanced triangles, 1,089 instances) is resident in HBM; L2 is flushed (a 512 MiB write)
before every timed step.  --workload cornell times the Cornell box instead (256x256, one
64-spp render per step, depth 8).

value  = paths / device time (CUDA events on the library's stream around its kernels).
e2e    = the same metric through bn_render with a host output buffer: the views' descriptors
         go host->device and the FP32 film comes back device->host inside the timed region.
roofline: the dominant kernel's algorithmic bytes (32 per BVH node tested, 48 per triangle
         tested, 152 per instance visited, counted by an instrumented run of the same step) over
         its event-timed duration, against the measured HBM copy bandwidth.
--impl reference: the CPU restatement of the reference path (the F# renderer cannot be built
         here) on all host cores, each step a bounded sample of the same workload.
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
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

METRIC = "paths/sec at equal image RMSE: batched wavefront vs plain megakernel; adjoint/fwd"
# name -> (description, samples per pixel per step, CPU sample: views, crop, spp)
WORKLOADS = {
    "instances": ("instances: 1024 instances of 4 displaced icospheres (20k/82k/200k/328k tris) + 64 emissive "
                  "triangles, 16 views 256x240..1920x1080, depth 12, rr 3", 4, (4, 128, 24)),
    "cornell": ("cornell: procedural Cornell box (24 triangles, two rotated boxes, ceiling light), 256x256, "
                "depth 8", 64, (1, 96, 64)),
}


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


def cpu_sample_render(bundle, render, spp, views, crop_size, threads):
    """Times the oracle (CPU restatement) on crops of the given views; returns (paths, seconds)."""
    from oracle import pyoracle

    osc = pyoracle.Scene(bundle.scene)
    r = render
    r.spp = spp
    paths, secs = 0, 0.0
    for v in views:
        cw, ch = min(crop_size, v.width), min(crop_size, v.height)
        x0, y0 = (v.width - cw) // 2, (v.height - ch) // 2
        t0 = time.perf_counter()
        osc.render_pt(r, v, crop=(x0, y0, x0 + cw, y0 + ch), threads=threads)
        secs += time.perf_counter() - t0
        paths += cw * ch * spp
    return paths, secs


def run_extras(ctx, args, torch, flush):
    """The other parts of the metric, each on its own workload (device-timed, L2 flushed first):
    the Cornell box (256^2, 64 spp, depth 8) against the CPU path on this host; PSSMLT (1024^2,
    2^20 bootstrap paths, 65,536 chains, 16 mutations per pixel, Kelemen(1/1024, 1/64), depth 16);
    adjoint / forward cost on the 32-slot material workload (256^2, 16 spp, depth 8)."""
    from barnacle_gb300 import Bundle, capi
    from barnacle_gb300.inverse import MaterialProblem

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
    pc, sc = cpu_sample_render(c0, c0.render, 64, v0, 96, threads)
    out["cornell"] = {"gpu_paths_per_s": gpu0, "gpu_ms": min(ms), "cpu_paths_per_s": pc / sc, "cpu_cores": threads,
                      "cpu_sample": "96x96 centre crop x 64 spp", "gpu_over_cpu": gpu0 / (pc / sc)}
    # PSSMLT
    c3 = Bundle.generate("pssmlt", 1)
    ctx.upload(c3)
    r3 = c3.render
    r3.frame_id = 0
    ctx.render(r3, c3.views, to_host=False)
    flush.zero_()
    torch.cuda.synchronize()
    ctx.reset_stats()
    r3.frame_id = 1
    ctx.render(r3, c3.views, to_host=False)
    st = ctx.stats()
    out["pssmlt"] = {"ms": st.last_kernel_ms, "chain_ms": st.last_dominant_ms,
                     "proposals_per_s": st.proposed / (st.last_dominant_ms / 1000.0),
                     "paths_per_s": st.paths / (st.last_kernel_ms / 1000.0),
                     "acceptance": st.accepted / max(1, st.proposed), "b": st.bootstrap_b}
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
    return out


def run_reference(args, world, rank, dist):
    """--impl reference: the CPU restatement on all host threads, bounded samples per step."""
    if rank != 0:
        return
    from barnacle_gb300 import Bundle

    b = Bundle.generate(args.workload, 1)
    views = b.views
    threads = os.cpu_count() or 1
    r = b.render
    # the same sample as the GPU arm's cpu_baseline (centre crops of the first views), at the
    # step's samples per pixel
    nv, crop, _ = WORKLOADS[args.workload][2]
    sample_views = views[:nv]
    for _ in range(args.warmup):
        cpu_sample_render(b, b.render, args.spp_per_step, sample_views[:1], 16, threads)
    paths, secs = 0, 0.0
    for _ in range(args.steps):
        p, s = cpu_sample_render(b, b.render, args.spp_per_step, sample_views, crop, threads)
        paths += p
        secs += s
    value = paths / secs
    line = {"metric": METRIC, "value": value, "unit": "paths/s", "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": 1000 * secs / args.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded procedural scene)",
            "impl": "reference",
            "config": {"workload": WORKLOADS[args.workload][0], "spp_per_step": args.spp_per_step,
                       "l2": "n/a (CPU)"},
            "cpu_baseline": {"value": value, "unit": "paths/s", "cores": threads, "kind": "port",
                             "sample": f"{crop}x{crop} centre crops of the first {len(sample_views)} view(s) x "
                                       f"{args.spp_per_step} spp per step (the F# reference cannot be built: no "
                                       f".NET SDK)"},
            "e2e": {"value": value, "unit": "paths/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def profile_figures(mode, workload, spp_per_step):
    """The ncu figures committed under profiles/ for this form and workload: the DRAM bytes of one
    render ("bytes_per_launch: N", measured at 4 spp per step; other step sizes report none) and
    the L2 side of the roofline of the dominant kernel ("l2: kernel=… hit_rate=… throughput_frac=…")."""
    traffic = None
    prof = ROOT / "profiles" / f"traffic_{mode}_{workload}.md"
    if prof.exists():
        for line in prof.read_text().splitlines():
            if line.startswith("bytes_per_launch:") and spp_per_step == 4:
                traffic = int(line.split(":")[1])
    l2 = None
    prof = ROOT / "profiles" / ("k_pt_mega_instances.md" if mode == "megakernel" else "k_wf_extend_instances.md")
    if workload == "instances" and prof.exists():
        for line in prof.read_text().splitlines():
            if line.startswith("l2:"):
                kv = dict(f.split("=") for f in line[3:].split())
                l2 = {"kernel": kv["kernel"], "hit_rate": float(kv["hit_rate"]),
                      "throughput_frac": float(kv["throughput_frac"]), "source": f"profiles/{prof.name} (ncu)"}
    return traffic, l2


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=4)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--mode", default="wavefront", choices=["megakernel", "wavefront"])
    ap.add_argument("--no-compare", action="store_true", help="skip timing the other render form")
    ap.add_argument("--workload", default="instances", choices=sorted(WORKLOADS))
    ap.add_argument("--spp-per-step", type=int, default=0, help="0 = the workload's default (instances 4, cornell 64)")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-extras", action="store_true",
                    help="skip the Cornell-box CPU ratio, PSSMLT and adjoint/forward measurements")
    ap.add_argument("--pool", type=int, default=0, help="wavefront path slots (0 = autotuned)")
    ap.add_argument("--cap", type=int, default=0, help="wavefront blocks per SM cap (0 = autotuned)")
    ap.add_argument("--bvh-width", type=int, default=0, choices=[0, 2, 4],
                    help="BVH walk: 0 = auto (wide records for BVHs of 64+ nodes), 2 = binary, 4 = wide")
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
    b = Bundle.generate(args.workload, 1)
    b.scene.contents.bvh_width = args.bvh_width
    ctx.upload(b)
    views = b.views
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
    rc = capi.bn_render_desc()
    C_copy = bytes(r)
    C.memmove(C.addressof(rc), C_copy, len(C_copy))
    rc.flags |= capi.BN_RENDER_COUNT
    rc.mode = primary
    rc.frame_id = 100
    ctx.reset_stats()
    ctx.render(rc, views, to_host=False)
    st = ctx.stats()
    bpu = bytes_per_unit()
    alg_bytes = bpu["node"] * st.nodes_visited + bpu["triangle"] * st.tris_tested + bpu["instance"] * st.instances_visited
    rays_per_step = st.rays

    def timed(mode, frame_base):
        r.mode = mode
        for w in range(args.warmup):
            r.frame_id = frame_base + w
            ctx.render(r, views, to_host=False)
        barrier(dist)
        torch.cuda.synchronize()
        dev_ms, dom_ms, launches = 0.0, 0.0, 0
        t0 = time.perf_counter()
        for k in range(args.steps):
            flush.zero_()
            torch.cuda.synchronize()
            r.frame_id = frame_base + 100 + k
            ctx.render(r, views, to_host=False)
            s = ctx.stats()
            dev_ms += s.last_kernel_ms
            dom_ms += s.last_dominant_ms
            launches += s.last_launches
        torch.cuda.synchronize()
        wall = time.perf_counter() - t0
        barrier(dist)
        return max_over_ranks(dist, dev_ms / 1000.0), dom_ms, launches, wall

    other = capi.BN_MODE_MEGAKERNEL if primary == capi.BN_MODE_WAVEFRONT else capi.BN_MODE_WAVEFRONT
    with ClockSampler(dev) as clk:
        dev_s, dom_ms, launches, wall = timed(primary, 0)
    other_s = None
    if not args.no_compare:
        other_s, _, _, _ = timed(other, 1000)

    # end to end through the C-ABI with a host film (pinned)
    r.mode = primary
    film = torch.empty(pixels * 3, dtype=torch.float32).pin_memory().numpy()
    view_arr = (capi.bn_view * len(views))(*views)
    barrier(dist)
    t0 = time.perf_counter()
    for k in range(args.steps):
        r.frame_id = 200 + k
        rcode = ctx.lib.bn_render(ctx._h, C.byref(r), view_arr, len(views), capi.ptr(film))
        if rcode:
            raise RuntimeError(ctx.error())
        float(film[0])  # the step's result is on the host
    e2e_s = max_over_ranks(dist, time.perf_counter() - t0)

    peak, peak_kind = measured_peak_gbs()
    dom_launch_s = dom_ms / 1000.0 / args.steps
    achieved = alg_bytes / dom_launch_s / 1e9
    traffic, l2 = profile_figures(args.mode, args.workload, args.spp_per_step)

    cpu = None
    if rank == 0 and not args.no_cpu_baseline:
        threads = os.cpu_count() or 1
        nv, crop, spp = WORKLOADS[args.workload][2]
        p, s = cpu_sample_render(b, b.render, spp, views[:nv], crop, threads)
        cpu = {"value": p / s, "unit": "paths/s", "cores": threads, "kind": "port",
               "sample": f"{crop}x{crop} centre crops of the first {nv} view(s) x {spp} spp "
                         "(oracle: CPU restatement of the F# path; the F# renderer cannot be built here)"}

    extras = None
    if rank == 0 and not args.no_extras:
        extras = run_extras(ctx, args, torch, flush)

    if rank == 0:
        value = world * paths_per_step * args.steps / dev_s
        line = {
            "metric": METRIC, "value": value, "unit": "paths/s", "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": 1000 * dev_s / args.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded procedural scene)",
            "config": {"workload": WORKLOADS[args.workload][0],
                       "mode": args.mode, "bvh_width": {0: "auto", 2: "binary", 4: "wide"}[args.bvh_width], "spp_per_step": r.spp, "pixels_per_step": pixels,
                       "rays_per_step": int(rays_per_step),
                       "per_ray": {"nodes": st.nodes_visited / max(1, st.rays), "triangles": st.tris_tested / max(1, st.rays),
                                   "instances": st.instances_visited / max(1, st.rays)},
                       "parallelism": "replicas" if world > 1 else "single",
                       "l2": "flushed before every timed step (512 MiB write)"},
            "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                         "frac": achieved / peak, "traffic": traffic, "peak_kind": peak_kind,
                         "kernel": "k_pt_mega" if args.mode == "megakernel" else
                                   "wavefront bounce loop (regen+extend+shade+shadow, one graph)",
                         "alg_bytes_per_launch": int(alg_bytes), "l2": l2},
            "cpu_baseline": cpu,
            "e2e": {"value": world * paths_per_step * args.steps / e2e_s, "unit": "paths/s",
                    "h2d_bytes_per_step": C.sizeof(capi.bn_view) * len(views),
                    "d2h_bytes_per_step": pixels * 3 * 4},
            "gpu_launches": launches,
            "clocks": clk.summary(),
            "mrays_per_s": world * rays_per_step * args.steps / dev_s / 1e6,
            "compare": None if other_s is None else {
                "other_mode": "megakernel" if primary == capi.BN_MODE_WAVEFRONT else "wavefront",
                "other_paths_per_s": world * paths_per_step * args.steps / other_s,
                "ratio_this_over_other": other_s / dev_s,
                "equal_rmse": "same per-path estimator and random streams in both forms (images equal to "
                              "float summation order, tests/test_gpu_wavefront.py)"},
            "wall_s": wall,
            "extras": extras,
        }
        print(json.dumps(line), flush=True)
    ctx.close()
    if dist is not None:
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
