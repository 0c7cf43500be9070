"""The GPU BVH builder (bn_bvh_build_device) against the host builder, node array and permutation
compared byte for byte; the host builder itself is pinned to the golden vectors and the oracle by
the CPU tests.  The cases aim at the places where an order-free device reduction could differ from
the reference's sequential fold: zero coordinates of both signs on box planes, duplicate boxes
(zero centroid extent, median split), large ranges split level by level and the depth cap."""
import json
from pathlib import Path

import numpy as np
import pytest

from barnacle_gb300 import Bundle, bvh_build, capi

pytestmark = pytest.mark.gpu

GOLDEN = Path(__file__).resolve().parent / "golden"


def same(ctx, boxes):
    hn, hp = bvh_build(boxes)
    dn, dp = ctx.bvh_build(boxes)
    assert len(hn) == len(dn), f"{len(dn)} nodes on the device, {len(hn)} on the host"
    diff = np.nonzero(hn.view(np.uint8).reshape(len(hn), 32) != dn.view(np.uint8).reshape(len(dn), 32))[0]
    assert diff.size == 0, f"{np.unique(diff).size} nodes differ, first {diff[0]}"
    assert np.array_equal(hp, dp)
    return hn


@pytest.mark.parametrize("case_index", range(9))
def test_device_builder_matches_golden_cases(ctx, case_index):
    case = json.loads((GOLDEN / "bvh.json").read_text())[case_index]
    same(ctx, np.array(case["boxes"], np.float32))


def random_boxes(rng, n, spread=100.0):
    c = rng.uniform(-spread, spread, size=(n, 3))
    e = rng.exponential(1.0, size=(n, 3))
    return np.concatenate([c - e, c + e], 1).astype(np.float32)


@pytest.mark.parametrize("n", [0, 1, 4, 5, 257, 3000, 70000, 400000])
def test_device_builder_random_sizes(ctx, n):
    same(ctx, random_boxes(np.random.default_rng(n), n))


def test_device_builder_signed_zeros_on_box_planes(ctx):
    """Coordinates drawn from {-0, +0, 1, 2} and integer grids: bounds that are zero come out of
    the fold with the sign of the last zero item, which the device must reproduce."""
    rng = np.random.default_rng(5)
    vals = np.array([-0.0, 0.0, 1.0, 2.0], np.float32)
    lo = vals[rng.integers(0, 2, size=(60000, 3))]
    hi = vals[rng.integers(0, 4, size=(60000, 3))]
    boxes = np.concatenate([np.minimum(lo, hi), np.maximum(lo, hi)], 1).astype(np.float32)
    boxes[:, 3:][hi == 0] = vals[rng.integers(0, 2, size=int((hi == 0).sum()))]
    same(ctx, boxes)
    g = rng.integers(-20, 20, size=(80000, 3)).astype(np.float32)
    g[g == 0] = np.where(rng.random(int((g == 0).sum())) < 0.5, -0.0, 0.0)
    same(ctx, np.concatenate([g, g + rng.integers(0, 2, size=(80000, 3))], 1).astype(np.float32))


def test_device_builder_duplicates_and_clusters(ctx):
    rng = np.random.default_rng(7)
    b = random_boxes(rng, 50000)
    b[:20000] = b[0]          # one cluster of identical boxes: zero extent, median splits
    b[20000:20600] = b[20000]
    same(ctx, b)
    # every box identical: median splits down to the depth cap
    same(ctx, np.tile(np.array([[0, 0, 0, 1, 1, 1]], np.float32), (4096, 1)))


def test_device_builder_depth_cap_and_overflow(ctx):
    """An infinite box makes every bin cost NaN, so each split keeps the whole range on the left
    and the recursion runs to the depth cap of 64: both builders make the same chain and capped
    leaf, and both refuse a capped leaf over 127 items (in the per-thread and the level-by-level
    part of the device build)."""
    from barnacle_gb300 import BarnacleError
    rng = np.random.default_rng(11)
    b = random_boxes(rng, 100)
    b[7, 3] = np.inf
    nodes = same(ctx, b)
    assert len(nodes) == 129 and nodes["count"].max() == 100
    for n in (150, 5000):
        b = random_boxes(rng, n)
        b[3, 4] = np.inf
        with pytest.raises(BarnacleError):
            bvh_build(b)
        with pytest.raises(BarnacleError):
            ctx.bvh_build(b)


@pytest.mark.parametrize("name", ["cornell-objects", "instances"])
def test_device_builder_on_workload_meshes(ctx, name):
    b = Bundle.generate(name, 1)
    s = b.scene.contents
    for mi in range(s.n_meshes):
        m = s.meshes[mi]
        if m.n_triangles < 10000:
            continue
        v = np.ctypeslib.as_array(m.vertices, shape=(m.n_vertices * 3,)).reshape(-1, 3)
        idx = np.ctypeslib.as_array(m.indices, shape=(m.n_triangles * 3,)).reshape(-1, 3)
        p = v[idx]
        boxes = np.concatenate([p.min(1), p.max(1)], 1).astype(np.float32)
        same(ctx, boxes)


def test_scene_upload_with_either_builder_traces_the_same(ctx):
    b = Bundle.generate("instances", 1)
    rng = np.random.default_rng(9)
    n = 20000
    rays = np.zeros(n, capi.RAY_DTYPE)
    rays["origin"] = rng.uniform([-60, 0, -60], [60, 25, 60], size=(n, 3)).astype(np.float32)
    d = rng.normal(size=(n, 3)).astype(np.float32)
    rays["direction"] = d / np.linalg.norm(d, axis=1, keepdims=True).astype(np.float32)
    rays["t_max"] = np.inf
    out = []
    for builder in (capi.BN_BUILDER_HOST, capi.BN_BUILDER_DEVICE):
        b.scene.contents.bvh_builder = builder
        ctx.upload(b)
        out.append((ctx.instance_order(b.scene.contents.n_instances), ctx.trace(rays, capi.BN_TRACE_COUNT), ctx.stats()))
    b.scene.contents.bvh_builder = capi.BN_BUILDER_AUTO
    (o1, h1, _), (o2, h2, _) = out
    assert np.array_equal(o1, o2)
    assert h1.tobytes() == h2.tobytes()
