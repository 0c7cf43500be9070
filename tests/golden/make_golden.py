"""Generates the golden fixtures in tests/golden/ from pure-Python restatements of the reference
formulas (numpy float32 scalars, one IEEE operation at a time, no fused multiply-add except where
the reference calls FusedMultiplyAdd).  These restatements are independent of the C++ oracle and
of the library; the CPU tests check both against the fixtures.

  sampler.json  Util/Hash.fs:6-32 (XXHash32Two/Three, LCG) and Base/Sampler.fs:7-16
  bvh.json      Util/BVH.fs:99-247 (binned SAH build, flatten, permutation) on seeded box sets
  triangle.json Extensions/Primitive/Mesh.fs:24-82 + Base/Ray.fs:29-39 (triangle AABB pre-test and
                Moller-Trumbore) on seeded rays against one triangle
  bsdf.json     Extensions/Material/{Lambertian,Mirror,Dielectric,PBR}.fs in float64

Run: python tests/golden/make_golden.py   (rewrites the four files)
"""
from __future__ import annotations

import json
import math
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
f32 = np.float32
M32 = 0xFFFFFFFF


# --------------------------------------------------------------------------- hash / sampler
def xxhash32_two(x: int, y: int) -> int:
    p2, p3, p4, p5 = 2246822519, 3266489917, 668265263, 374761393
    h = (y + p5 + x * p3) & M32
    h = (p4 * (((h << 17) | (h >> 15)) & M32)) & M32
    h = (p2 * (h ^ (h >> 15))) & M32
    h = (p3 * (h ^ (h >> 13))) & M32
    return h ^ (h >> 16)


def xxhash32_three(x: int, y: int, z: int) -> int:
    p2, p3, p4, p5 = 2246822519, 3266489917, 668265263, 374761393
    h = (z + p5 + x * p3) & M32
    h = (p4 * (((h << 17) | (h >> 15)) & M32)) & M32
    h = (h + y * p3) & M32
    h = (p4 * (((h << 17) | (h >> 15)) & M32)) & M32
    h = (p2 * (h ^ (h >> 15))) & M32
    h = (p3 * (h ^ (h >> 13))) & M32
    return h ^ (h >> 16)


def lcg_stream(seed: int, n: int) -> list[float]:
    out = []
    for _ in range(n):
        seed = (0x00269EC3 + seed * 0x000343FD) & M32
        bits = (seed >> 9) | 0x3F800000
        out.append(float(np.array([bits], np.uint32).view(np.float32)[0] - f32(1)))
    return out


def make_sampler():
    rng = np.random.default_rng(20260101)
    seeds = [[0, 0, 0], [1, 2, 3], [255, 255, 63], [0xFFFFFFFF, 0, 7]]
    seeds += rng.integers(0, 2**32, size=(12, 3), dtype=np.uint64).tolist()
    streams = []
    for x, y, z in seeds:
        s = xxhash32_three(int(x), int(y), int(z))
        streams.append({"seed": [int(x), int(y), int(z)], "hash": s, "draws": lcg_stream(s, 16)})
    twos = []
    for x, y in [[0, 0xDEADBEEF], [1, 2], [12345, 67890]] + rng.integers(0, 2**32, size=(5, 2), dtype=np.uint64).tolist():
        twos.append({"xy": [int(x), int(y)], "hash": xxhash32_two(int(x), int(y))})
    return {"three": streams, "two": twos}


# --------------------------------------------------------------------------- BVH (Util/BVH.fs)
INF = f32(np.inf)


def v_min(a, b):  # MinNative: a < b ? a : b
    return [a[i] if a[i] < b[i] else b[i] for i in range(3)]


def v_max(a, b):
    return [a[i] if a[i] > b[i] else b[i] for i in range(3)]


def box_union(a, b):
    return (v_min(a[0], b[0]), v_max(a[1], b[1]))


def centroid(b):
    return [f32(0.5) * (b[0][i] + b[1][i]) for i in range(3)]


def surface_area(b):
    d = [b[1][i] - b[0][i] for i in range(3)]
    return f32(2) * ((d[0] * d[1] + d[1] * d[2]) + d[2] * d[0])


def split_axis(b):
    d = [b[1][i] - b[0][i] for i in range(3)]
    if d[0] >= d[1] and d[0] >= d[2]:
        return 0
    return 1 if d[1] >= d[2] else 2


def box_default():
    return ([INF, INF, INF], [-INF, -INF, -INF])


def tree_build(items, first, last, depth):
    n = last - first
    sub = items[first:last]
    bounds = box_default()
    for b, _ in sub:
        bounds = box_union(bounds, b)
    if n <= 4 or depth >= 64:
        return ("leaf", bounds, first, n)
    cb = box_default()
    for b, _ in sub:
        c = centroid(b)
        cb = (v_min(cb[0], c), v_max(cb[1], c))
    axis = split_axis(cb)
    extent = cb[1][axis] - cb[0][axis]
    if extent == f32(0):
        mid = first + n // 2
        return ("node", bounds, axis, tree_build(items, first, mid, depth + 1), tree_build(items, mid, last, depth + 1))

    def find_bin(b):
        return min(11, int((f32(12) * (centroid(b)[axis] - cb[0][axis])) / extent))

    bins = [[box_default(), 0] for _ in range(12)]
    for b, _ in sub:
        k = find_bin(b)
        bins[k][0] = box_union(bins[k][0], b)
        bins[k][1] += 1
    costs = [f32(0)] * 11
    lb, rb, lc, rc = box_default(), box_default(), 0, 0
    with np.errstate(invalid="ignore", over="ignore"):
        for i in range(11):
            lb = box_union(lb, bins[i][0])
            lc += bins[i][1]
            costs[i] = costs[i] + f32(lc) * surface_area(lb)
            rb = box_union(rb, bins[11 - i][0])
            rc += bins[11 - i][1]
            costs[10 - i] = costs[10 - i] + f32(rc) * surface_area(rb)
        best, min_cost = 0, INF
        for i in range(11):
            cost = costs[i] + f32(n) * surface_area(cb)
            if cost < min_cost:
                min_cost, best = cost, i
    left, right = first, last - 1
    for it in sub:
        if find_bin(it[0]) > best:
            items[right] = it
            right -= 1
        else:
            items[left] = it
            left += 1
    return ("node", bounds, axis, tree_build(items, first, left, depth + 1), tree_build(items, right + 1, last, depth + 1))


def flatten(tree, out):
    idx = len(out)
    if tree[0] == "leaf":
        _, b, off, cnt = tree
        out.append([[float(x) for x in b[0]], [float(x) for x in b[1]], off, 1, 0, cnt])
    else:
        _, b, axis, l, r = tree
        out.append(None)
        flatten(l, out)
        ri = flatten(r, out)
        out[idx] = [[float(x) for x in b[0]], [float(x) for x in b[1]], ri, 0, axis, 0]
    return idx


def bvh_build(boxes):
    items = [(([f32(x) for x in b[:3]], [f32(x) for x in b[3:]]), i) for i, b in enumerate(boxes)]
    with np.errstate(invalid="ignore", over="ignore"):
        tree = tree_build(items, 0, len(items), 0)
    nodes = []
    flatten(tree, nodes)
    return nodes, [i for _, i in items]


def make_bvh():
    rng = np.random.default_rng(7)
    cases = []
    for n, kind in [(1, "random"), (4, "random"), (5, "random"), (13, "random"), (64, "random"), (200, "random"),
                    (9, "same-centroid"), (40, "grid"), (30, "flat")]:
        if kind == "random":
            c = rng.uniform(-10, 10, size=(n, 3))
            e = rng.uniform(0.01, 2, size=(n, 3))
        elif kind == "same-centroid":
            c = np.zeros((n, 3))
            e = rng.uniform(0.1, 1, size=(n, 3))
        elif kind == "grid":
            g = np.arange(n)
            c = np.stack([g % 4, (g // 4) % 5, g // 20], 1).astype(float)
            e = np.full((n, 3), 0.25)
        else:  # flat boxes in a plane, zero thickness in y
            c = rng.uniform(-5, 5, size=(n, 3))
            c[:, 1] = 1.0
            e = rng.uniform(0.1, 1, size=(n, 3))
            e[:, 1] = 0.0
        boxes = np.concatenate([c - e, c + e], 1).astype(np.float32)
        nodes, perm = bvh_build(boxes.tolist())
        cases.append({"kind": kind, "boxes": boxes.tolist(), "nodes": nodes, "perm": perm})
    return cases


# --------------------------------------------------------------------------- triangle test
def dot(a, b):
    return (a[0] * b[0] + a[1] * b[1]) + a[2] * b[2]


def cross(a, b):
    return [a[1] * b[2] - a[2] * b[1], a[2] * b[0] - a[0] * b[2], a[0] * b[1] - a[1] * b[0]]


def sub3(a, b):
    return [a[i] - b[i] for i in range(3)]


def math_max(a, b):
    return f32(np.nan) if (a != a or b != b) else (a if a > b else b)


def math_min(a, b):
    return f32(np.nan) if (a != a or b != b) else (a if a < b else b)


def box_hit(lo, hi, o, d, t):
    with np.errstate(divide="ignore", invalid="ignore"):
        inv = [f32(1) / d[i] for i in range(3)]
        t0 = [(lo[i] - o[i]) * inv[i] for i in range(3)]
        t1 = [(hi[i] - o[i]) * inv[i] for i in range(3)]
    a, c = v_min(t0, t1), v_max(t0, t1)
    tmin = math_max(f32(1e-3), math_max(a[0], math_max(a[1], a[2])))
    tmax = math_min(t, math_min(c[0], math_min(c[1], c[2])))
    return bool(tmin <= tmax)


def mt(p0, p1, p2, o, d, t):
    eps = f32(np.finfo(np.float32).smallest_subnormal)
    e0, e1 = sub3(p1, p0), sub3(p2, p0)
    rce1 = cross(d, e1)
    det = dot(e0, rce1)
    if abs(det) < eps:
        return None
    inv = f32(1) / det
    s = sub3(o, p0)
    u = inv * dot(s, rce1)
    if u < 0 or u > 1:
        return None
    sce0 = cross(s, e0)
    v = inv * dot(d, sce0)
    if v < 0 or u + v > 1:
        return None
    tt = inv * dot(e1, sce0)
    if not (tt > eps and tt < t):
        return None
    return tt, u, v


def make_triangle():
    rng = np.random.default_rng(11)
    p = [[f32(-1), f32(0), f32(-1)], [f32(1), f32(0.25), f32(-1)], [f32(0.2), f32(0.5), f32(1.5)]]
    lo, hi = v_min(v_min(p[0], p[1]), p[2]), v_max(v_max(p[0], p[1]), p[2])
    rays = []
    for k in range(64):
        o = [f32(x) for x in rng.uniform(-2, 2, 3)]
        o[1] = f32(rng.uniform(2, 4))
        target = [f32(x) for x in rng.uniform(-1.2, 1.2, 3)]
        target[1] = f32(0.25)
        d = sub3(target, o)
        ln = np.sqrt(np.float32(dot(d, d)), dtype=np.float32)
        d = [d[i] / ln for i in range(3)]
        if k % 16 == 0:  # an axis-aligned ray (zero direction components: inf reciprocals)
            d = [f32(0), f32(-1), f32(0)]
        t = f32(np.inf)
        hit = None
        if box_hit(lo, hi, o, d, t):
            hit = mt(p[0], p[1], p[2], o, d, t)
        rays.append({"o": [float(x) for x in o], "d": [float(x) for x in d],
                     "hit": None if hit is None else [float(x) for x in hit]})
    return {"triangle": [[float(x) for x in q] for q in p], "rays": rays}


# --------------------------------------------------------------------------- BSDFs in float64
PI = float(np.float32(3.14159265))


def normalize(v):
    n = math.sqrt(v[0] * v[0] + v[1] * v[1] + v[2] * v[2])
    return [x / n for x in v]


def pbr_eval(base, rough, metal, wo, wi):
    a = max(float(f32(rough) * f32(rough)), 1e-3)
    a = float(f32(a))
    m = min(max(metal, 0.0), 1.0)

    def lam(w):
        s2 = w[0] * w[0] + w[1] * w[1]
        if s2 == 0:
            return 0.0
        return (-1 + math.sqrt(1 + a * a * s2 / (w[2] * w[2]))) / 2

    wh = normalize([wo[i] + wi[i] for i in range(3)])
    c = abs(wh[2])
    k = 1 + (a * a - 1) * c * c
    D = a * a / (PI * k * k)
    G = 1 / (1 + lam(wo) + lam(wi))
    spec = D * G / (4 * abs(wo[2]))
    coh = sum(wo[i] * wh[i] for i in range(3))
    cc = 1 - coh
    c5 = cc ** 5
    fc = [base[i] + (1 - base[i]) * c5 for i in range(3)]
    fd = 0.04 + 0.96 * c5
    diffuse = [base[i] * abs(wi[2]) / PI for i in range(3)]
    inner = [diffuse[i] * (1 - fd) + spec * fd for i in range(3)]
    f = [inner[i] * (1 - m) + spec * fc[i] * m for i in range(3)]
    t = 0.5 * (1 - m)
    pdf = (D * abs(wh[2]) / (4 * coh)) * (1 - t) + abs(wi[2]) / PI * t
    return f, pdf


def make_bsdf():
    rng = np.random.default_rng(5)
    mats = [
        {"type": 0, "base": [0.73, 0.5, 0.2], "ior": 1.5, "roughness": 1.0, "metallic": 0.0},
        {"type": 1, "base": [0.9, 0.8, 0.7], "ior": 1.5, "roughness": 1.0, "metallic": 0.0},
        {"type": 2, "base": [1.0, 1.0, 1.0], "ior": 1.5, "roughness": 1.0, "metallic": 0.0},
        {"type": 3, "base": [0.8, 0.3, 0.1], "ior": 1.5, "roughness": 0.4, "metallic": 0.0},
        {"type": 3, "base": [0.9, 0.7, 0.3], "ior": 1.5, "roughness": 0.7, "metallic": 1.0},
        {"type": 3, "base": [0.5, 0.5, 0.5], "ior": 1.5, "roughness": 0.2, "metallic": 0.35},
    ]
    cases = []
    for mi, m in enumerate(mats):
        for _ in range(12):
            # directions above the surface, away from grazing (|z| >= 0.2)
            def hemi():
                while True:
                    v = rng.normal(size=3)
                    v /= np.linalg.norm(v)
                    v[2] = abs(v[2])
                    if v[2] >= 0.2:
                        return [float(f32(x)) for x in v]

            wo, wi = hemi(), hemi()
            if m["type"] == 0:
                pdf = abs(wi[2]) / PI
                f = [b * pdf for b in m["base"]]
            elif m["type"] == 3:
                f, pdf = pbr_eval([float(f32(b)) for b in m["base"]], m["roughness"], m["metallic"], wo, wi)
            else:
                f, pdf = [0.0, 0.0, 0.0], 0.0
            cases.append({"material": mi, "wo": wo, "wi": wi, "bsdf": f, "pdf": pdf})
    return {"materials": mats, "cases": cases}


if __name__ == "__main__":
    for name, fn in [("sampler", make_sampler), ("bvh", make_bvh), ("triangle", make_triangle), ("bsdf", make_bsdf)]:
        (HERE / f"{name}.json").write_text(json.dumps(fn(), separators=(",", ":")))
        print("wrote", HERE / f"{name}.json")
