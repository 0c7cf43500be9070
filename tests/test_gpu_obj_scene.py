"""A mesh read from an OBJ file through the JSON loader's "uri" (MeshPrimitive.Load,
Extensions/Primitive/Mesh.fs:246-279), on the device: the file is written by the test (a displaced
geodesic sphere of 20,480 triangles taken from the procedural workload, with some faces as
quads and some indices negative), the scene references it by a path relative to the scene file,
and the device's closest hits and renders are checked against the oracle on the same scene."""
import json

import numpy as np
import pytest

from barnacle_gb300 import Bundle, capi
from oracle import pyoracle

pytestmark = pytest.mark.gpu


def write_obj(path, vertices, tris):
    lines = ["# geodesic sphere"] + [f"v {x:.9g} {y:.9g} {z:.9g}" for x, y, z in vertices]
    nv = len(vertices)
    k = 0
    while k < len(tris):
        a, b, c = tris[k] + 1
        if k % 7 == 0 and k + 1 < len(tris) and tris[k + 1][0] == tris[k][0] and tris[k + 1][1] == tris[k][2]:
            d = tris[k + 1][2] + 1  # a fan of two triangles (a b c), (a c d) as one quad
            lines.append(f"f {a} {b} {c} {d}")
            k += 2
            continue
        if k % 5 == 0:  # negative (relative) indices
            lines.append(f"f {a - nv - 1} {b - nv - 1} {c - nv - 1}")
        else:
            lines.append(f"f {a}/{a} {b}//{b} {c}")
        k += 1
    path.write_text("\n".join(lines) + "\n")


@pytest.fixture(scope="module")
def obj_scene(tmp_path_factory):
    d = tmp_path_factory.mktemp("obj")
    src = Bundle.generate("cornell-objects", 1)
    s = src.scene.contents
    # the level-5 dielectric icosphere of the workload (20,480 triangles)
    m = max((s.meshes[i] for i in range(s.n_meshes)), key=lambda m: (m.n_triangles == 20480, m.n_triangles))
    v = np.ctypeslib.as_array(m.vertices, shape=(m.n_vertices, 3)).astype(np.float64)
    t = np.ctypeslib.as_array(m.indices, shape=(m.n_triangles, 3)).copy()
    write_obj(d / "sphere.obj", v, t)
    scene = {
        "nodes": [{"instances": [0, 1, 2], "children": [1]}, {"transform": 0, "has-camera": True}],
        "instances": [{"primitive": 0, "material": 0}, {"primitive": 1, "material": 1}, {"primitive": 2, "light": 0}],
        "primitives": [{"type": "mesh", "vertices": [-4, -1, -4, 4, -1, -4, 4, -1, 4, -4, -1, 4],
                        "indices": [0, 2, 1, 0, 3, 2]},
                       {"type": "mesh", "uri": "sphere.obj"},
                       {"type": "mesh", "vertices": [-1, 3, -1, 1, 3, -1, 1, 3, 1, -1, 3, 1], "indices": [0, 1, 2, 0, 2, 3]}],
        "materials": [{"type": "lambertian", "albedo": [0.7, 0.7, 0.7]},
                      {"type": "pbr", "albedo": [0.8, 0.5, 0.3], "roughness": 0.4, "metallic": 0.5}],
        "lights": [{"type": "diffuse", "emission": [10, 10, 10]}],
        "transforms": [{"keyframes": [{"time": 0.0, "translation": [0, 0.5, 4.0]}]}],
        "integrator": {"type": "path-tracing", "spp": 8, "max-depth": 6, "rr-depth": 3},
        "camera": {"type": "pinhole", "fov": 45.0, "aspect-ratio": 1.0},
        "film": {"width": 64, "height": 64, "tone-mapping": "aces"}}
    (d / "scene.json").write_text(json.dumps(scene))
    b = Bundle.load_json(str(d / "scene.json"))
    assert b.scene.contents.meshes[1].n_triangles == 20480
    return b


def test_obj_mesh_traces_like_the_oracle(ctx, obj_scene):
    b = obj_scene
    ctx.upload(b)
    o = pyoracle.Scene(b.scene)
    rng = np.random.default_rng(5)
    n = 20000
    rays = np.zeros(n, capi.RAY_DTYPE)
    rays["origin"] = rng.uniform(-2.5, 2.5, (n, 3)).astype(np.float32)
    dd = rng.normal(size=(n, 3)).astype(np.float32)
    rays["direction"] = dd / np.sqrt((dd ** 2).sum(1, dtype=np.float32))[:, None]
    rays["t_max"] = np.inf
    g = ctx.trace(rays)
    h, _ = o.trace(rays)
    assert (g["instance"] >= 0).mean() > 0.2
    assert np.array_equal(g["instance"], h["instance"]) and np.array_equal(g["primitive"], h["primitive"])
    assert np.array_equal(g["t"].view(np.uint32), h["t"].view(np.uint32))


@pytest.mark.parametrize("mode", [capi.BN_MODE_MEGAKERNEL, capi.BN_MODE_WAVEFRONT], ids=["megakernel", "wavefront"])
def test_obj_scene_renders_like_the_oracle(ctx, obj_scene, mode):
    b = obj_scene
    ctx.upload(b)
    o = pyoracle.Scene(b.scene)
    v = b.views[0]
    r = b.render
    r.mode = mode
    r.spp = 16
    gpu, cpu = [], []
    for f in range(16):
        r.frame_id = f
        gpu.append(ctx.render(r, v)[0])
        r.frame_id = 1000 + f
        cpu.append(o.render_pt(r, v)[0])
    g, c = np.stack(gpu).astype(np.float64), np.stack(cpu).astype(np.float64)
    ok = np.isfinite(g).all(0) & np.isfinite(c).all(0)
    se = np.sqrt(g.var(0, ddof=1) / len(g) + c.var(0, ddof=1) / len(c))
    z = np.abs(g.mean(0) - c.mean(0)) / np.maximum(se, 1e-12)
    valid = ok & (se > 0)
    assert g.mean() > 0.01
    assert (z[valid] > 3).mean() < 0.02, f"{(z[valid] > 3).mean():.3%} of pixel means beyond 3 standard errors"
