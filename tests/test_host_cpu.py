"""CPU tests: the oracle against the golden vectors, the library's host preparation against the
oracle (bit-exact BVH builds), the scene generators and loaders, and the C-ABI symbol table."""
import json
import re
from pathlib import Path

import numpy as np
import pytest

from barnacle_gb300 import Bundle, BarnacleError, bvh_build, capi, mat4_invert
from oracle import pyoracle

GOLDEN = Path(__file__).resolve().parent / "golden"
ROOT = Path(__file__).resolve().parent.parent


def load(name):
    return json.loads((GOLDEN / f"{name}.json").read_text())


# ------------------------------------------------------------------ sampler (Util/Hash.fs)
def test_oracle_hash_and_lcg_match_golden():
    g = load("sampler")
    L = pyoracle.lib()
    for case in g["three"]:
        assert L.or_xxhash32_three(*case["seed"]) == case["hash"]
    for case in g["two"]:
        assert L.or_xxhash32_two(*case["xy"]) == case["hash"]
    seeds = np.array([c["seed"] for c in g["three"]], np.uint32)
    draws = pyoracle.sampler_stream(seeds, 16)
    want = np.array([c["draws"] for c in g["three"]], np.float32)
    assert draws.tobytes() == want.tobytes()


# ------------------------------------------------------------------ BVH builder (Util/BVH.fs)
def nodes_tuple(nodes):
    return [(list(map(float, n["bounds_min"])), list(map(float, n["bounds_max"])), int(n["right_or_offset"]),
             int(n["is_leaf"]), int(n["split_axis"]) if not n["is_leaf"] else 0,
             int(n["count"]) if n["is_leaf"] else 0) for n in nodes]


@pytest.mark.parametrize("case_index", range(9))
def test_bvh_oracle_and_library_match_golden(case_index):
    case = load("bvh")[case_index]
    boxes = np.array(case["boxes"], np.float32)
    want = [(n[0], n[1], n[2], n[3], n[4], n[5]) for n in case["nodes"]]
    on, op = pyoracle.bvh_build(boxes)
    ln, lp = bvh_build(boxes)
    assert nodes_tuple(on) == want, f"oracle differs from golden ({case['kind']})"
    assert list(op) == case["perm"]
    assert nodes_tuple(ln) == want, f"library differs from golden ({case['kind']})"
    assert list(lp) == case["perm"]


def test_bvh_empty_and_single():
    n, p = bvh_build(np.zeros((0, 6), np.float32))
    assert len(n) == 1 and n[0]["is_leaf"] == 1 and n[0]["count"] == 0
    n, p = bvh_build(np.array([[0, 0, 0, 1, 1, 1]], np.float32))
    assert len(n) == 1 and n[0]["count"] == 1 and list(p) == [0]


@pytest.mark.parametrize("seed", [1, 2, 3])
def test_bvh_library_matches_oracle_random_large(seed):
    rng = np.random.default_rng(seed)
    n = 5000
    c = rng.uniform(-100, 100, size=(n, 3))
    # clusters and duplicates exercise the zero-extent median split
    c[: n // 10] = c[0]
    e = rng.exponential(1.0, size=(n, 3))
    boxes = np.concatenate([c - e, c + e], 1).astype(np.float32)
    on, op = pyoracle.bvh_build(boxes)
    ln, lp = bvh_build(boxes)
    assert on.tobytes() == ln.tobytes()
    assert np.array_equal(op, lp)


@pytest.mark.parametrize("name", ["cornell", "cornell-objects", "instances"])
def test_scene_blas_and_tlas_library_match_oracle(name):
    b = Bundle.generate(name, 1)
    s = b.scene.contents
    osc = pyoracle.Scene(b.scene)
    for mi in range(s.n_meshes):
        m = s.meshes[mi]
        nt = m.n_triangles
        V = np.ctypeslib.as_array(m.vertices, shape=(m.n_vertices * 3,)).reshape(-1, 3)
        I = np.ctypeslib.as_array(m.indices, shape=(nt * 3,)).reshape(-1, 3)
        P = V[I]
        # Triangle.Bounds = MinNative/MaxNative of the vertices (no NaNs here, so min/max agree)
        boxes = np.concatenate([P.min(1), P.max(1)], 1).astype(np.float32)
        ln, lp = bvh_build(boxes)
        on, op = osc.blas(mi, nt)
        assert ln.tobytes() == on.tobytes(), f"{name}: BLAS of mesh {mi} differs"
        assert np.array_equal(lp, op)


# ------------------------------------------------------------------ triangle test (Mesh.fs)
def one_triangle_desc(tri, keep):
    import ctypes as C
    v = np.ascontiguousarray(np.array(tri, np.float32).reshape(-1))
    idx = np.array([0, 1, 2], np.int32)
    mesh = capi.bn_mesh_desc(v.ctypes.data_as(C.POINTER(C.c_float)), idx.ctypes.data_as(C.POINTER(C.c_int32)), None, 3, 1)
    prims = (capi.bn_primitive_desc * 1)(capi.bn_primitive_desc(0, 0, 0.0))
    meshes = (capi.bn_mesh_desc * 1)(mesh)
    eye = (C.c_float * 16)(*np.eye(4, dtype=np.float32).reshape(-1))
    inst = capi.bn_instance_desc(0, 0, 0, 0, eye, eye)
    insts = (capi.bn_instance_desc * 1)(inst)
    mats = (capi.bn_material_desc * 1)(capi.bn_material_desc(0, (C.c_float * 3)(1, 1, 1), 1.5, 1.0, 0.0, 0.0))
    lights = (capi.bn_light_desc * 1)(capi.bn_light_desc((C.c_float * 3)(1, 1, 1), 1))
    d = capi.bn_scene_desc(prims, 1, meshes, 1, insts, 1, mats, 1, lights, 1, 0)
    keep += [v, idx, mesh, prims, meshes, insts, mats, lights, d]
    return C.pointer(d)


def test_oracle_triangle_intersection_matches_golden():
    g = load("triangle")
    keep = []
    desc = one_triangle_desc(g["triangle"], keep)
    osc = pyoracle.Scene(desc)
    rays = np.zeros(len(g["rays"]), capi.RAY_DTYPE)
    for i, r in enumerate(g["rays"]):
        rays[i]["origin"] = r["o"]
        rays[i]["direction"] = r["d"]
        rays[i]["t_max"] = np.inf
    hits, _ = osc.trace(rays)
    n_hit = 0
    for i, r in enumerate(g["rays"]):
        if r["hit"] is None:
            assert hits[i]["instance"] == -1, f"ray {i}: oracle hit, golden missed"
        else:
            n_hit += 1
            assert hits[i]["instance"] == 0, f"ray {i}: oracle missed, golden hit"
            t, u, v = r["hit"]
            assert np.float32(hits[i]["t"]) == np.float32(t)
            assert np.float32(hits[i]["u"]) == np.float32(u)
            assert np.float32(hits[i]["v"]) == np.float32(v)
    assert n_hit > 10


# ------------------------------------------------------------------ BSDFs in FP64
def bsdf_queries(g):
    q = np.zeros(len(g["cases"]), capi.BSDF_QUERY_DTYPE)
    for i, c in enumerate(g["cases"]):
        q[i]["material"] = c["material"]
        q[i]["wo"] = c["wo"]
        q[i]["wi"] = c["wi"]
    return q


def golden_materials(g):
    import ctypes as C
    return [capi.bn_material_desc(m["type"], (C.c_float * 3)(*m["base"]), m["ior"], m["roughness"], m["metallic"], 0)
            for m in g["materials"]]


def test_oracle_bsdf_eval_fp64_and_fp32_match_golden():
    g = load("bsdf")
    q = bsdf_queries(g)
    mats = golden_materials(g)
    o64 = pyoracle.bsdf(mats, q, sample=False, use_double=True)
    o32 = pyoracle.bsdf(mats, q, sample=False, use_double=False)
    want = np.array([c["bsdf"] + [c["pdf"]] for c in g["cases"]])
    np.testing.assert_allclose(o64[:, :4], want, rtol=1e-6, atol=1e-12)
    # the FP32 restatement keeps the reference's GGX D = a^2 / (pi (1 + (a^2 - 1) c^2)^2), whose
    # cancellation costs ~eps/a^2 relative for sharp lobes (a = 0.04 here): 1e-4, not 1e-5
    np.testing.assert_allclose(o32[:, :4], want, rtol=1e-4, atol=1e-7)


# ------------------------------------------------------------------ scenes and loaders
def test_generated_workloads_have_the_stated_sizes():
    c0 = Bundle.generate("cornell")
    assert c0.n_triangles_instanced == 36
    v = c0.views[0]
    assert (v.width, v.height) == (256, 256) and c0.render.spp == 64 and c0.render.max_depth == 8
    c1 = Bundle.generate("cornell-objects")
    assert c1.n_triangles_instanced == 36 + 81920 + 20480 + 2
    assert c1.render.spp == 256 and c1.render.max_depth == 16
    c2 = Bundle.generate("instances")
    assert c2.scene.contents.n_instances == 1 + 1024 + 64
    assert len(c2.views) == 16
    assert 140_000_000 < c2.n_triangles_instanced < 180_000_000
    pix = [(v.width, v.height) for v in c2.views]
    assert min(w * h for w, h in pix) >= 256 * 240 and max(w * h for w, h in pix) <= 1920 * 1080
    c3 = Bundle.generate("pssmlt")
    r = c3.render
    assert r.integrator == capi.BN_INTEGRATOR_PSSMLT and r.n_chains == 65536 and r.n_bootstrap == 1 << 20
    assert abs(r.large_step_prob - 0.3) < 1e-7 and r.mutation == capi.BN_MUTATION_KELEMEN
    assert abs(r.eps_max - 1 / 64) < 1e-9 and c3.views[0].width == 1024
    c4 = Bundle.generate("materials")
    assert c4.n_slots == 32 and c4.emissive_slot_base == 28 and len(c4.slot_params()) == 32 * 6


def test_generation_is_deterministic():
    a = Bundle.generate("instances", 3)
    b = Bundle.generate("instances", 3)
    sa, sb = a.scene.contents, b.scene.contents
    for i in range(sa.n_instances):
        assert bytes(sa.instances[i]) == bytes(sb.instances[i])
    m = sa.meshes[3]
    va = np.ctypeslib.as_array(m.vertices, shape=(m.n_vertices * 3,))
    vb = np.ctypeslib.as_array(sb.meshes[3].vertices, shape=(m.n_vertices * 3,))
    assert va.tobytes() == vb.tobytes()


def test_geodesic_meshes_are_closed():
    c2 = Bundle.generate("instances")
    s = c2.scene.contents
    for mi in range(4):
        m = s.meshes[mi]
        I = np.ctypeslib.as_array(m.indices, shape=(m.n_triangles * 3,)).reshape(-1, 3)
        e = np.sort(np.concatenate([I[:, [0, 1]], I[:, [1, 2]], I[:, [2, 0]]]), axis=1)
        _, counts = np.unique(e, axis=0, return_counts=True)
        assert np.all(counts == 2), "every edge of a closed mesh is shared by exactly two triangles"
        assert m.n_vertices == m.n_triangles // 2 + 2  # Euler characteristic 2


def test_json_loader_reference_schema(tmp_path):
    scene = GOLDEN / "scenes" / "spheres_thinlens.json"
    b = Bundle.load_json(str(scene))
    s = b.scene.contents
    assert s.n_primitives == 5 and s.n_instances == 7
    r = b.render
    assert r.integrator == capi.BN_INTEGRATOR_PSSMLT and r.spp == 4 and r.max_depth == 6
    assert r.mutation == capi.BN_MUTATION_KELEMEN and abs(r.eps_max - 1 / 16) < 1e-9
    v = b.views[0]
    assert v.camera.type == capi.BN_CAM_THIN_LENS and v.width == 96 and v.height == 72
    assert abs(v.camera.aperture - 0.5) < 1e-7 and abs(v.camera.push_forward - 10) < 1e-6
    # camera node translation (50, 40.8, 295.6); rotations are radians
    assert np.allclose(list(v.camera.camera_to_world)[12:15], [50, 40.8, 295.6], atol=1e-4)
    # the instance under two nodes is listed twice with the last traversal's transform
    prims = [s.instances[i].primitive for i in range(s.n_instances)]
    assert prims.count(4) == 2
    twice = [i for i in range(s.n_instances) if s.instances[i].primitive == 4]
    assert list(s.instances[twice[0]].object_to_world) == list(s.instances[twice[1]].object_to_world)
    # defaults: albedo 1, roughness 1, metallic 0, ior 1.5; two-sided default true
    m = s.materials[3]
    assert list(m.base_color) == [1, 1, 1] and m.roughness == 1 and m.metallic == 0 and abs(m.ior - 1.5) < 1e-7
    assert s.lights[0].two_sided == 1


def test_json_loader_errors(tmp_path):
    p = tmp_path / "bad.json"
    p.write_text('{"nodes": [{}], "integrator": {"type": "nope"}, "camera": {"type": "pinhole"}, '
                 '"film": {"width": 4, "height": 4, "tone-mapping": "aces"}}')
    with pytest.raises(BarnacleError, match="Unknown integrator type"):
        Bundle.load_json(str(p))
    p.write_text("{ not json")
    with pytest.raises(BarnacleError):
        Bundle.load_json(str(p))
    with pytest.raises(BarnacleError):
        Bundle.load_json(str(tmp_path / "missing.json"))
    with pytest.raises(BarnacleError, match="unknown workload"):
        Bundle.generate("no-such-workload")


def test_json_loader_reads_reference_cbox():
    """The reference's scene file, loaded unchanged (UTF-8 BOM, radians, thin lens, PSSMLT)."""
    from cbox_common import CBOX
    b = Bundle.load_json(str(CBOX))
    s = b.scene.contents
    assert s.n_instances == 9 and s.n_primitives == 9
    assert b.render.integrator == capi.BN_INTEGRATOR_PSSMLT and b.render.spp == 16 and b.render.max_depth == 8
    assert b.render.n_chains == 1024 and b.render.n_bootstrap == 4 * 1024 * 1024
    v = b.views[0]
    assert v.width == 1024 and v.height == 768 and v.camera.type == capi.BN_CAM_THIN_LENS
    assert v.camera.aperture == 4.0 and v.camera.focus_distance == 210.0
    assert b.tone_mapping == capi.BN_TONE_ACES


def test_oracle_render_of_cbox_matches_the_reference_sample_image():
    """Pins the oracle to the reference's own output, coarsely: the oracle's path tracer renders
    cbox.json (16 spp, ACES, 8-bit as Film.Save) and the 16x16 block means of the image must be
    within the PSNR bound of the reference's "Sample - Path Tracing.png" (render settings not
    recorded; see cbox_common.PSNR_MIN for what the bound separates)."""
    from cbox_common import CBOX, PSNR_MIN, block_means, psnr, samples
    b = Bundle.load_json(str(CBOX))
    r = b.render
    r.integrator = capi.BN_INTEGRATOR_PATH
    r.spp = 16
    v = b.views[0]
    img, _ = pyoracle.Scene(b.scene).render_pt(r, v)
    got = block_means(pyoracle.tonemap(img, capi.BN_TONE_ACES))
    ref = samples()
    assert psnr(got, ref["pt"]) > PSNR_MIN, psnr(got, ref["pt"])
    assert psnr(got, ref["pssmlt"]) > PSNR_MIN, psnr(got, ref["pssmlt"])


def test_obj_loader_fan_triangulation_and_negative_indices(tmp_path):
    obj = tmp_path / "m.obj"
    obj.write_text("v 0 0 0\nv 1 0 0\nv 1 1 0\nv 0 1 0\nf 1 2 3 4\nf -4/1 -2/2 -1/3\n")
    scene = tmp_path / "s.json"
    scene.write_text(json.dumps({
        "nodes": [{"instances": [0], "children": [1]}, {"has-camera": True}],
        "instances": [{"primitive": 0, "light": 0}],
        "primitives": [{"type": "mesh", "uri": str(obj)}],
        "lights": [{"type": "diffuse", "emission": [1, 1, 1]}],
        "integrator": {"type": "path-tracing"}, "camera": {"type": "pinhole"},
        "film": {"width": 8, "height": 8, "tone-mapping": "identity"}}))
    b = Bundle.load_json(str(scene))
    m = b.scene.contents.meshes[0]
    idx = np.ctypeslib.as_array(m.indices, shape=(m.n_triangles * 3,)).tolist()
    assert idx == [0, 1, 2, 0, 2, 3, 0, 2, 3]


def test_mat4_invert():
    rng = np.random.default_rng(0)
    for _ in range(20):
        m = rng.normal(size=(4, 4)).astype(np.float32)
        m[:, 3] = [0, 0, 0, 1]
        inv = mat4_invert(m).reshape(4, 4)
        np.testing.assert_allclose(m.astype(np.float64) @ inv, np.eye(4), atol=1e-4)


# ------------------------------------------------------------------ the C-ABI surface
def test_library_exports_every_declared_symbol():
    header = (ROOT / "include" / "barnacle_gpu.h").read_text()
    declared = set(re.findall(r"^(?:int|const char\*|void)\s+(bn_[a-z0-9_]+)\s*\(", header, flags=re.M))
    assert len(declared) >= 20
    lib = capi.load_library()
    missing = [s for s in sorted(declared) if not hasattr(lib, s)]
    assert not missing, f"declared but not exported: {missing}"
    assert declared <= set(capi.SIGNATURES), "every declared entry point has a ctypes signature"
    assert lib.bn_version().decode().startswith("barnacle-gb300")


# ------------------------------------------------------------------ film output and integrators
def test_json_loader_integrators_and_tone_mapping(tmp_path):
    base = {"nodes": [{"instances": [0], "children": [1]}, {"has-camera": True}],
            "instances": [{"primitive": 0, "light": 0}],
            "primitives": [{"type": "sphere", "radius": 1.0}],
            "lights": [{"type": "diffuse", "emission": [1, 1, 1]}],
            "camera": {"type": "pinhole"}}
    want = {"normal": capi.BN_INTEGRATOR_NORMAL, "direct": capi.BN_INTEGRATOR_DIRECT,
            "path-tracing": capi.BN_INTEGRATOR_PATH}
    tones = {"aces": capi.BN_TONE_ACES, "gamma": capi.BN_TONE_GAMMA, "identity": capi.BN_TONE_IDENTITY}
    for (itype, ival), (tname, tval) in zip(want.items(), tones.items()):
        p = tmp_path / f"{itype}.json"
        p.write_text(json.dumps({**base, "integrator": {"type": itype, "spp": 3},
                                 "film": {"width": 4, "height": 2, "tone-mapping": tname}}))
        b = Bundle.load_json(str(p))
        assert b.render.integrator == ival and b.render.spp == 3 and b.tone_mapping == tval
    p = tmp_path / "bad.json"
    p.write_text(json.dumps({**base, "integrator": {"type": "normal"},
                             "film": {"width": 4, "height": 2, "tone-mapping": "filmic"}}))
    with pytest.raises(BarnacleError, match="Unknown tone mapping type"):
        Bundle.load_json(str(p))
    assert Bundle.generate("cornell").tone_mapping == capi.BN_TONE_ACES


def test_oracle_tonemap_against_float32_formulas():
    """Film.PostProcess restated independently in numpy float32 (ACES fit, clamp) and the Rgba32
    packing floor(255 v + 0.5)."""
    from oracle import pyoracle
    rng = np.random.default_rng(3)
    x = np.concatenate([rng.uniform(0, 4, (4000, 3)), [[0, 0.5, 1], [2, 1e-8, 100]]]).astype(np.float32)
    f = np.float32
    aces = (x * (f(2.51) * x + f(0.03))) / (x * (f(2.43) * x + f(0.59)) + f(0.14))
    for tm, y in ((capi.BN_TONE_IDENTITY, x), (capi.BN_TONE_ACES, aces)):
        y = np.clip(y, f(0), f(1))
        want = np.floor(y * f(255) + f(0.5)).astype(np.uint8)
        got = pyoracle.tonemap(x, tm)
        assert np.array_equal(got[:, :3], want) and (got[:, 3] == 255).all()
    g = pyoracle.tonemap(x, capi.BN_TONE_GAMMA)[:, :3].astype(int)
    ref = np.floor(np.clip(x.astype(np.float64) ** (1 / 2.2), 0, 1) * 255 + 0.5)
    assert np.abs(g - ref).max() <= 1
    # NaN packs to 0; the ACES fit maps -1 to 2.48 / 1.98 > 1 and 7 near 1
    nan = pyoracle.tonemap(np.array([[np.nan, -1, 7]], np.float32), capi.BN_TONE_ACES)
    assert nan[0].tolist() == [0, 255, 255, 255]
    assert pyoracle.tonemap(np.array([[np.nan, -1, 0.25]], np.float32), capi.BN_TONE_IDENTITY)[0].tolist() == \
        [0, 0, 64, 255]


def test_png_writer_round_trip(tmp_path):
    import struct
    import zlib
    from barnacle_gb300 import write_png
    rng = np.random.default_rng(0)
    for h, w in ((1, 1), (7, 13), (300, 200)):  # 300 x 801 bytes: several stored blocks
        img = rng.integers(0, 256, (h, w, 4), dtype=np.uint8)
        p = tmp_path / f"i{h}.png"
        write_png(p, img)
        data = p.read_bytes()
        assert data[:8] == b"\x89PNG\r\n\x1a\n"
        pos, chunks = 8, {}
        while pos < len(data):
            n = struct.unpack(">I", data[pos:pos + 4])[0]
            typ = data[pos + 4:pos + 8]
            body = data[pos + 8:pos + 8 + n]
            assert struct.unpack(">I", data[pos + 8 + n:pos + 12 + n])[0] == zlib.crc32(typ + body)
            chunks[typ] = chunks.get(typ, b"") + body
            pos += 12 + n
        assert struct.unpack(">IIBBBBB", chunks[b"IHDR"]) == (w, h, 8, 6, 0, 0, 0)
        raw = np.frombuffer(zlib.decompress(chunks[b"IDAT"]), np.uint8).reshape(h, 1 + 4 * w)
        assert (raw[:, 0] == 0).all() and np.array_equal(raw[:, 1:].reshape(h, w, 4), img)


def test_json_loader_interpolates_keyframes_around_time_zero(tmp_path):
    """Scene.Render renders t = 0 (Program.fs:27); a transform with keyframes at t = -1 and t = 1
    is interpolated (Scene.fs:13-20): scales and translations lerp to their midpoints, and
    Transform.Compose (Util/Transform.fs:6-9) then builds CreateTranslation(scale) *
    CreateFromQuaternion(rotation) * CreateScale(translation) — scale and translation swapped, as
    in the reference."""
    def scene(keys):
        return {"transforms": [{"keyframes": keys}],
                "nodes": [{"instances": [0], "transform": 0, "children": [1]}, {"has-camera": True}],
                "instances": [{"primitive": 0, "light": 0}],
                "primitives": [{"type": "sphere", "radius": 1.0}],
                "lights": [{"type": "diffuse", "emission": [1, 1, 1]}],
                "integrator": {"type": "path-tracing"}, "camera": {"type": "pinhole"},
                "film": {"width": 4, "height": 4, "tone-mapping": "aces"}}
    p = tmp_path / "kf.json"
    p.write_text(json.dumps(scene([
        {"time": -1, "scale": [1, 1, 1], "translation": [0, 0, 0]},
        {"time": 1, "scale": [3, 3, 3], "translation": [2, 4, 6]}])))
    m = np.array(Bundle.load_json(str(p)).scene.contents.instances[0].object_to_world, np.float32).reshape(4, 4)
    want = np.diag([1, 2, 3, 1]).astype(np.float32)   # CreateScale(translation (1, 2, 3))
    want[3, :3] = [2 * 1, 2 * 2, 2 * 3]                 # CreateTranslation(scale (2, 2, 2)) * that
    np.testing.assert_allclose(m, want, atol=1e-6)
    # a rotation interpolated by Slerp: 0 and pi/2 about y give pi/4
    p.write_text(json.dumps(scene([
        {"time": -1, "rotation": [0, 0, 0], "translation": [1, 1, 1]},
        {"time": 1, "rotation": [0, np.pi / 2, 0], "translation": [1, 1, 1]}])))
    m = np.array(Bundle.load_json(str(p)).scene.contents.instances[0].object_to_world, np.float32).reshape(4, 4)
    c = np.cos(np.pi / 4)
    rot = np.array([[c, 0, -c], [0, 1, 0], [c, 0, c]], np.float32)  # CreateRotationY(pi/4), row vectors
    np.testing.assert_allclose(m[:3, :3], rot, atol=1e-5)  # CreateScale(translation (1, 1, 1)) = I
    np.testing.assert_allclose(m[3, :3], rot.sum(0), atol=1e-5)  # translation row (1, 1, 1) * R
    # at or after the last keyframe, and before the first, no interpolation
    p.write_text(json.dumps(scene([{"time": 0, "translation": [5, 0, 0]}, {"time": 2, "translation": [9, 0, 0]}])))
    m = np.array(Bundle.load_json(str(p)).scene.contents.instances[0].object_to_world, np.float32).reshape(4, 4)
    assert list(m[3, :3]) == [5, 0, 0]


def test_bench_reads_the_committed_profile_figures():
    """bench.py reports the DRAM traffic per ray and the L2 side of the roofline from the
    machine-readable ncu figures under profiles/; each must parse, carry its source and hold
    plausible values."""
    sys_path = str(ROOT)
    import sys
    if sys_path not in sys.path:
        sys.path.insert(0, sys_path)
    import bench

    prof = bench.profile_figures("instances")
    tr = prof["traffic"]["wavefront"]
    assert 10 < tr["dram_bytes_per_ray"] < 10 ** 5 and "ncu" in tr["source"]
    for mode, kernel in (("wavefront", "k_wf_extend"), ("megakernel", "k_pt_mega")):
        l2 = prof["l2"][mode]
        assert l2["kernel"] == kernel and 0 < l2["hit_rate"] < 1 and 0 < l2["throughput_frac"] < 1
        assert l2["source"].startswith("profiles/")
    assert bench.profile_figures("cornell") is None


def test_bench_reference_arm_prints_the_contract_line():
    """`bench.py --impl reference` (the CPU restatement, no GPU library loaded) prints one JSON line
    with the GPU arm's metric, unit and workload config, `impl: reference`, a `cpu_baseline`
    describing the run and an `e2e` object without host-device copies."""
    import subprocess
    import sys
    out = subprocess.run([sys.executable, str(ROOT / "bench.py"), "--impl", "reference", "--steps", "1",
                          "--warmup", "0", "--views", "2"], capture_output=True, text=True, timeout=600,
                         cwd=str(ROOT))
    assert out.returncode == 0, out.stderr[-2000:]
    lines = [l for l in out.stdout.splitlines() if l.startswith("{")]
    assert len(lines) == 1
    d = json.loads(lines[0])
    assert d["impl"] == "reference" and d["unit"] == "paths/s" and d["higher_is_better"] is True
    assert d["value"] > 0 and d["steps"] == 1 and d["n_gpus"] == 1
    assert d["config"]["workload"].startswith("instances") and d["config"]["views"] == 2
    cb = d["cpu_baseline"]
    assert cb["kind"] == "port" and cb["cores"] >= 1 and cb["value"] == d["value"] and "tiles" in cb["sample"]
    e = d["e2e"]
    assert e["value"] == d["value"] and e["h2d_bytes_per_step"] == 0 and e["d2h_bytes_per_step"] == 0


def test_bench_cpu_tiles_cover_every_view():
    """The CPU arms sample 16x16 tiles of every view, a different cell of a 4x4 grid per step;
    16 steps visit every cell of every view once."""
    import sys
    if str(ROOT) not in sys.path:
        sys.path.insert(0, str(ROOT))
    import bench
    from barnacle_gb300 import Bundle

    b = Bundle.generate("instances", 1)  # the views live in the bundle's memory: keep it alive
    views = b.views
    seen = set()
    for step in range(16):
        tiles = bench.cpu_tiles(views, step, 1)
        assert sorted(vi for vi, _ in tiles) == list(range(len(views)))
        for vi, (x0, y0, x1, y1) in tiles:
            v = views[vi]
            assert x1 - x0 == 16 and y1 - y0 == 16 and 0 <= x0 and x1 <= v.width and 0 <= y0 and y1 <= v.height
            seen.add((vi, x0, y0))
    assert len(seen) == 16 * len(views)


def _bundle_digest(b):
    import hashlib
    s = b.scene.contents
    h = hashlib.sha256()
    for i in range(s.n_meshes):
        m = s.meshes[i]
        h.update(np.ctypeslib.as_array(m.vertices, shape=(m.n_vertices * 3,)).tobytes())
        h.update(np.ctypeslib.as_array(m.indices, shape=(m.n_triangles * 3,)).tobytes())
    for arr, n in ((s.instances, s.n_instances), (s.materials, s.n_materials), (s.lights, s.n_lights)):
        for i in range(n):
            h.update(bytes(arr[i]))
    for v in b.views:
        h.update(bytes(v))
    return h.hexdigest()[:16]


# the generated workloads' bits (meshes, instances, materials, lights, views), the same on every
# host: the converged images under tests/golden/ were rendered from exactly these scenes
WORKLOAD_DIGESTS = {"cornell": "7117cb82e4469383", "cornell-objects": "fe156941062dffd7",
                    "instances": "6dc4b549805dc09b", "pssmlt": "4524a4473e1f2b88", "materials": "9d3871172b53493e"}


@pytest.mark.parametrize("name", sorted(WORKLOAD_DIGESTS))
def test_generated_workloads_have_the_same_bits_on_every_host(name):
    b = Bundle.generate(name, 1)  # b owns the views' memory while they are hashed
    assert _bundle_digest(b) == WORKLOAD_DIGESTS[name]


def test_scene_library_without_cuda_builds_the_same_scenes():
    """The CPU arms build their scenes with the host code alone (oracle/_build/libbarnacle_scenes.so,
    the same sources without the CUDA parts): the same bits as the GPU library's host code."""
    b = Bundle.generate("instances", 1, lib=pyoracle.scenes_library())
    assert _bundle_digest(b) == WORKLOAD_DIGESTS["instances"]
