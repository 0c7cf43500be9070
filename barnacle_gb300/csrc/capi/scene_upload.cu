// bn_scene_upload: the host preparation of the render call, then one upload.
//
//  1. BLAS per mesh over the triangle AABBs (MeshPrimitive.BVHNodes, Mesh.fs:159-169), which
//     permutes the mesh's triangles in place; triangles are stored in that order.  Built on the
//     GPU (bvh_gpu.cu) or the host (bvh_build.cpp), which give the same trees.
//  2. the reference AliasTable of each mesh over triangle areas in permuted order
//     (Mesh.fs:181-186, Util/AliasTable.fs:14-27): entry pdf = area / (sequential float sum).
//  3. instance world bounds = AxisAlignedBoundingBox.Transform(BLAS root bounds, ObjectToWorld)
//     over the 8 corners (Util/BVH.fs:29-40, Primitive.fs:131-138).
//  4. TLAS over the instance bounds (BVHAggregate, Aggregate/BVH.fs:9), which permutes instances.
//  5. light tables: uniform = emissive instances in TLAS order (LightSampler.fs:7); alias =
//     Vose table over emissive triangles weighted by world area x Rec.709 luminance.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <limits>
#include <string>
#include <vector>

#include "../host/bvh_build.hpp"
#include "../host/host_math.hpp"
#include "context.hpp"

using bnh::M4;
using bnh::V3;

namespace {

V3 vtx(const bn_mesh_desc& m, int i) {
  return {m.vertices[3 * i], m.vertices[3 * i + 1], m.vertices[3 * i + 2]};
}

void put_node(float4* dst, const bn_bvh_node& n) {
  dst[0] = make_float4(n.bounds_min[0], n.bounds_min[1], n.bounds_min[2], n.bounds_max[0]);
  int packed = static_cast<int>(n.is_leaf) | (static_cast<int>(static_cast<uint8_t>(n.split_axis)) << 8) |
               (static_cast<int>(static_cast<uint8_t>(n.count)) << 16) |
               (static_cast<int>(n.visibility_mask) << 24);
  float link, pk;
  std::memcpy(&link, &n.right_or_offset, 4);
  std::memcpy(&pk, &packed, 4);
  dst[1] = make_float4(n.bounds_max[1], n.bounds_max[2], link, pk);
}

void columns(const float* m, float4 out[3]) {
  // (M1r, M2r, M3r, M4r) for r = 1..3
  for (int r = 0; r < 3; ++r) out[r] = make_float4(m[r], m[4 + r], m[8 + r], m[12 + r]);
}

struct MeshPrep {
  std::vector<bn_bvh_node> nodes;
  std::vector<int32_t> perm;
  int node_base = 0, tri_base = 0, node4_root = -1;
};

// The wide records of one binary BVH (layout in dev_types.cuh).  A record stands for an
// interior node g and holds the boxes the reference tests in the two steps below g: g's
// children's children, or a child itself when it is a leaf.  The walk over records makes the
// binary walk's decisions because a box nested in another is never entered when the outer one
// is not: slab distances are monotone in the box planes under round-to-nearest (and a zero
// direction component admits exactly the boxes whose open slab holds the origin), so testing a
// grandchild alone gives the answer of testing it after its parent with the same t.  That
// needs every child box to contain its children's boxes, which the builder's unions guarantee
// for finite bounds; the check below rejects the rest (NaN coordinates).
struct Collapse {
  const std::vector<bn_bvh_node>& b;
  std::vector<float4>& out;
  bool nested = true;

  static bool inside(const bn_bvh_node& in, const bn_bvh_node& outer) {
    for (int a = 0; a < 3; ++a)
      if (!(outer.bounds_min[a] <= in.bounds_min[a] && in.bounds_max[a] <= outer.bounds_max[a])) return false;
    return true;
  }

  int emit(int g) {
    const int idx = static_cast<int>(out.size() / 8);
    out.resize(out.size() + 8);
    const int kids[2] = {g + 1, b[g].right_or_offset};
    int slot[4] = {-1, -1, -1, -1};
    int axis[3] = {b[g].split_axis, 0, 0};
    for (int c = 0; c < 2; ++c) {
      const bn_bvh_node& k = b[kids[c]];
      if (k.is_leaf) {
        slot[2 * c] = kids[c];
      } else {
        slot[2 * c] = kids[c] + 1;
        slot[2 * c + 1] = k.right_or_offset;
        axis[1 + c] = k.split_axis;
        nested = nested && inside(b[kids[c] + 1], k) && inside(b[k.right_or_offset], k);
      }
    }
    const float nan = std::numeric_limits<float>::quiet_NaN();
    float box[6][4];
    int ref[4] = {0, 0, 0, 0};
    unsigned counts = 0, leaf_mask = 0;
    for (int s = 0; s < 4; ++s) {
      if (slot[s] < 0) {
        for (int r = 0; r < 6; ++r) box[r][s] = nan;
        continue;
      }
      const bn_bvh_node& n = b[slot[s]];
      for (int a = 0; a < 3; ++a) {
        box[a][s] = n.bounds_min[a];
        box[3 + a][s] = n.bounds_max[a];
      }
      if (n.is_leaf) {
        ref[s] = n.right_or_offset;
        counts |= static_cast<unsigned>(static_cast<uint8_t>(n.count)) << (8 * s);
        leaf_mask |= 1u << s;
      } else {
        ref[s] = emit(slot[s]);  // grows out: the record is written by index below
      }
    }
    float4* r = &out[8 * static_cast<size_t>(idx)];
    for (int k = 0; k < 6; ++k) r[k] = make_float4(box[k][0], box[k][1], box[k][2], box[k][3]);
    float4 rf, mt;
    std::memcpy(&rf, ref, 16);
    // slot order per ray octant (bit a of the octant: d[a] > 0): the near child's pair first (left
    // when d[axis of g] > 0), each pair ordered by its child's split axis; 2 bits per slot
    unsigned orders[2] = {0u, 0u};
    for (int oct = 0; oct < 8; ++oct) {
      const bool lf = (oct >> (axis[0] & 3)) & 1;
      const bool fa = (oct >> (axis[lf ? 1 : 2] & 3)) & 1;
      const bool fb = (oct >> (axis[lf ? 2 : 1] & 3)) & 1;
      const int pa = lf ? 0 : 2, pb = 2 - pa;
      const unsigned v0 = pa + (fa ? 0 : 1), v1 = pa + (fa ? 1 : 0), v2 = pb + (fb ? 0 : 1), v3 = pb + (fb ? 1 : 0);
      orders[oct >> 2] |= (v0 | (v1 << 2) | (v2 << 4) | (v3 << 6)) << (8 * (oct & 3));
    }
    const int meta[4] = {static_cast<int>(counts),
                         static_cast<int>(leaf_mask | (static_cast<unsigned>(axis[0] & 3) << 4) |
                                          (static_cast<unsigned>(axis[1] & 3) << 6) |
                                          (static_cast<unsigned>(axis[2] & 3) << 8)),
                         static_cast<int>(orders[0]), static_cast<int>(orders[1])};
    std::memcpy(&mt, meta, 16);
    r[6] = rf;
    r[7] = mt;
    return idx;
  }
};

// Vose's alias method over non-negative weights (double precision build)
void build_vose(const std::vector<double>& w, std::vector<float>* prob, std::vector<int>* alias, std::vector<float>* pmf) {
  const size_t n = w.size();
  double sum = 0.0;
  for (double x : w) sum += x;
  prob->assign(n, 1.f);
  alias->resize(n);
  pmf->resize(n);
  std::vector<double> scaled(n);
  std::vector<size_t> small, large;
  for (size_t i = 0; i < n; ++i) {
    (*alias)[i] = static_cast<int>(i);
    (*pmf)[i] = static_cast<float>(sum > 0 ? w[i] / sum : 1.0 / n);
    scaled[i] = sum > 0 ? w[i] * n / sum : 1.0;
    (scaled[i] < 1.0 ? small : large).push_back(i);
  }
  while (!small.empty() && !large.empty()) {
    const size_t s = small.back(), l = large.back();
    small.pop_back();
    (*prob)[s] = static_cast<float>(scaled[s]);
    (*alias)[s] = static_cast<int>(l);
    scaled[l] = (scaled[l] + scaled[s]) - 1.0;
    if (scaled[l] < 1.0) {
      large.pop_back();
      small.push_back(l);
    }
  }
  for (size_t i : large) (*prob)[i] = 1.f;
  for (size_t i : small) (*prob)[i] = 1.f;
}

template <class T>
cudaError_t upload(DevBuf& b, const std::vector<T>& v, cudaStream_t st) {
  const size_t bytes = std::max<size_t>(v.size() * sizeof(T), 16);
  cudaError_t e = b.reserve(bytes);
  if (e != cudaSuccess) return e;
  if (!v.empty()) e = cudaMemcpyAsync(b.ptr, v.data(), v.size() * sizeof(T), cudaMemcpyHostToDevice, st);
  return e;
}

}  // namespace

extern "C" int bn_scene_upload(bn_context* ctx, const bn_scene_desc* d) {
  if (!ctx) return BN_ERR_INVALID_ARG;
  if (!d) return ctx->fail(BN_ERR_INVALID_ARG, "bn_scene_upload: null scene");
  cudaSetDevice(ctx->device);
  ctx->has_scene = false;
  // ---- validation
  if (d->n_instances <= 0 || !d->instances) return ctx->fail(BN_ERR_INVALID_ARG, "scene has no instances");
  if (d->n_primitives < 0 || (d->n_primitives > 0 && !d->primitives)) return ctx->fail(BN_ERR_INVALID_ARG, "bad primitives");
  if (d->n_meshes < 0 || (d->n_meshes > 0 && !d->meshes)) return ctx->fail(BN_ERR_INVALID_ARG, "bad meshes");
  if (d->n_materials < 0 || (d->n_materials > 0 && !d->materials)) return ctx->fail(BN_ERR_INVALID_ARG, "bad materials");
  if (d->n_lights < 0 || (d->n_lights > 0 && !d->lights)) return ctx->fail(BN_ERR_INVALID_ARG, "bad lights");
  for (int i = 0; i < d->n_meshes; ++i) {
    const bn_mesh_desc& m = d->meshes[i];
    if (m.n_triangles < 0 || m.n_vertices < 0 || (m.n_triangles > 0 && (!m.indices || !m.vertices)))
      return ctx->fail(BN_ERR_INVALID_ARG, "mesh " + std::to_string(i) + ": bad arrays");
    for (long long k = 0; k < 3LL * m.n_triangles; ++k)
      if (m.indices[k] < 0 || m.indices[k] >= m.n_vertices)
        return ctx->fail(BN_ERR_INVALID_ARG, "mesh " + std::to_string(i) + ": vertex index out of range");
    if (m.tri_material)
      for (int k = 0; k < m.n_triangles; ++k)
        if (m.tri_material[k] < -1 || m.tri_material[k] >= d->n_materials)
          return ctx->fail(BN_ERR_INVALID_ARG, "mesh " + std::to_string(i) + ": triangle material out of range");
  }
  for (int i = 0; i < d->n_primitives; ++i) {
    const bn_primitive_desc& p = d->primitives[i];
    if (p.type == BN_PRIM_MESH && (p.mesh < 0 || p.mesh >= d->n_meshes))
      return ctx->fail(BN_ERR_INVALID_ARG, "primitive " + std::to_string(i) + ": mesh out of range");
    if (p.type != BN_PRIM_MESH && p.type != BN_PRIM_SPHERE)
      return ctx->fail(BN_ERR_INVALID_ARG, "primitive " + std::to_string(i) + ": unknown type");
  }
  for (int i = 0; i < d->n_instances; ++i) {
    const bn_instance_desc& in = d->instances[i];
    if (in.primitive < 0 || in.primitive >= d->n_primitives)
      return ctx->fail(BN_ERR_INVALID_ARG, "instance " + std::to_string(i) + ": primitive out of range");
    if (in.material < -1 || in.material >= d->n_materials)
      return ctx->fail(BN_ERR_INVALID_ARG, "instance " + std::to_string(i) + ": material out of range");
    if (in.light < -1 || in.light >= d->n_lights)
      return ctx->fail(BN_ERR_INVALID_ARG, "instance " + std::to_string(i) + ": light out of range");
  }
  for (int i = 0; i < d->n_materials; ++i)
    if (d->materials[i].type < BN_MAT_LAMBERTIAN || d->materials[i].type > BN_MAT_PBR)
      return ctx->fail(BN_ERR_INVALID_ARG, "material " + std::to_string(i) + ": unknown type");

  // ---- 1+2: BLAS per mesh, permuted triangles, reference alias pdf
  if (d->bvh_builder != BN_BUILDER_AUTO && d->bvh_builder != BN_BUILDER_HOST && d->bvh_builder != BN_BUILDER_DEVICE)
    return ctx->fail(BN_ERR_INVALID_ARG, "bvh_builder must be 0 (auto), 1 (host) or 2 (device)");
  auto on_device = [&](int n) {
    return d->bvh_builder == BN_BUILDER_DEVICE || (d->bvh_builder == BN_BUILDER_AUTO && n >= 16384);
  };
  std::vector<MeshPrep> mp(d->n_meshes);
  std::vector<float4> tris;
  std::vector<float> tri_pdf;
  std::vector<bn_bvh_node> all_nodes;  // TLAS inserted in front later
  size_t blas_nodes = 0;
  for (int i = 0; i < d->n_meshes; ++i) {
    const bn_mesh_desc& m = d->meshes[i];
    std::vector<float> boxes(6 * static_cast<size_t>(m.n_triangles));
    for (int t = 0; t < m.n_triangles; ++t) {
      const V3 p0 = vtx(m, m.indices[3 * t]), p1 = vtx(m, m.indices[3 * t + 1]), p2 = vtx(m, m.indices[3 * t + 2]);
      const V3 lo = bnh::min_native(bnh::min_native(p0, p1), p2), hi = bnh::max_native(bnh::max_native(p0, p1), p2);
      float* b = &boxes[6 * static_cast<size_t>(t)];
      b[0] = lo.x; b[1] = lo.y; b[2] = lo.z; b[3] = hi.x; b[4] = hi.y; b[5] = hi.z;
    }
    if (on_device(m.n_triangles)) {
      const int rc = bnc::gpu_bvh_build(ctx, boxes.data(), m.n_triangles, &mp[i].nodes, &mp[i].perm, 256);
      if (rc) return rc;
    } else if (!bnh::bvh_build(boxes.data(), m.n_triangles, &mp[i].nodes, &mp[i].perm)) {
      return ctx->fail(BN_ERR_UNSUPPORTED, "mesh " + std::to_string(i) + ": BVH leaf larger than 127 triangles");
    }
    mp[i].tri_base = static_cast<int>(tris.size() / 3);
    mp[i].node_base = static_cast<int>(blas_nodes);
    blas_nodes += mp[i].nodes.size();
    std::vector<float> areas(m.n_triangles);
    float sum = 0.f;
    for (int k = 0; k < m.n_triangles; ++k) {
      const int t = mp[i].perm[k];
      const V3 p0 = vtx(m, m.indices[3 * t]), p1 = vtx(m, m.indices[3 * t + 1]), p2 = vtx(m, m.indices[3 * t + 2]);
      const int slot = m.tri_material ? m.tri_material[t] : -1;
      float slotf, tf;
      std::memcpy(&slotf, &slot, 4);
      std::memcpy(&tf, &t, 4);
      tris.push_back(make_float4(p0.x, p0.y, p0.z, slotf));
      tris.push_back(make_float4(p1.x, p1.y, p1.z, tf));
      tris.push_back(make_float4(p2.x, p2.y, p2.z, 0.f));
      areas[k] = 0.5f * bnh::length(bnh::cross(p1 - p0, p2 - p0));
      sum = sum + areas[k];
    }
    for (int k = 0; k < m.n_triangles; ++k)
      tri_pdf.push_back(sum == 0.f ? 1.f / static_cast<float>(m.n_triangles) : areas[k] / sum);
  }

  // ---- 3: instance world bounds
  const int ni = d->n_instances;
  std::vector<float> ibox(6 * static_cast<size_t>(ni));
  for (int i = 0; i < ni; ++i) {
    const bn_instance_desc& in = d->instances[i];
    const bn_primitive_desc& p = d->primitives[in.primitive];
    V3 lo, hi;
    if (p.type == BN_PRIM_SPHERE) {
      lo = {-p.radius, -p.radius, -p.radius};
      hi = {p.radius, p.radius, p.radius};
    } else {
      const bn_bvh_node& r = mp[p.mesh].nodes[0];
      lo = {r.bounds_min[0], r.bounds_min[1], r.bounds_min[2]};
      hi = {r.bounds_max[0], r.bounds_max[1], r.bounds_max[2]};
    }
    M4 o2w;
    std::memcpy(o2w.m, in.object_to_world, sizeof(o2w.m));
    const float inf = std::numeric_limits<float>::infinity();
    V3 wlo = {inf, inf, inf}, whi = {-inf, -inf, -inf};
    for (int c = 0; c < 8; ++c) {
      const V3 q = {(c & 1) ? hi.x : lo.x, (c & 2) ? hi.y : lo.y, (c & 4) ? hi.z : lo.z};
      const V3 w = bnh::transform_point(q, o2w);
      wlo = bnh::min_native(wlo, w);
      whi = bnh::max_native(whi, w);
    }
    float* b = &ibox[6 * static_cast<size_t>(i)];
    b[0] = wlo.x; b[1] = wlo.y; b[2] = wlo.z; b[3] = whi.x; b[4] = whi.y; b[5] = whi.z;
  }

  // ---- 4: TLAS
  std::vector<bn_bvh_node> tlas;
  std::vector<int32_t> order;
  if (on_device(ni)) {
    const int rc = bnc::gpu_bvh_build(ctx, ibox.data(), ni, &tlas, &order, 256);
    if (rc) return rc;
  } else if (!bnh::bvh_build(ibox.data(), ni, &tlas, &order)) {
    return ctx->fail(BN_ERR_UNSUPPORTED, "TLAS leaf larger than 127 instances");
  }
  const int n_tlas = static_cast<int>(tlas.size());
  std::vector<float4> nodes(2 * (tlas.size() + blas_nodes));
  for (size_t k = 0; k < tlas.size(); ++k) put_node(&nodes[2 * k], tlas[k]);
  for (int i = 0; i < d->n_meshes; ++i)
    for (size_t k = 0; k < mp[i].nodes.size(); ++k) put_node(&nodes[2 * (n_tlas + mp[i].node_base + k)], mp[i].nodes[k]);
  // wide records for every BVH with an interior root (the TLAS's first, at record 0) when the
  // scene is walked wide: asked for, or automatically for scenes of 1,024+ nodes
  if (d->bvh_width != BN_BVH_AUTO && d->bvh_width != BN_BVH_BINARY && d->bvh_width != BN_BVH_WIDE)
    return ctx->fail(BN_ERR_INVALID_ARG, "bvh_width must be 0 (auto), 2 or 4");
  const bool scene_wide = d->bvh_width == BN_BVH_WIDE || (d->bvh_width == BN_BVH_AUTO && nodes.size() / 2 >= 1024);
  std::vector<float4> nodes4;
  bool nested = true;
  if (scene_wide && !tlas[0].is_leaf) {
    Collapse c{tlas, nodes4};
    c.emit(0);
    nested = nested && c.nested;
  }
  for (int i = 0; i < d->n_meshes; ++i) {
    if (!scene_wide || mp[i].nodes[0].is_leaf) continue;
    Collapse c{mp[i].nodes, nodes4};
    mp[i].node4_root = c.emit(0);
    nested = nested && c.nested;
  }
  if (!nested) return ctx->fail(BN_ERR_INVALID_ARG, "non-finite triangle or instance bounds");
  if (nodes4.size() / 8 >= (size_t{1} << 29))  // a stacked leaf slot is -1 - (4 * record + slot)
    return ctx->fail(BN_ERR_UNSUPPORTED, "scene too large for the wide BVH records");
  if (nodes4.empty()) nodes4.resize(8);  // keep the buffer non-null

  std::vector<bn::DevInstance> dinst(ni);
  std::vector<int32_t> inst_light(ni);
  for (int k = 0; k < ni; ++k) {
    const bn_instance_desc& in = d->instances[order[k]];
    const bn_primitive_desc& p = d->primitives[in.primitive];
    bn::DevInstance& di = dinst[k];
    const float* b = &ibox[6 * static_cast<size_t>(order[k])];
    di.bmin = make_float4(b[0], b[1], b[2], 0.f);
    di.bmax = make_float4(b[3], b[4], b[5], p.type == BN_PRIM_SPHERE ? p.radius : 0.f);
    columns(in.world_to_object, di.w2o);
    columns(in.object_to_world, di.o2w);
    di.prim_type = p.type == BN_PRIM_SPHERE ? bn::kPrimSphere : bn::kPrimMesh;
    di.node_base = p.type == BN_PRIM_MESH ? n_tlas + mp[p.mesh].node_base : 0;
    di.tri_base = p.type == BN_PRIM_MESH ? mp[p.mesh].tri_base : 0;
    di.n_tris = p.type == BN_PRIM_MESH ? d->meshes[p.mesh].n_triangles : 0;
    di.material = in.material;
    di.light = in.light;
    di.light_entry_base = -1;
    di.node4_root = p.type == BN_PRIM_MESH ? mp[p.mesh].node4_root : -1;
    if (p.type == BN_PRIM_MESH) {
      const bn_bvh_node& r = mp[p.mesh].nodes[0];
      di.rbmin = make_float4(r.bounds_min[0], r.bounds_min[1], r.bounds_min[2], 0.f);
      di.rbmax = make_float4(r.bounds_max[0], r.bounds_max[1], r.bounds_max[2], 0.f);
    }
    inst_light[k] = in.light;
  }

  // ---- 5: light tables
  std::vector<int32_t> light_inst;
  for (int k = 0; k < ni; ++k)
    if (dinst[k].light >= 0) light_inst.push_back(k);
  if (light_inst.empty()) return ctx->fail(BN_ERR_INVALID_ARG, "LightSamplerBase: No light primitives found.");
  std::vector<bn::DevTriLight> tl;
  if (d->light_sampler == BN_LIGHTS_ALIAS_TRIANGLES) {
    std::vector<double> w;
    for (int k : light_inst) {
      bn::DevInstance& di = dinst[k];
      if (di.prim_type != bn::kPrimMesh)
        return ctx->fail(BN_ERR_UNSUPPORTED, "the alias-table light sampler needs triangle-mesh emitters");
      const bn_instance_desc& in = d->instances[order[k]];
      M4 o2w;
      std::memcpy(o2w.m, in.object_to_world, sizeof(o2w.m));
      const bn_light_desc& L = d->lights[in.light];
      const double lum = 0.2126 * L.emission[0] + 0.7152 * L.emission[1] + 0.0722 * L.emission[2];
      di.light_entry_base = static_cast<int>(tl.size());
      for (int j = 0; j < di.n_tris; ++j) {
        const float4* t = &tris[3 * static_cast<size_t>(di.tri_base + j)];
        const V3 p0 = bnh::transform_point({t[0].x, t[0].y, t[0].z}, o2w);
        const V3 p1 = bnh::transform_point({t[1].x, t[1].y, t[1].z}, o2w);
        const V3 p2 = bnh::transform_point({t[2].x, t[2].y, t[2].z}, o2w);
        const float area = 0.5f * bnh::length(bnh::cross(p1 - p0, p2 - p0));
        bn::DevTriLight e{};
        e.area = area;
        e.inst = k;
        e.tri = j;
        tl.push_back(e);
        w.push_back(static_cast<double>(area) * std::max(lum, 0.0));
      }
    }
    std::vector<float> prob, pmf;
    std::vector<int> alias;
    build_vose(w, &prob, &alias, &pmf);
    for (size_t e = 0; e < tl.size(); ++e) {
      tl[e].prob = prob[e];
      tl[e].alias = alias[e];
      tl[e].pmf = pmf[e];
    }
  } else if (d->light_sampler != BN_LIGHTS_UNIFORM) {
    return ctx->fail(BN_ERR_INVALID_ARG, "unknown light sampler");
  }

  // ---- materials and lights
  std::vector<bn::DevMaterial> mats(std::max(d->n_materials, 1));
  for (int i = 0; i < d->n_materials; ++i) {
    const bn_material_desc& m = d->materials[i];
    bn::DevMaterial& dm = mats[i];
    dm.type = m.type;
    dm.base[0] = m.base_color[0]; dm.base[1] = m.base_color[1]; dm.base[2] = m.base_color[2];
    dm.ior = m.ior;
    const float a = m.roughness * m.roughness;
    dm.alpha = a > 1e-3f ? a : 1e-3f;  // MathF.Max(roughness^2, 1e-3) (PBR.fs:106)
    dm.metallic = std::min(std::max(m.metallic, 0.f), 1.f);
    dm.roughness = m.roughness;
  }
  std::vector<bn::DevLight> lights(std::max(d->n_lights, 1));
  for (int i = 0; i < d->n_lights; ++i) {
    lights[i].emission[0] = d->lights[i].emission[0];
    lights[i].emission[1] = d->lights[i].emission[1];
    lights[i].emission[2] = d->lights[i].emission[2];
    lights[i].two_sided = d->lights[i].two_sided;
  }

  // ---- upload
  cudaStream_t st = ctx->stream;
  cudaError_t e;
  if ((e = upload(ctx->nodes, nodes, st)) != cudaSuccess) return ctx->cuda_fail(e, "upload nodes");
  if ((e = upload(ctx->nodes4, nodes4, st)) != cudaSuccess) return ctx->cuda_fail(e, "upload wide nodes");
  if ((e = upload(ctx->tris, tris, st)) != cudaSuccess) return ctx->cuda_fail(e, "upload triangles");
  if ((e = upload(ctx->inst, dinst, st)) != cudaSuccess) return ctx->cuda_fail(e, "upload instances");
  if ((e = upload(ctx->mats, mats, st)) != cudaSuccess) return ctx->cuda_fail(e, "upload materials");
  if ((e = upload(ctx->lights, lights, st)) != cudaSuccess) return ctx->cuda_fail(e, "upload lights");
  if ((e = upload(ctx->light_inst, light_inst, st)) != cudaSuccess) return ctx->cuda_fail(e, "upload light list");
  if ((e = upload(ctx->tri_pdf, tri_pdf, st)) != cudaSuccess) return ctx->cuda_fail(e, "upload triangle pdf");
  if ((e = upload(ctx->tri_lights, tl, st)) != cudaSuccess) return ctx->cuda_fail(e, "upload light table");
  if ((e = cudaStreamSynchronize(st)) != cudaSuccess) return ctx->cuda_fail(e, "scene upload");

  bn::DevScene& s = ctx->scene;
  s.nodes = ctx->nodes.as<float4>();
  s.nodes4 = ctx->nodes4.as<float4>();
  s.tris = ctx->tris.as<float4>();
  s.inst = ctx->inst.as<bn::DevInstance>();
  s.mats = ctx->mats.as<bn::DevMaterial>();
  s.lights = ctx->lights.as<bn::DevLight>();
  s.light_inst = ctx->light_inst.as<int>();
  s.tri_pdf = ctx->tri_pdf.as<float>();
  s.tri_lights = ctx->tri_lights.as<bn::DevTriLight>();
  s.n_inst = ni;
  s.n_tlas_nodes = n_tlas;
  s.n_nodes = static_cast<int>(nodes.size() / 2);
  s.n_nodes4 = static_cast<int>(nodes4.size() / 8);
  s.wide = scene_wide ? 1 : 0;
  s.n_tris = static_cast<int>(tris.size() / 3);
  s.n_light_inst = static_cast<int>(light_inst.size());
  s.n_tri_lights = static_cast<int>(tl.size());
  s.light_sampler = d->light_sampler;
  s.n_mats = d->n_materials;
  s.stack_cap = ctx->limit_stack > 0 ? ctx->limit_stack : bn::kStackSize;
  s.error_word = ctx->error_word.as<unsigned int>();
  for (int a = 0; a < 3; ++a) {
    ctx->scene_lo[a] = tlas[0].bounds_min[a];
    ctx->scene_hi[a] = tlas[0].bounds_max[a];
  }
  bool simple = d->light_sampler == BN_LIGHTS_UNIFORM;
  for (int i = 0; i < d->n_materials; ++i) simple = simple && d->materials[i].type == BN_MAT_LAMBERTIAN;
  for (int k = 0; k < ni; ++k) simple = simple && dinst[k].prim_type == bn::kPrimMesh;
  ctx->scene_simple = simple;
  ctx->inst_order.assign(order.begin(), order.end());
  ctx->host_mats = mats;
  ctx->host_inst_light = inst_light;
  ctx->n_lights = d->n_lights;
  ctx->scene_generation += 1;
  ctx->has_scene = true;
  return BN_OK;
}
