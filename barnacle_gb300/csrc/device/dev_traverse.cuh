// Two-level BVH traversal: TLAS -> PrimitiveInstance -> BLAS (included by dev_geometry.cuh).
//
// The reference pops a node, tests its box, and pushes both children of a hit interior node
// (Aggregate/BVH.fs:11-58, Mesh.fs:188-242).  Here an interior node tests both children at once:
// their four 16-byte halves load together, the near child (left when d[axis] > 0, as in the
// reference) is entered, and the far child is pushed with its entry distance.  A pushed child is
// entered on pop only if that distance is still <= t, which is exactly the reference's box test
// at pop time (a box that passed with a larger t passes with the current t iff its entry
// distance is <= t).  Nodes are therefore visited in the reference's order with the reference's
// culling, closest hits (and ties) come out identical, and the closest-hit visit counts equal
// the reference's (root + both children of every entered interior node).

namespace bn {

constexpr int kStackSize = 136;  // TLAS and BLAS far-child entries of a depth-64 BVH pair

// the slab test that also reports the entry distance max(1e-3, t0') used by the pop check
__device__ __forceinline__ bool box_hit_t(V3 bmin, V3 bmax, const Ray& r, V3 inv, float tmax_in, float* tentry) {
  const float t0x = __fmul_rn(__fsub_rn(bmin.x, r.o.x), inv.x), t1x = __fmul_rn(__fsub_rn(bmax.x, r.o.x), inv.x);
  const float t0y = __fmul_rn(__fsub_rn(bmin.y, r.o.y), inv.y), t1y = __fmul_rn(__fsub_rn(bmax.y, r.o.y), inv.y);
  const float t0z = __fmul_rn(__fsub_rn(bmin.z, r.o.z), inv.z), t1z = __fmul_rn(__fsub_rn(bmax.z, r.o.z), inv.z);
  const float lx = t0x < t1x ? t0x : t1x, hx = t0x > t1x ? t0x : t1x;
  const float ly = t0y < t1y ? t0y : t1y, hy = t0y > t1y ? t0y : t1y;
  const float lz = t0z < t1z ? t0z : t1z, hz = t0z > t1z ? t0z : t1z;
  const float tmin = fmaxf(1e-3f, fmaxf(lx, fmaxf(ly, lz)));
  const float tmax = fminf(tmax_in, fminf(hx, fminf(hy, hz)));
  const bool nan = (t1x != t1x) | (t1y != t1y) | (t1z != t1z);
  *tentry = tmin;
  return (tmin <= tmax) & !nan;
}

// result of a BLAS walk
struct BlasHit {
  float t, u, v;
  int tri;
};

// MeshPrimitive.Intersect (closest, Mesh.fs:217-242; any, Mesh.fs:188-215) on the object-space
// ray.  Uses the shared stack above `sp0`.  kAny: returns at the first hit.
template <bool kAny, bool kWT, bool kCount>
__device__ __forceinline__ bool blas_walk(const DevScene& s, int node_base, int tri_base, const Ray& oray, float t,
                                          BlasHit* out, int* sn, float* st, int sp0, TraceCounters* cnt) {
  const V3 oinv = inv_dir(oray.d);
  WtRay wt;
  if (kWT) wt = wt_setup(oray.d);
  bool found = false;
  int sp = sp0;
  NodeRec n = load_node(s.nodes, node_base);
  if (kCount) cnt->nodes++;
  float te;
  if (!box_hit_t(n.bmin, n.bmax, oray, oinv, t, &te)) return false;
  int cur = 0;
  for (;;) {
    if (n.leaf) {
      for (int j = n.link; j < n.link + n.count; ++j) {
        const float4* tp = s.tris + 3 * (tri_base + j);
        const float4 a = __ldg(tp), b = __ldg(tp + 1), c = __ldg(tp + 2);
        if (kCount) cnt->tris++;
        const V3 p0 = xyz(a), p1 = xyz(b), p2 = xyz(c);
        // the triangle's own AABB pre-test (Mesh.fs:204,231) then the triangle test
        const V3 lo = min_native(min_native(p0, p1), p2), hi = max_native(max_native(p0, p1), p2);
        if (!box_hit(lo, hi, oray, oinv, t)) continue;
        float tt, uu, vv;
        const bool h = kWT ? tri_wt(p0, p1, p2, oray, wt, t, &tt, &uu, &vv) : tri_mt(p0, p1, p2, oray, t, &tt, &uu, &vv);
        if (h) {
          if (kAny) return true;
          t = tt;
          found = true;
          out->t = tt; out->u = uu; out->v = vv; out->tri = j;
        }
      }
    } else {
      const int li = cur + 1, ri = n.link;
      const NodeRec a = load_node(s.nodes, node_base + li);
      const NodeRec b = load_node(s.nodes, node_base + ri);
      if (kCount) cnt->nodes += 2;
      float ta, tb;
      const bool ha = box_hit_t(a.bmin, a.bmax, oray, oinv, t, &ta);
      const bool hb = box_hit_t(b.bmin, b.bmax, oray, oinv, t, &tb);
      const bool left_first = comp(oray.d, n.axis) > 0.f;
      if (ha && hb) {
        if (sp >= kStackSize) { flag_error(s, BN_DEVERR_STACK_OVERFLOW); return found; }
        if (left_first) { sn[sp] = ri; st[sp] = tb; ++sp; cur = li; n = a; }
        else { sn[sp] = li; st[sp] = ta; ++sp; cur = ri; n = b; }
        continue;
      }
      if (ha) { cur = li; n = a; continue; }
      if (hb) { cur = ri; n = b; continue; }
    }
    bool next = false;
    while (sp > sp0) {
      --sp;
      if (st[sp] <= t) {
        cur = sn[sp];
        n = load_node(s.nodes, node_base + cur);
        next = true;
        break;
      }
    }
    if (!next) break;
  }
  return found;
}

// PrimitiveAggregate.Intersect: closest hit (kAny = false, Aggregate/BVH.fs:37-58) or any hit
// (kAny = true, :11-35), through PrimitiveInstance.Intersect (Primitive.fs:111-129).
template <bool kAny, bool kWT, bool kCount>
__device__ __forceinline__ bool trace_walk(const DevScene& s, const Ray& ray, float tmax, HitRec* hit, TraceCounters* cnt) {
  int sn[kStackSize];
  float st[kStackSize];
  int sp = 0;
  const V3 inv = inv_dir(ray.d);
  float t = tmax;
  bool found = false;
  if (!kAny) hit->inst = -1;
  NodeRec n = load_node(s.nodes, 0);
  if (kCount) cnt->nodes++;
  float te;
  if (!box_hit_t(n.bmin, n.bmax, ray, inv, t, &te)) return false;
  int cur = 0;
  for (;;) {
    if (n.leaf) {
      for (int k = n.link; k < n.link + n.count; ++k) {
        const DevInstance* I = s.inst + k;
        if (kCount) cnt->insts++;
        const float4 bmin = __ldg(&I->bmin), bmax = __ldg(&I->bmax);
        if (!box_hit(xyz(bmin), xyz(bmax), ray, inv, t)) continue;
        float4 w2o[3];
        load_xf(I->w2o, w2o);
        Ray oray;
        oray.o = xf_point(w2o, ray.o);
        oray.d = xf_dir(w2o, ray.d);
        if (__ldg(&I->prim_type) == kPrimSphere) {
          float ts;
          const int root = sphere_hit(bmax.w, oray, t, &ts);
          if (root) {
            if (kAny) return true;
            t = ts;
            found = true;
            hit->inst = k; hit->tri = 0; hit->sphere_root = root; hit->t = ts; hit->u = 0.f; hit->v = 0.f;
          }
          continue;
        }
        BlasHit bh;
        if (blas_walk<kAny, kWT, kCount>(s, __ldg(&I->node_base), __ldg(&I->tri_base), oray, t, &bh, sn, st, sp, cnt)) {
          if (kAny) return true;
          t = bh.t;
          found = true;
          hit->inst = k; hit->tri = bh.tri; hit->t = bh.t; hit->u = bh.u; hit->v = bh.v; hit->sphere_root = 0;
        }
      }
    } else {
      const int li = cur + 1, ri = n.link;
      const NodeRec a = load_node(s.nodes, li);
      const NodeRec b = load_node(s.nodes, ri);
      if (kCount) cnt->nodes += 2;
      float ta, tb;
      const bool ha = box_hit_t(a.bmin, a.bmax, ray, inv, t, &ta);
      const bool hb = box_hit_t(b.bmin, b.bmax, ray, inv, t, &tb);
      const bool left_first = comp(ray.d, n.axis) > 0.f;
      if (ha && hb) {
        if (sp >= kStackSize) { flag_error(s, BN_DEVERR_STACK_OVERFLOW); return found; }
        if (left_first) { sn[sp] = ri; st[sp] = tb; ++sp; cur = li; n = a; }
        else { sn[sp] = li; st[sp] = ta; ++sp; cur = ri; n = b; }
        continue;
      }
      if (ha) { cur = li; n = a; continue; }
      if (hb) { cur = ri; n = b; continue; }
    }
    bool next = false;
    while (sp > 0) {
      --sp;
      if (st[sp] <= t) {
        cur = sn[sp];
        n = load_node(s.nodes, cur);
        next = true;
        break;
      }
    }
    if (!next) break;
  }
  return found;
}

template <bool kWT, bool kCount>
__device__ __forceinline__ bool trace_closest(const DevScene& s, const Ray& ray, float tmax, HitRec* hit, TraceCounters* cnt) {
  return trace_walk<false, kWT, kCount>(s, ray, tmax, hit, cnt);
}

template <bool kWT, bool kCount>
__device__ __forceinline__ bool trace_any(const DevScene& s, const Ray& ray, float tmax, TraceCounters* cnt) {
  HitRec h;
  return trace_walk<true, kWT, kCount>(s, ray, tmax, &h, cnt);
}

}  // namespace bn
