// Two-level BVH traversal: TLAS -> PrimitiveInstance -> BLAS (included by dev_geometry.cuh).
//
// Order and culling are the reference's (Aggregate/BVH.fs:11-58, Primitive.fs:111-129,
// Mesh.fs:188-242): near child first (left when d[axis] > 0), the instances of a TLAS leaf in
// order, each instance's BLAS walked completely before the next, every box tested against the
// current t with tMin = 1e-3.  Two changes of form keep the SIMT lanes together:
//  * an interior node tests both children at once (their four 16-byte halves load together),
//    enters the near one and pushes the far one with its entry distance; on pop the far child is
//    entered only if that distance is still <= t, which is exactly the reference's box test at
//    pop time (a box that passed with a larger t passes with the current t iff its entry
//    distance is <= t).  Closest-hit visit counts equal the reference's: the root plus both
//    children of every entered interior node.
//  * the walk is a flat state machine: each step is one bounded unit of work (a node pair, one
//    triangle or one instance) at either BVH level, with pops folded into the step that needs
//    them, so lanes at different levels run the same loop body and reconverge after every step
//    instead of waiting out each other's nested BLAS loops.  A caller can refill a lane with a new
//    ray as soon as its walk finishes.

namespace bn {

constexpr int kStackSize = 136;  // TLAS and BLAS far-child entries of a depth-64 BVH pair

// the slab test that also reports the entry distance max(1e-3, t0') used by the pop check
__device__ __forceinline__ bool box_hit_t(V3 bmin, V3 bmax, const Ray& r, V3 inv, float tmax_in, float* tentry) {
  const float t0x = __fmul_rn(__fsub_rn(bmin.x, r.o.x), inv.x), t1x = __fmul_rn(__fsub_rn(bmax.x, r.o.x), inv.x);
  const float t0y = __fmul_rn(__fsub_rn(bmin.y, r.o.y), inv.y), t1y = __fmul_rn(__fsub_rn(bmax.y, r.o.y), inv.y);
  const float t0z = __fmul_rn(__fsub_rn(bmin.z, r.o.z), inv.z), t1z = __fmul_rn(__fsub_rn(bmax.z, r.o.z), inv.z);
  // fminf/fmaxf give the same decisions as MinNative/MaxNative here: they differ only when t1 is
  // NaN (minps/maxps return t1), and such boxes are rejected by the NaN check anyway; the sign of
  // a zero cannot change max(1e-3, ...) <= min(t, ...)
  const float tmin = fmaxf(1e-3f, fmaxf(fminf(t0x, t1x), fmaxf(fminf(t0y, t1y), fminf(t0z, t1z))));
  const float tmax = fminf(tmax_in, fminf(fmaxf(t0x, t1x), fminf(fmaxf(t0y, t1y), fmaxf(t0z, t1z))));
  const bool nan = (t1x != t1x) | (t1y != t1y) | (t1z != t1z);
  *tentry = tmin;
  return (tmin <= tmax) & !nan;
}

enum : int { kTravNode = 0, kTravTri = 1, kTravInst = 2, kTravDone = 3 };

struct Trav {
  Ray wr;            // world ray
  V3 winv;
  Ray orr;           // object-space ray of the instance being walked
  V3 oinv;
  WtRay wt;
  float t;
  NodeRec n;         // current interior node (kTravNode), its box already passed
  int mode, level;   // level 0 = TLAS, 1 = BLAS
  int cur, base;     // node index within the level, the level's base in nodes[]
  int tri_base, inst;
  int sp, blas_sp0;
  int ii, ii_end;    // instances of the TLAS leaf being processed
  int ti, ti_end;    // triangles of the BLAS leaf being processed
  bool found;
  HitRec hit;
};

// enter a node whose box passed: an interior node is walked, a leaf's items are iterated
__device__ __forceinline__ void trav_enter(Trav& tr, int cur, const NodeRec& n) {
  tr.cur = cur;
  if (!n.leaf) {
    tr.n = n;
    tr.mode = kTravNode;
  } else if (tr.level == 0) {
    tr.ii = n.link;
    tr.ii_end = n.link + n.count;
    tr.mode = kTravInst;
  } else {
    tr.ti = n.link;
    tr.ti_end = n.link + n.count;
    tr.mode = kTravTri;
  }
}

// the next stacked node still within reach; an exhausted BLAS returns to the instances of its
// TLAS leaf, an exhausted TLAS ends the walk
__device__ __forceinline__ void trav_pop(Trav& tr, const DevScene& s, const int* sn, const float* st) {
  for (;;) {
    const int bottom = tr.level ? tr.blas_sp0 : 0;
    while (tr.sp > bottom) {
      --tr.sp;
      if (st[tr.sp] <= tr.t) {
        const int c = sn[tr.sp];
        trav_enter(tr, c, load_node(s.nodes, tr.base + c));
        return;
      }
    }
    if (tr.level == 1) {
      tr.level = 0;
      tr.base = 0;
      if (tr.ii < tr.ii_end) {
        tr.mode = kTravInst;
        return;
      }
      continue;  // the TLAS leaf had no instance left: keep popping the TLAS
    }
    tr.mode = kTravDone;
    return;
  }
}

template <bool kCount>
__device__ __forceinline__ void trav_init(Trav& tr, const DevScene& s, const Ray& ray, float tmax, TraceCounters* cnt) {
  tr.wr = ray;
  tr.winv = inv_dir(ray.d);
  tr.t = tmax;
  tr.found = false;
  tr.hit.inst = -1;
  tr.sp = 0;
  tr.blas_sp0 = 0;
  tr.level = 0;
  tr.base = 0;
  tr.ii = tr.ii_end = 0;
  tr.ti = tr.ti_end = 0;
  const NodeRec root = load_node(s.nodes, 0);
  if (kCount) cnt->nodes++;
  float te;
  if (box_hit_t(root.bmin, root.bmax, tr.wr, tr.winv, tr.t, &te)) trav_enter(tr, 0, root);
  else tr.mode = kTravDone;
}

// one step (a node pair, one instance, and one triangle (kFine) or the rest of a leaf's
// triangles); returns true once the walk is finished (tr.found / tr.hit hold the answer).
// kFine suits lanes that are refilled with new rays; a single-ray walk runs fewer, coarser steps.
template <bool kAny, bool kWT, bool kCount, bool kFine = true>
__device__ __forceinline__ bool trav_step(Trav& tr, const DevScene& s, int* sn, float* st, TraceCounters* cnt) {
  if (tr.mode == kTravNode) {
    const Ray& r = tr.level ? tr.orr : tr.wr;
    const V3 inv = tr.level ? tr.oinv : tr.winv;
    const int li = tr.cur + 1, ri = tr.n.link;
    const NodeRec a = load_node(s.nodes, tr.base + li);
    const NodeRec b = load_node(s.nodes, tr.base + ri);
    if (kCount) cnt->nodes += 2;
    float ta, tb;
    const bool ha = box_hit_t(a.bmin, a.bmax, r, inv, tr.t, &ta);
    const bool hb = box_hit_t(b.bmin, b.bmax, r, inv, tr.t, &tb);
    const bool left_first = comp(r.d, tr.n.axis) > 0.f;
    if (ha && hb) {
      if (tr.sp >= kStackSize) {
        flag_error(s, BN_DEVERR_STACK_OVERFLOW);
        tr.mode = kTravDone;
        return true;
      }
      if (left_first) { sn[tr.sp] = ri; st[tr.sp] = tb; ++tr.sp; trav_enter(tr, li, a); }
      else { sn[tr.sp] = li; st[tr.sp] = ta; ++tr.sp; trav_enter(tr, ri, b); }
    } else if (ha) {
      trav_enter(tr, li, a);
    } else if (hb) {
      trav_enter(tr, ri, b);
    } else {
      trav_pop(tr, s, sn, st);
    }
  } else if (tr.mode == kTravTri) {
    // one triangle of a BLAS leaf: its AABB pre-test (Mesh.fs:204,231), then the triangle test
#pragma unroll 1
    while (tr.ti < tr.ti_end) {
    const int j = tr.ti++;
    const float4* tp = s.tris + 3 * (tr.tri_base + j);
    const float4 a = __ldg(tp), b = __ldg(tp + 1), c = __ldg(tp + 2);
    if (kCount) cnt->tris++;
    const V3 p0 = xyz(a), p1 = xyz(b), p2 = xyz(c);
    const V3 lo = min_native(min_native(p0, p1), p2), hi = max_native(max_native(p0, p1), p2);
    if (box_hit(lo, hi, tr.orr, tr.oinv, tr.t)) {
      float tt, uu, vv;
      const bool h = kWT ? tri_wt(p0, p1, p2, tr.orr, tr.wt, tr.t, &tt, &uu, &vv)
                         : tri_mt(p0, p1, p2, tr.orr, tr.t, &tt, &uu, &vv);
      if (h) {
        tr.found = true;
        if (kAny) {
          tr.mode = kTravDone;
          return true;
        }
        tr.t = tt;
        tr.hit.inst = tr.inst; tr.hit.tri = j; tr.hit.t = tt; tr.hit.u = uu; tr.hit.v = vv; tr.hit.sphere_root = 0;
      }
    }
    if (kFine) break;
    }
    if (tr.ti >= tr.ti_end) trav_pop(tr, s, sn, st);
  } else if (tr.mode == kTravInst) {
    // one instance of a TLAS leaf (PrimitiveInstance.Intersect, Primitive.fs:111-129)
    bool entered = false;
    if (tr.ii < tr.ii_end) {
    const int k = tr.ii++;
    const DevInstance* I = s.inst + k;
    if (kCount) cnt->insts++;
    const float4 bmin = __ldg(&I->bmin), bmax = __ldg(&I->bmax);
    if (box_hit(xyz(bmin), xyz(bmax), tr.wr, tr.winv, tr.t)) {
      float4 w2o[3];
      load_xf(I->w2o, w2o);
      tr.orr.o = xf_point(w2o, tr.wr.o);
      tr.orr.d = xf_dir(w2o, tr.wr.d);
      if (__ldg(&I->prim_type) == kPrimSphere) {
        float ts;
        const int root = sphere_hit(bmax.w, tr.orr, tr.t, &ts);
        if (root) {
          tr.found = true;
          if (kAny) {
            tr.mode = kTravDone;
            return true;
          }
          tr.t = ts;
          tr.hit.inst = k; tr.hit.tri = 0; tr.hit.sphere_root = root; tr.hit.t = ts; tr.hit.u = 0.f; tr.hit.v = 0.f;
        }
      } else {
        tr.oinv = inv_dir(tr.orr.d);
        if (kWT) tr.wt = wt_setup(tr.orr.d);
        const int base = __ldg(&I->node_base);
        const NodeRec root = load_node(s.nodes, base);
        if (kCount) cnt->nodes++;
        float te;
        if (box_hit_t(root.bmin, root.bmax, tr.orr, tr.oinv, tr.t, &te)) {
          tr.level = 1;
          tr.base = base;
          tr.tri_base = __ldg(&I->tri_base);
          tr.inst = k;
          tr.blas_sp0 = tr.sp;
          trav_enter(tr, 0, root);
          entered = true;
        }
      }
    }
    }
    if (!entered && tr.ii >= tr.ii_end) trav_pop(tr, s, sn, st);
  }
  return tr.mode == kTravDone;
}

template <bool kAny, bool kWT, bool kCount>
__device__ __forceinline__ bool trace_walk(const DevScene& s, const Ray& ray, float tmax, HitRec* hit, TraceCounters* cnt) {
  int sn[kStackSize];
  float st[kStackSize];
  Trav tr;
  trav_init<kCount>(tr, s, ray, tmax, cnt);
  while (!trav_step<kAny, kWT, kCount, false>(tr, s, sn, st, cnt)) {
  }
  if (!kAny) *hit = tr.hit;
  return tr.found;
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
