// Two-level BVH traversal: TLAS -> PrimitiveInstance -> BLAS (included by dev_geometry.cuh).
//
// Order and culling are the reference's (Aggregate/BVH.fs:11-58, Primitive.fs:111-129,
// Mesh.fs:188-242): near child first (left when d[axis] > 0), the instances of a TLAS leaf in
// order, each instance's BLAS walked completely before the next, every box tested against the
// current t with tMin = 1e-3.  Changes of form keep the SIMT lanes together and the loads few:
//  * an interior node tests its children at once, enters the near one and pushes the far one
//    with its entry distance; on pop the far child is entered only if that distance is still
//    <= t, which is exactly the reference's box test at pop time (a box that passed with a
//    larger t passes with the current t iff its entry distance is <= t).
//  * the wide walk reads one 128-byte record per step that holds the two binary levels below
//    the node (its grandchildren, see dev_types.cuh) and tests the four boxes together.  It
//    visits them in the binary walk's order (near child's near child first, by the split axes
//    of the node and of each child) and stacks the hits that pass so that they pop in that
//    order.  Because a nested box passes whenever its parent box would with the same t, it
//    visits the same leaves in the same order with the same t as the binary walk.  A scene is
//    walked wide (kWalkWide) when the upload built records for it (large scenes; small BVHs gain
//    nothing from them).  The counting walk (kWalkCount) is always the binary one, so its counts
//    equal the reference's (the root plus both children of every entered interior node).
//  * the walk is a flat state machine: each step is one bounded unit of work (a node record or
//    pair, a leaf's triangles, a TLAS leaf's instances) at either BVH level, with pops folded
//    into the step that needs them, so lanes at different levels run the same loop body and
//    reconverge after every step instead of waiting out each other's nested BLAS loops.  A
//    caller can refill a lane with a new ray as soon as its walk finishes, and let only the
//    lanes at one kind of unit take a step (trav_vote).

namespace bn {

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

// the reference's near-child test d[axis] > 0 for the three axes at once (a zero or NaN component
// is not > 0, as in BVH.fs)
__device__ __forceinline__ int octant(V3 d) { return int(d.x > 0.f) | (int(d.y > 0.f) << 1) | (int(d.z > 0.f) << 2); }

struct Trav {
  Ray wr;            // world ray
  V3 winv;
  int woct;          // octant of the world direction: bit a set when d[a] > 0
  Ray orr;           // object-space ray of the instance being walked
  V3 oinv;
  int ooct;          // the same for the object-space direction
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
  bool any;          // any-hit query (runtime choice, kAnyRuntime walks)
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

// a leaf's item range: instances at the TLAS level, triangles at the BLAS level
__device__ __forceinline__ void trav_enter_leaf(Trav& tr, int first, int count) {
  if (tr.level == 0) {
    tr.ii = first;
    tr.ii_end = first + count;
    tr.mode = kTravInst;
  } else {
    tr.ti = first;
    tr.ti_end = first + count;
    tr.mode = kTravTri;
  }
}

// The walk's stack of far entries: a node or record index (or a leaf slot) with its entry
// distance.  LocalStack keeps them in the thread's local memory.  SharedStack keeps the bottom
// kShared entries in shared memory, one column per thread of a kBlock-thread block (lanes at
// different depths then fall on different banks), and the deeper ones in local memory, so the
// pushes and pops of a typical walk stay out of the L1 data cache the node loads use.
struct LocalStack {
  int sn[kStackSize];
  float st[kStackSize];
  __device__ __forceinline__ void put(int i, int n, float t) { sn[i] = n; st[i] = t; }
  __device__ __forceinline__ void get(int i, int* n, float* t) const { *n = sn[i]; *t = st[i]; }
};

template <int kShared, int kBlock>
struct SharedStack {
  int2* col;  // this thread's column of the block's kShared x kBlock array
  int sn[kStackSize - kShared];
  float st[kStackSize - kShared];
  __device__ __forceinline__ explicit SharedStack(int2* block_array) : col(block_array + threadIdx.x) {}
  __device__ __forceinline__ void put(int i, int n, float t) {
    if (i < kShared) {
      col[i * kBlock] = make_int2(n, __float_as_int(t));
    } else {
      sn[i - kShared] = n;
      st[i - kShared] = t;
    }
  }
  __device__ __forceinline__ void get(int i, int* n, float* t) const {
    if (i < kShared) {
      const int2 e = col[i * kBlock];
      *n = e.x;
      *t = __int_as_float(e.y);
    } else {
      *n = sn[i - kShared];
      *t = st[i - kShared];
    }
  }
};

__device__ __forceinline__ const float4* node4_at(const DevScene& s, int i) {
  return s.nodes4 + 8 * static_cast<size_t>(i);
}

// the next stacked node still within reach; an exhausted BLAS returns to the instances of its
// TLAS leaf, an exhausted TLAS ends the walk.  Binary entries are node indices within the level;
// wide entries are record indices (>= 0) or -1 - (4 * record + slot) for a leaf slot.
template <bool kWide, class Stack>
__device__ __forceinline__ void trav_pop(Trav& tr, const DevScene& s, const Stack& stk) {
  for (;;) {
    const int bottom = tr.level ? tr.blas_sp0 : 0;
    while (tr.sp > bottom) {
      --tr.sp;
      int c;
      float te;
      stk.get(tr.sp, &c, &te);
      if (te <= tr.t) {
        if (!kWide) {
          trav_enter(tr, c, load_node(s.nodes, tr.base + c));
        } else if (c >= 0) {
          tr.cur = c;
          tr.mode = kTravNode;
        } else {
          const int k = -1 - c, sl = k & 3;
          const int* rec = reinterpret_cast<const int*>(node4_at(s, k >> 2) + 6);
          trav_enter_leaf(tr, __ldg(rec + sl), (__ldg(rec + 4) >> (8 * sl)) & 0xff);
        }
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

// kWalk: which walk and whether it counts its visits
enum : int { kWalkBinary = 0, kWalkCount = 1, kWalkWide = 2 };

template <int kWalk>
__device__ __forceinline__ void trav_init(Trav& tr, const DevScene& s, const Ray& ray, float tmax, TraceCounters* cnt) {
  tr.wr = ray;
  tr.winv = inv_dir(ray.d);
  tr.woct = octant(ray.d);
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
  if (kWalk == kWalkCount) cnt->nodes++;
  float te;
  if (!box_hit_t(root.bmin, root.bmax, tr.wr, tr.winv, tr.t, &te)) {
    tr.mode = kTravDone;
  } else if (kWalk != kWalkWide || root.leaf) {
    trav_enter(tr, 0, root);
  } else {
    tr.cur = 0;  // the TLAS root's record
    tr.mode = kTravNode;
  }
}

__device__ __forceinline__ float sel4(float a, float b, float c, float d, int i) {
  return (i & 2) ? ((i & 1) ? d : c) : ((i & 1) ? b : a);
}
__device__ __forceinline__ int sel4(int a, int b, int c, int d, int i) {
  return (i & 2) ? ((i & 1) ? d : c) : ((i & 1) ? b : a);
}

// one wide step: the four slot boxes of record tr.cur; returns kStepPop when none is entered,
// kStepOverflow when the stack is full
enum : int { kStepOk = 0, kStepPop = 1, kStepOverflow = 2 };
template <class Stack>
__device__ __forceinline__ int trav_node4(Trav& tr, const DevScene& s, Stack& stk) {
  const Ray& r = tr.level ? tr.orr : tr.wr;
  const V3 inv = tr.level ? tr.oinv : tr.winv;
  const float4* q = node4_at(s, tr.cur);
  const float4 lx = __ldg(q), ly = __ldg(q + 1), lz = __ldg(q + 2);
  const float4 hx = __ldg(q + 3), hy = __ldg(q + 4), hz = __ldg(q + 5);
  const int4 ref = __ldg(reinterpret_cast<const int4*>(q + 6));
  const int4 meta = __ldg(reinterpret_cast<const int4*>(q + 7));
  float e0, e1, e2, e3;
  const bool h0 = box_hit_t(mk(lx.x, ly.x, lz.x), mk(hx.x, hy.x, hz.x), r, inv, tr.t, &e0);
  const bool h1 = box_hit_t(mk(lx.y, ly.y, lz.y), mk(hx.y, hy.y, hz.y), r, inv, tr.t, &e1);
  const bool h2 = box_hit_t(mk(lx.z, ly.z, lz.z), mk(hx.z, hy.z, hz.z), r, inv, tr.t, &e2);
  const bool h3 = box_hit_t(mk(lx.w, ly.w, lz.w), mk(hx.w, hy.w, hz.w), r, inv, tr.t, &e3);
  const int hm = int(h0) | (int(h1) << 1) | (int(h2) << 2) | (int(h3) << 3);
  if (!hm) return kStepPop;
  // the binary walk's order (the near child's slots, then the far child's, each pair ordered by
  // that child's own split axis: BVH.fs near-child rule at both levels) depends on the ray only
  // through its octant; the upload stored the slot order of each octant, 8 bits per octant
  const int m = meta.y;
  const int oct = tr.level ? tr.ooct : tr.woct;
  const unsigned order = (static_cast<unsigned>(oct & 4 ? meta.w : meta.z) >> (8 * (oct & 3))) & 0xffu;
  int v[4];
  v[0] = order & 3;
  v[1] = (order >> 2) & 3;
  v[2] = (order >> 4) & 3;
  v[3] = (order >> 6) & 3;
  int first = 3;
#pragma unroll
  for (int k = 2; k >= 0; --k)
    if ((hm >> v[k]) & 1) first = k;
  const int extra = __popc(hm) - 1;
  if (tr.sp + extra > s.stack_cap) return kStepOverflow;
  // stack the later hits so that they pop in visit order
#pragma unroll
  for (int k = 3; k >= 1; --k) {
    const int sl = v[k];
    if (k > first && ((hm >> sl) & 1)) {
      stk.put(tr.sp, ((m >> sl) & 1) ? -1 - (4 * tr.cur + sl) : sel4(ref.x, ref.y, ref.z, ref.w, sl),
              sel4(e0, e1, e2, e3, sl));
      ++tr.sp;
    }
  }
  const int sl = v[first];
  const int rf = sel4(ref.x, ref.y, ref.z, ref.w, sl);
  if ((m >> sl) & 1) trav_enter_leaf(tr, rf, (meta.x >> (8 * sl)) & 0xff);
  else tr.cur = rf;
  return kStepOk;
}

// one step: a wide record or a node pair, one instance (kInstRun: the leaf's instances until one
// is entered), or kTris triangles of a leaf (0 = the rest of it); returns true once the walk is
// finished (tr.found / tr.hit hold the answer).
// kAny: kClosest, kAnyHit, or kAnyRuntime (tr.any decides).  Every branch that exhausts its unit
// asks for a pop, which runs once at the end of the step.
enum : int { kClosest = 0, kAnyHit = 1, kAnyRuntime = 2 };
template <int kAny, bool kWT, int kWalk, int kTris = 1, bool kInstRun = false, class Stack>
__device__ __forceinline__ bool trav_step(Trav& tr, const DevScene& s, Stack& stk, TraceCounters* cnt) {
  constexpr bool kCount = kWalk == kWalkCount, kWide = kWalk == kWalkWide;
  const bool any = kAny == kAnyRuntime ? tr.any : kAny == kAnyHit;
  bool pop = false;
  if (kWide && tr.mode == kTravNode) {
    const int r = trav_node4(tr, s, stk);
    if (r == kStepOverflow) {
      flag_error(s, BN_DEVERR_STACK_OVERFLOW);
      tr.mode = kTravDone;
      return true;
    }
    pop = r == kStepPop;
  } else if (tr.mode == kTravNode) {
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
      if (tr.sp >= s.stack_cap) {
        flag_error(s, BN_DEVERR_STACK_OVERFLOW);
        tr.mode = kTravDone;
        return true;
      }
      if (left_first) { stk.put(tr.sp, ri, tb); ++tr.sp; trav_enter(tr, li, a); }
      else { stk.put(tr.sp, li, ta); ++tr.sp; trav_enter(tr, ri, b); }
    } else if (ha) {
      trav_enter(tr, li, a);
    } else if (hb) {
      trav_enter(tr, ri, b);
    } else {
      pop = true;
    }
  } else if (tr.mode == kTravTri) {
    // kTris triangles of a BLAS leaf (0: the rest of the leaf): each its AABB pre-test
    // (Mesh.fs:204,231), then the triangle test
    int done = 0;
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
          if (any) {
            tr.mode = kTravDone;
            return true;
          }
          tr.t = tt;
          tr.hit.inst = tr.inst; tr.hit.tri = j; tr.hit.t = tt; tr.hit.u = uu; tr.hit.v = vv; tr.hit.sphere_root = 0;
        }
      }
      if (kTris > 0 && ++done >= kTris) break;
    }
    pop = tr.ti >= tr.ti_end;
  } else if (tr.mode == kTravInst) {
    // the next instance of a TLAS leaf, or with kInstRun the leaf's instances until one is
    // entered (PrimitiveInstance.Intersect, Primitive.fs:111-129)
    bool entered = false;
#pragma unroll 1
    while (!entered && tr.ii < tr.ii_end) {
      const int k = tr.ii++;
      const DevInstance* I = s.inst + k;
      if (kCount) cnt->insts++;
      // the instance's first line in eight independent loads: bounds, WorldToObject, the BLAS
      // root's box and the indices, so one memory round trip serves the whole visit
      const float4* line = reinterpret_cast<const float4*>(I);
      const float4 bmin = __ldg(line), bmax = __ldg(line + 1);
      float4 w2o[3];
      w2o[0] = __ldg(line + 2); w2o[1] = __ldg(line + 3); w2o[2] = __ldg(line + 4);
      const float4 rlo = __ldg(line + 5), rhi = __ldg(line + 6);
      const int4 ids = __ldg(reinterpret_cast<const int4*>(line + 7));  // prim_type, node_base, tri_base, node4_root
      if (box_hit(xyz(bmin), xyz(bmax), tr.wr, tr.winv, tr.t)) {
        tr.orr.o = xf_point(w2o, tr.wr.o);
        tr.orr.d = xf_dir(w2o, tr.wr.d);
        if (ids.x == kPrimSphere) {
          float ts;
          const int root = sphere_hit(bmax.w, tr.orr, tr.t, &ts);
          if (root) {
            tr.found = true;
            if (any) {
              tr.mode = kTravDone;
              return true;
            }
            tr.t = ts;
            tr.hit.inst = k; tr.hit.tri = 0; tr.hit.sphere_root = root; tr.hit.t = ts; tr.hit.u = 0.f; tr.hit.v = 0.f;
          }
        } else {
          tr.oinv = inv_dir(tr.orr.d);
          tr.ooct = octant(tr.orr.d);
          if (kWT) tr.wt = wt_setup(tr.orr.d);
          const int base = ids.y;
          float te;
          if (kWide && ids.w >= 0) {
            // the root's box from the instance line, its record next (the root is interior)
            if (box_hit_t(xyz(rlo), xyz(rhi), tr.orr, tr.oinv, tr.t, &te)) {
              tr.level = 1;
              tr.base = base;
              tr.tri_base = ids.z;
              tr.inst = k;
              tr.blas_sp0 = tr.sp;
              tr.cur = ids.w;
              tr.mode = kTravNode;
              entered = true;
            }
          } else {
            const NodeRec root = load_node(s.nodes, base);
            if (kCount) cnt->nodes++;
            if (box_hit_t(root.bmin, root.bmax, tr.orr, tr.oinv, tr.t, &te)) {
              tr.level = 1;
              tr.base = base;
              tr.tri_base = ids.z;
              tr.inst = k;
              tr.blas_sp0 = tr.sp;
              trav_enter(tr, 0, root);
              entered = true;
            }
          }
        }
      }
      if (!kInstRun) break;
    }
    pop = !entered && tr.ii >= tr.ii_end;
  }
  if (pop) trav_pop<kWide>(tr, s, stk);
  return tr.mode == kTravDone;
}

// Lanes of a warp at different kinds of unit (a node record, a leaf's triangles, instances) run
// different branches of a step one after the other, each with its own chain of dependent loads.
// With this vote only the lanes in the mode with the largest weighted count take the step
// (instances weigh 3, nodes and triangles 2); the others keep their state and wait.  Each lane's
// sequence of units is unchanged, so its result is too.  Call it with every lane of the warp
// that is in the loop; walking = the lane holds a walk that is not finished.
__device__ __forceinline__ bool trav_vote(bool walking, int mode) {
  static_assert(kTravNode == 0 && kTravTri == 1 && kTravInst == 2 && kTravDone == 3, "mode bits");
  // two ballots on the mode's bits; a lane that is not walking counts as done (both bits)
  const unsigned act = __activemask();
  const unsigned b0 = __ballot_sync(act, !walking || (mode & 1)), b1 = __ballot_sync(act, !walking || (mode & 2));
  const int cn = 2 * __popc(act & ~(b0 | b1));
  const int ct = 2 * __popc(b0 & ~b1);
  const int ci = 3 * __popc(b1 & ~b0);
  const int pick = (cn >= ct && cn >= ci) ? kTravNode : (ct >= ci ? kTravTri : kTravInst);
  return mode == pick || mode == kTravDone;
}

// A walk, inlined at its call site with the query fixed at compile time.
template <int kAny, bool kWT, int kWalk>
__device__ __forceinline__ bool trace_walk_inline(const DevScene& s, const Ray& ray, float tmax, HitRec* hit,
                                                  TraceCounters* cnt) {
  LocalStack stk;
  Trav tr;
  trav_init<kWalk>(tr, s, ray, tmax, cnt);
  while (!trav_step<kAny, kWT, kWalk, 0>(tr, s, stk, cnt)) {
  }
  if (kAny == kClosest) *hit = tr.hit;
  return tr.found;
}

// One walk for both queries, kept out of line: a path loop that traces closest and any hits
// then holds a single copy of the traversal code.  That keeps a large kernel whose time goes to
// shading within the instruction cache; a kernel whose time goes to long walks keeps them
// inlined, where the walk's registers are allocated with the loop around it.
template <bool kWT, int kWalk>
__device__ __noinline__ bool trace_walk_outline(const DevScene& s, const Ray& ray, float tmax, bool any, HitRec* hit,
                                                TraceCounters* cnt) {
  LocalStack stk;
  Trav tr;
  tr.any = any;
  trav_init<kWalk>(tr, s, ray, tmax, cnt);
  while (!trav_step<kAnyRuntime, kWT, kWalk, 0>(tr, s, stk, cnt)) {
  }
  if (!any) *hit = tr.hit;
  return tr.found;
}

template <bool kWT, int kWalk, bool kOutline = false>
__device__ __forceinline__ bool trace_closest(const DevScene& s, const Ray& ray, float tmax, HitRec* hit, TraceCounters* cnt) {
  if (kOutline) return trace_walk_outline<kWT, kWalk>(s, ray, tmax, false, hit, cnt);
  return trace_walk_inline<kClosest, kWT, kWalk>(s, ray, tmax, hit, cnt);
}

template <bool kWT, int kWalk, bool kOutline = false>
__device__ __forceinline__ bool trace_any(const DevScene& s, const Ray& ray, float tmax, TraceCounters* cnt) {
  HitRec h;
  if (kOutline) return trace_walk_outline<kWT, kWalk>(s, ray, tmax, true, &h, cnt);
  return trace_walk_inline<kAnyHit, kWT, kWalk>(s, ray, tmax, &h, cnt);
}

}  // namespace bn
