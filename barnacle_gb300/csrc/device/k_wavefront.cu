// The batched wavefront form of PathTracingIntegrator.Li (PathTracing.fs:14-81) over many views.
//
// A pool of P path slots lives in HBM, one array per kind of record (WfParams: each slot's ray,
// throughput + radiance and hit are 32-byte records, one DRAM sector each).  One iteration of the
// bounce loop is:
//   regen    every slot (four 32-slot rows per warp): retire a finished path into the FP64 film,
//            refill free slots with new camera paths (warp-aggregated claims on a global path
//            counter), and append the active slots to the ray queue (ballot + popc compaction)
//            with their sort keys
//   sort     counting sort of the ray queue by key (octant, origin cell): scan + scatter
//   extend   closest hit for the ray queue (persistent lanes that vote on the kind of traversal
//            step, trav_vote); each hit is binned by the material type it shades
//            with (__match_any_sync groups, one atomic per group) so shading runs type-sorted
//   shade    emission with MIS, light sample + BSDF eval (a shadow-ray record), BSDF sample,
//            Russian roulette; marks paths that end
//   sort     the same counting sort of the shadow queue
//   shadow   any hit for the shadow queue; unoccluded records add their NEE term to L
//   control  one thread: decides whether another iteration is needed, resets the counters and
//            sets the CUDA-graph while-condition (or a flag for host-driven loops); an iteration
//            cap stops a runaway loop with BN_DEVERR_WATCHDOG.
// The arithmetic per path is the megakernel's (same helpers, same draw order, same operation
// order), so both forms produce the same per-path radiance; only the film summation order
// differs.  Kernels are persistent grid-stride loops whose trip counts come from device counters,
// so one captured graph serves every iteration.
#include "dev_shading.cuh"
#include "launch.hpp"
#include "wavefront.hpp"

namespace bn {
namespace {

constexpr int kStatusFree = 0, kStatusActive = 1, kStatusDone = 2;
constexpr int kBinMiss = 4, kBinNoMaterial = 5;
// the wavefront's traversal step: one wide record, up to 4 triangles of a BLAS leaf (a whole leaf
// but for the builder's depth-capped ones), or a TLAS leaf's instances until one is entered; only
// the lanes that win the mode vote (trav_vote) take it
constexpr int kWfTris = 4;
constexpr bool kWfInstRun = true;
// blocks of 128 per SM the traversal kernels are compiled for (registers: 65,536 / (128 x blocks))
constexpr int kExtendBlocks = 7, kShadowBlocks = 8;
// stack entries per lane kept in shared memory (8 bytes each, x 128 lanes per block)
constexpr int kWfSharedStack = 16;
using WfStack = SharedStack<kWfSharedStack, 128>;

__device__ __forceinline__ int warp_append(int* counter, bool pred) {
  // ballot + popc compaction: one atomic per warp
  const unsigned mask = __ballot_sync(0xffffffffu, pred);
  int base = 0;
  const int lane = threadIdx.x & 31;
  const int leader = __ffs(mask) - 1;
  if (lane == leader && mask) base = atomicAdd(counter, __popc(mask));
  base = __shfl_sync(0xffffffffu, base, leader < 0 ? 0 : leader);
  return base + __popc(mask & ((1u << lane) - 1u));
}

__device__ __forceinline__ int find_view(const WfParams& p, long long id) {
  int v = 0;
  while (v + 1 < p.n_views && p.views[v + 1].path_offset <= id) ++v;
  return v;
}

// Sort key of a ray: direction octant over the Morton code of the origin's cell in a
// 2^b x 8 x 2^b grid over the scene bounds (b = p.key_bits).  Rays next to each other in key order
// start in the same region in the same octant, so a warp of them walks much the same nodes.
__device__ __forceinline__ int ray_key(const WfParams& p, V3 o, V3 d) {
  const int nb = p.key_bits;
  const float top = static_cast<float>((1 << nb) - 1);
  // fmaxf maps a NaN coordinate to cell 0
  const unsigned x = static_cast<unsigned>(fminf(fmaxf((o.x - p.key_lo.x) * p.key_scale.x, 0.f), top));
  const unsigned y = static_cast<unsigned>(fminf(fmaxf((o.y - p.key_lo.y) * p.key_scale.y, 0.f), 7.f));
  const unsigned z = static_cast<unsigned>(fminf(fmaxf((o.z - p.key_lo.z) * p.key_scale.z, 0.f), top));
  // interleave x(b-1) z(b-1) y2 x(b-2) z(b-2) y1 x(b-3) z(b-3) y0 ... x0 z0 (2b + 3 bits)
  unsigned m = 0;
  int b = 0;
  for (int k = 0; k < nb; ++k) {
    m |= ((z >> k) & 1u) << b++;
    m |= ((x >> k) & 1u) << b++;
    if (k >= nb - 3) m |= ((y >> (k - (nb - 3))) & 1u) << b++;
  }
  const unsigned oct = (d.x < 0.f ? 1u : 0u) | (d.y < 0.f ? 2u : 0u) | (d.z < 0.f ? 4u : 0u);
  return static_cast<int>((oct << b) | m);
}

// histogram of the keys of the lanes with pred; lanes with equal keys share one atomic.  Called
// by whole warps.
__device__ __forceinline__ void hist_add(unsigned* hist, int key, bool pred) {
  const unsigned peers = __match_any_sync(0xffffffffu, pred ? key : -1);
  if (pred && (threadIdx.x & 31) == __ffs(peers) - 1) atomicAdd(hist + key, static_cast<unsigned>(__popc(peers)));
}

// One warp takes kRegenRows rows of 32 slots at a time: their states are loaded together, so a
// warp has that many independent loads in flight instead of one dependent chain per row, and the
// path claims and queue appends of all its rows share one atomic each.
constexpr int kRegenRows = 4;

__global__ void __launch_bounds__(256) k_wf_regen(const WfParams* __restrict__ pp) {
  const WfParams& p = *pp;
  const float inv_spp = __frcp_rn(static_cast<float>(p.spp));
  const int lane = threadIdx.x & 31;
  const unsigned below = (1u << lane) - 1u;
  const int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, n_warps = (gridDim.x * blockDim.x) >> 5;
  const int rows = (p.pool + 31) >> 5;
  // the loop runs in whole warps so the warp-wide claims and appends see all 32 lanes
  for (int r0 = warp * kRegenRows; r0 < rows; r0 += n_warps * kRegenRows) {
    int slot[kRegenRows];
    bool valid[kRegenRows];
    int4 m[kRegenRows];
#pragma unroll
    for (int k = 0; k < kRegenRows; ++k) {
      slot[k] = (r0 + k) * 32 + lane;
      valid[k] = slot[k] < p.pool;
      m[k] = valid[k] ? p.meta[slot[k]] : make_int4(0, 0, 0, kStatusActive);
    }
    // retire finished paths into the film
    float4 L[kRegenRows];
#pragma unroll
    for (int k = 0; k < kRegenRows; ++k)
      if (valid[k] && m[k].w == kStatusDone) L[k] = p.bl[2 * slot[k] + 1];
    // (lanes retiring samples of the same pixel could first sum in a warp and share one set of
    // atomics; measured 0.5% slower than one set per lane on the instanced workload)
#pragma unroll
    for (int k = 0; k < kRegenRows; ++k) {
      if (valid[k] && m[k].w == kStatusDone) {
        double* f = p.film_acc + 3LL * m[k].x;
        atomicAdd(f, static_cast<double>(__fmul_rn(L[k].x, inv_spp)));
        atomicAdd(f + 1, static_cast<double>(__fmul_rn(L[k].y, inv_spp)));
        atomicAdd(f + 2, static_cast<double>(__fmul_rn(L[k].z, inv_spp)));
        m[k].w = kStatusFree;
      }
    }
    // claim new paths for the free slots of all rows with one atomic
    unsigned wmask[kRegenRows];
    int nwant = 0;
#pragma unroll
    for (int k = 0; k < kRegenRows; ++k) {
      wmask[k] = __ballot_sync(0xffffffffu, valid[k] && m[k].w == kStatusFree);
      nwant += __popc(wmask[k]);
    }
    if (nwant) {
      unsigned long long first = 0;
      if (lane == 0) first = atomicAdd(p.work_next, static_cast<unsigned long long>(nwant));
      first = __shfl_sync(0xffffffffu, first, 0);
#pragma unroll
      for (int k = 0; k < kRegenRows; ++k) {
        const long long id = static_cast<long long>(first) + __popc(wmask[k] & below);
        first += __popc(wmask[k]);
        if (!((wmask[k] >> lane) & 1u) || id >= p.total_paths) continue;
        const int vi = find_view(p, id);
        const DevView& v = p.views[vi];
        // path ids run over the samples of a pixel first, so a warp's claims are mostly the
        // samples of one pixel (their retirements share atomics, see above)
        const long long local = id - v.path_offset;
        const long long pix = local / p.spp;
        const int sid = static_cast<int>(local - pix * p.spp);
        const int x = static_cast<int>(pix % v.width), y = static_cast<int>(pix / v.width);
        IndepSampler smp{xxhash32_three(static_cast<uint32_t>(x), static_cast<uint32_t>(y),
                                        static_cast<uint32_t>(p.frame_id * p.spp + sid))};
        const float upx = smp.next(), upy = smp.next();
        const float ulx = smp.next(), uly = smp.next();
        const Ray ray = camera_ray(v, x, y, upx, upy, ulx, uly);
        float4* rr = p.ray + 2 * slot[k];
        rr[0] = make_float4(ray.o.x, ray.o.y, ray.o.z, 0.f);
        rr[1] = make_float4(ray.d.x, ray.d.y, ray.d.z, 0.f);  // .w: pdf of the last BSDF sample
        if (p.sort) p.slot_key[slot[k]] = ray_key(p, ray.o, ray.d);
        float4* bl = p.bl + 2 * slot[k];
        bl[0] = make_float4(1.f, 1.f, 1.f, 0.f);
        bl[1] = make_float4(0.f, 0.f, 0.f, 0.f);
        const long long film_pix = v.pixel_offset + static_cast<long long>(v.height - y - 1) * v.width + x;
        m[k] = make_int4(static_cast<int>(film_pix), 0, static_cast<int>(smp.state), kStatusActive);
        // PathTracing: while (depth < maxDepth) never runs; Normal and Direct ignore maxDepth
        if (p.max_depth <= 0 && p.integrator == BN_INTEGRATOR_PATH) m[k].w = kStatusDone;
      }
    }
    // append the active slots of all rows to the ray queue with one atomic
    unsigned amask[kRegenRows];
    int nact = 0;
#pragma unroll
    for (int k = 0; k < kRegenRows; ++k) {
      amask[k] = __ballot_sync(0xffffffffu, valid[k] && m[k].w == kStatusActive);
      nact += __popc(amask[k]);
    }
    int qbase = 0;
    if (nact && lane == 0) qbase = atomicAdd(&p.counters[kCntActive], nact);
    qbase = __shfl_sync(0xffffffffu, qbase, 0);
#pragma unroll
    for (int k = 0; k < kRegenRows; ++k) {
      const bool active = (amask[k] >> lane) & 1u;
      const int qi = qbase + __popc(amask[k] & below);
      qbase += __popc(amask[k]);
      // a queue holds at most one entry per slot; the checks only guard the buffers
      const bool fits = qi < p.pool;
      if (active && !fits) flag_error(p.scene, BN_DEVERR_QUEUE_OVERFLOW);
      if (active && fits) p.q_active[qi] = slot[k];
      if (p.sort) {
        const int key = active ? p.slot_key[slot[k]] : 0;
        if (active && fits) p.q_key[qi] = key;
        hist_add(p.hist, key, active && fits);
      }
      if (valid[k]) p.meta[slot[k]] = m[k];
    }
  }
}

// a counting walk's totals: one atomic per warp and counter (every lane of the warp reaches it)
__device__ __forceinline__ void add_trace_counts(void* out, unsigned long long rays, const TraceCounters& tc) {
  unsigned long long r = rays, nn = tc.nodes, tt = tc.tris, ii = tc.insts;
  for (int o = 16; o > 0; o >>= 1) {
    r += __shfl_down_sync(0xffffffffu, r, o);
    nn += __shfl_down_sync(0xffffffffu, nn, o);
    tt += __shfl_down_sync(0xffffffffu, tt, o);
    ii += __shfl_down_sync(0xffffffffu, ii, o);
  }
  if ((threadIdx.x & 31) == 0) {
    DevCounters* c = static_cast<DevCounters*>(out);
    atomicAdd(&c->rays, r);
    atomicAdd(&c->nodes, nn);
    atomicAdd(&c->tris, tt);
    atomicAdd(&c->insts, ii);
  }
}

// Persistent lanes with dynamic ray fetch: a lane whose ray finished claims the next queued ray
// (one atomic per warp for all lanes that need one) and keeps stepping, so a warp never waits
// out its slowest ray with idle lanes while work remains in the queue.  Finished lanes wait until
// at most refill_below lanes of the warp still walk and are then written out and refilled
// together: the result stores, material lookups and ray loads are dependent-load chains, and
// running them for one lane at a time would stall the whole warp on almost every step.
__device__ __forceinline__ int fetch_next(int* counter, bool need) {
  const unsigned act = __activemask();
  const unsigned m = __ballot_sync(act, need);
  if (!m) return -1;
  const int lane = threadIdx.x & 31;
  const int leader = __ffs(m) - 1;
  int base = 0;
  if (lane == leader) base = atomicAdd(counter, __popc(m));
  base = __shfl_sync(act, base, leader);
  return need ? base + __popc(m & ((1u << lane) - 1u)) : -1;
}

// Lanes per warp that take rays.  A queue shorter than the resident lanes (the last bounces of a
// render, or PSSMLT's one ray per chain) is spread over every warp instead of filling the first
// warps' 32 lanes: more warps then walk at once and hide each other's load latency, and a launch
// ends sooner after its slowest walk.  Counting walks keep all lanes (their totals are reduced
// over whole warps).
template <int kWalk>
__device__ __forceinline__ int lanes_taking_rays(int n) {
  if (kWalk == kWalkCount) return 32;
  const int warps = (gridDim.x * blockDim.x) >> 5;
  return min(32, max(1, (n + warps - 1) / warps));
}

template <bool kWT, int kWalk>
__global__ void __launch_bounds__(128, kExtendBlocks) k_wf_extend(const WfParams* __restrict__ pp) {
  const WfParams& p = *pp;
  const DevScene& s = p.scene;
  const int n = min(p.counters[kCntActive], p.pool);
  const int refill_below = p.refill_extend;
  if ((threadIdx.x & 31) >= lanes_taking_rays<kWalk>(n)) return;
  __shared__ int2 stack_block[kWfSharedStack * 128];
  WfStack stk(stack_block);
  Trav tr;
  TraceCounters tc{0, 0, 0};
  unsigned long long nrays = 0;  // rays this lane walked (counting walks)
  int slot = -1;
  bool have = false, pending = false;
  for (;;) {
    if (__popc(__ballot_sync(__activemask(), have)) <= refill_below) {
      if (pending) {
        pending = false;
        int bin = kBinMiss;
        if (tr.found) {
          const HitRec& h = tr.hit;
          float4* hr = p.hit + 2 * slot;
          hr[0] = make_float4(h.t, h.u, h.v, __int_as_float(h.inst));
          hr[1] = make_float4(__int_as_float(h.sphere_root ? h.sphere_root : h.tri), 0.f, 0.f, 0.f);
          const DevInstance* I = s.inst + h.inst;
          int m = __ldg(&I->material);
          if (m >= 0 && __ldg(&I->prim_type) == kPrimMesh) {
            const int slot_m = __float_as_int(__ldg(&s.tris[3 * (__ldg(&I->tri_base) + h.tri)].w));
            if (slot_m >= 0) m = slot_m;
          }
          bin = m < 0 ? kBinNoMaterial : s.mats[m].type;
        } else {
          p.hit[2 * slot] = make_float4(0.f, 0.f, 0.f, __int_as_float(-1));
        }
        // material binning among the lanes finishing together: equal keys share one atomic
        const unsigned act = __activemask();
        const unsigned peers = __match_any_sync(act, bin);
        const int leader = __ffs(peers) - 1;
        const int lane = threadIdx.x & 31;
        int base = 0;
        if (lane == leader) base = atomicAdd(&p.counters[kCntBin0 + bin], __popc(peers));
        base = __shfl_sync(peers, base, leader);
        const int qb = base + __popc(peers & ((1u << lane) - 1u));
        if (qb < p.pool) p.q_bins[static_cast<long long>(bin) * p.pool + qb] = slot;
        else flag_error(s, BN_DEVERR_QUEUE_OVERFLOW);
      }
      const int qi = fetch_next(&p.counters[kCntFetchRay], !have);
      if (!have) {
        if (qi >= n) break;
        slot = p.q_ray[qi];
        const float4 o = p.ray[2 * slot], d = p.ray[2 * slot + 1];
        Ray ray;
        ray.o = mk(o.x, o.y, o.z);
        ray.d = mk(d.x, d.y, d.z);
        trav_init<kWalk>(tr, s, ray, CUDART_INF_F, &tc);
        have = true;
        ++nrays;
      }
    }
    // a walk can end at init (root box missed)
    const bool go = trav_vote(have, tr.mode);
    if (have && go && (tr.mode == kTravDone || trav_step<kClosest, kWT, kWalk, kWfTris, kWfInstRun>(tr, s, stk, &tc))) {
      have = false;
      pending = true;
    }
  }
  if (kWalk == kWalkCount) add_trace_counts(p.trace_counters, nrays, tc);
}

// DirectIntegrator.Li (Extensions/Integrator/Direct.fs:10-40) as two wavefront vertices.  At the
// camera hit: emission seen directly (EvalEmit(-d)), a shadow record for one light sample (a = f,
// b = L_light / pdf_light; the shadow kernel adds fma(a, b, L) if unoccluded, as the reference's
// FusedMultiplyAdd), and a BSDF sample that always continues with beta = f.  At the second hit:
// a light scores fma(beta, Le / pdf_light, L); the path ends either way.
__device__ __forceinline__ void shade_direct(const WfParams& p, const DevScene& s, int slot, const Ray& ray,
                                             const Interaction& it, int depth, IndepSampler& smp, V3* beta, V3* L,
                                             bool* done, bool* cont, bool* shadow, float4* sh_o, float4* sh_d,
                                             float4* sh_a, float4* sh_b) {
  const int light = __ldg(&s.inst[it.inst].light);
  if (depth > 0) {
    if (light >= 0) {
      V3 le;
      float pdf_l;
      eval_light(s, ray.o, it, &le, &pdf_l);
      *L = fma3(*beta, scale(__frcp_rn(pdf_l), le), *L);
    }
    *done = true;
    return;
  }
  const V3 wo_w = neg(ray.d);
  if (light >= 0) *L = add(*L, light_le(s.lights[light], dot(wo_w, it.f.n)));
  const int mat = hit_material(s, it);
  if (mat < 0) {
    *done = true;
    return;
  }
  const float u_sel = smp.next(), ulx = smp.next(), uly = smp.next();
  const DevMaterial mt = s.mats[mat];
  const LightSample ls = sample_light(s, it.p, u_sel, ulx, uly);
  const float dist = length(sub(ls.p, it.p));
  const BsdfEval be = bsdf_eval(mt, to_local(it.f, wo_w), to_local(it.f, ls.wi));
  const V3 bb = scale(__frcp_rn(ls.pdf), ls.L);
  *sh_o = make_float4(it.p.x, it.p.y, it.p.z, __fsub_rn(dist, 1e-3f));
  *sh_d = make_float4(ls.wi.x, ls.wi.y, ls.wi.z, __int_as_float(slot));
  *sh_a = make_float4(be.f.x, be.f.y, be.f.z, 0.f);
  *sh_b = make_float4(bb.x, bb.y, bb.z, 0.f);
  *shadow = shadow_contributes(be.f, bb, *L);
  const float u_lobe = smp.next(), ubx = smp.next(), uby = smp.next();
  const BsdfSample bs = bsdf_sample(mt, to_local(it.f, wo_w), u_lobe, ubx, uby);
  const V3 nd = to_world(it.f, bs.wi);
  *beta = bs.f;
  p.ray[2 * slot] = make_float4(it.p.x, it.p.y, it.p.z, 0.f);
  p.ray[2 * slot + 1] = make_float4(nd.x, nd.y, nd.z, bs.pdf);
  p.bl[2 * slot] = make_float4(bs.f.x, bs.f.y, bs.f.z, 0.f);
  if (p.sort) p.slot_key[slot] = ray_key(p, it.p, nd);
  *cont = true;
}

template <bool kWT>
__global__ void __launch_bounds__(128) k_wf_shade(const WfParams* __restrict__ pp) {
  const WfParams& p = *pp;
  const DevScene& s = p.scene;
  int cnt[kNumBins], total = 0;
  for (int b = 0; b < kNumBins; ++b) { cnt[b] = min(p.counters[kCntBin0 + b], p.pool); total += cnt[b]; }
  const int stride = gridDim.x * blockDim.x;
  const int nw = (total + 31) & ~31;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < nw; i += stride) {
    const bool valid = i < total;
    bool done = false, cont = false, shadow = false;
    int slot = 0;
    float4 sh_o, sh_d, sh_a, sh_b;
    if (valid) {
      int b = 0, off = i;
      while (off >= cnt[b]) { off -= cnt[b]; ++b; }
      slot = p.q_bins[static_cast<long long>(b) * p.pool + off];
      int4 m = p.meta[slot];
      const float4 hf = p.hit[2 * slot];
      const int hinst = __float_as_int(hf.w);
      if (hinst < 0) {
        done = true;
      } else {
        const float4 o = p.ray[2 * slot], d = p.ray[2 * slot + 1];
        Ray ray;
        ray.o = mk(o.x, o.y, o.z);
        ray.d = mk(d.x, d.y, d.z);
        const float pdf_bsdf = d.w;
        const int hprim = __float_as_int(p.hit[2 * slot + 1].x);
        HitRec h;
        h.t = hf.x; h.u = hf.y; h.v = hf.z;
        h.inst = hinst;
        const bool sphere = __ldg(&s.inst[hinst].prim_type) == kPrimSphere;
        h.tri = sphere ? 0 : hprim;
        h.sphere_root = sphere ? hprim : 0;
        const Interaction it = make_interaction(s, ray, h);
        const float4 b4 = p.bl[2 * slot];
        V3 beta = mk(b4.x, b4.y, b4.z);
        float4 L4 = p.bl[2 * slot + 1];
        V3 L = mk(L4.x, L4.y, L4.z);
        const int depth = m.y;
        const DevInstance* I = s.inst + it.inst;
        IndepSampler smp{static_cast<uint32_t>(m.z)};
        if (p.integrator == BN_INTEGRATOR_NORMAL) {
          L = normal_color(it.f.n);
          done = true;
        } else if (p.integrator == BN_INTEGRATOR_DIRECT) {
          shade_direct(p, s, slot, ray, it, depth, smp, &beta, &L, &done, &cont, &shadow, &sh_o, &sh_d, &sh_a, &sh_b);
          if (cont) m.y = 1;
        } else {
        if (__ldg(&I->light) >= 0) {
          V3 le;
          float pdf_l;
          eval_light(s, ray.o, it, &le, &pdf_l);
          const float mis = depth == 0 ? 1.f : __fmul_rn(pdf_bsdf, __frcp_rn(__fadd_rn(pdf_l, pdf_bsdf)));
          L = fma3(beta, scale(mis, le), L);
        }
        const int mat = hit_material(s, it);
        if (mat < 0) {
          done = true;
        } else {
          const float u_sel = smp.next(), ulx = smp.next(), uly = smp.next();
          const DevMaterial mt = s.mats[mat];
          const V3 wo_w = neg(ray.d);
          const LightSample ls = sample_light(s, it.p, u_sel, ulx, uly);
          const float dist = length(sub(ls.p, it.p));
          if (ls.pdf != 0.f) {
            const BsdfEval be = bsdf_eval(mt, to_local(it.f, wo_w), to_local(it.f, ls.wi));
            const V3 a = mul(beta, be.f);
            const V3 bb = scale(__frcp_rn(__fadd_rn(be.pdf, ls.pdf)), ls.L);
            sh_o = make_float4(it.p.x, it.p.y, it.p.z, __fsub_rn(dist, 1e-3f));
            sh_d = make_float4(ls.wi.x, ls.wi.y, ls.wi.z, __int_as_float(slot));
            sh_a = make_float4(a.x, a.y, a.z, 0.f);
            sh_b = make_float4(bb.x, bb.y, bb.z, 0.f);
            shadow = shadow_contributes(a, bb, L);
          }
          const float u_lobe = smp.next(), ubx = smp.next(), uby = smp.next();
          const BsdfSample bs = bsdf_sample(mt, to_local(it.f, wo_w), u_lobe, ubx, uby);
          if (bs.pdf == 0.f) {
            done = true;
          } else {
            const V3 nd = to_world(it.f, bs.wi);
            beta = scale(__frcp_rn(bs.pdf), mul(beta, bs.f));
            bool alive = true;
            if (depth >= p.rr_depth) {
              const float q = fminf(1.f, fmaxf(beta.x, fmaxf(beta.y, beta.z)));
              if (smp.next() < q) beta = scale(__frcp_rn(q), beta);
              else alive = false;
            }
            if (alive && depth + 1 < p.max_depth) {
              cont = true;
              p.ray[2 * slot] = make_float4(it.p.x, it.p.y, it.p.z, 0.f);
              p.ray[2 * slot + 1] = make_float4(nd.x, nd.y, nd.z, bs.pdf);
              if (p.sort) p.slot_key[slot] = ray_key(p, it.p, nd);
              p.bl[2 * slot] = make_float4(beta.x, beta.y, beta.z, 0.f);
              m.y = depth + 1;
            } else {
              done = true;
            }
          }
        }
        }
        p.bl[2 * slot + 1] = make_float4(L.x, L.y, L.z, 0.f);
        m.z = static_cast<int>(smp.state);
      }
      if (done) m.w = kStatusDone;
      p.meta[slot] = m;
    }
    int si = warp_append(&p.counters[kCntShadow], shadow);
    if (shadow && si >= p.pool) {
      flag_error(s, BN_DEVERR_QUEUE_OVERFLOW);
      shadow = false;
    }
    if (shadow) {
      float4* r = p.shadow + 4LL * si;
      r[0] = sh_o; r[1] = sh_d; r[2] = sh_a; r[3] = sh_b;
    }
    if (p.sort_shadow) {
      const int key = shadow ? ray_key(p, mk(sh_o.x, sh_o.y, sh_o.z), mk(sh_d.x, sh_d.y, sh_d.z)) : 0;
      if (shadow) p.sh_key[si] = key;
      hist_add(p.hist, key, shadow);
    }
    const unsigned cm = __ballot_sync(0xffffffffu, cont), dm = __ballot_sync(0xffffffffu, done);
    if ((threadIdx.x & 31) == 0) {
      if (cm) atomicAdd(&p.counters[kCntCont], __popc(cm));
      if (dm) atomicAdd(&p.counters[kCntDone], __popc(dm));
    }
  }
}

template <bool kWT, int kWalk>
__global__ void __launch_bounds__(128, kShadowBlocks) k_wf_shadow(const WfParams* __restrict__ pp) {
  const WfParams& p = *pp;
  const int n = min(p.counters[kCntShadow], p.pool);
  const int refill_below = p.refill_shadow;
  if ((threadIdx.x & 31) >= lanes_taking_rays<kWalk>(n)) return;
  __shared__ int2 stack_block[kWfSharedStack * 128];
  WfStack stk(stack_block);
  Trav tr;
  TraceCounters tc{0, 0, 0};
  unsigned long long nrays = 0;  // rays this lane walked (counting walks)
  int rec = -1;
  bool have = false, pending = false;
  for (;;) {
    if (__popc(__ballot_sync(__activemask(), have)) <= refill_below) {
      if (pending) {
        pending = false;
        if (!tr.found) {
          const float4* r = p.shadow + 4LL * rec;
          const int slot = __float_as_int(r[1].w);
          const float4 a = r[2], b = r[3];
          float4 L = p.bl[2 * slot + 1];
          L.x = fmaf(a.x, b.x, L.x);
          L.y = fmaf(a.y, b.y, L.y);
          L.z = fmaf(a.z, b.z, L.z);
          p.bl[2 * slot + 1] = L;
        }
      }
      const int qi = fetch_next(&p.counters[kCntFetchShadow], !have);
      if (!have) {
        if (qi >= n) break;
        rec = p.sort_shadow ? p.q_shadow[qi] : qi;
        const float4* r = p.shadow + 4LL * rec;
        const float4 o = r[0], d = r[1];
        Ray ray;
        ray.o = mk(o.x, o.y, o.z);
        ray.d = mk(d.x, d.y, d.z);
        trav_init<kWalk>(tr, p.scene, ray, o.w, &tc);
        have = true;
        ++nrays;
      }
    }
    const bool go = trav_vote(have, tr.mode);
    if (have && go && (tr.mode == kTravDone || trav_step<kAnyHit, kWT, kWalk, kWfTris, kWfInstRun>(tr, p.scene, stk, &tc))) {
      have = false;
      pending = true;
    }
  }
  if (kWalk == kWalkCount) add_trace_counts(p.trace_counters, nrays, tc);
}

// counting sort, steps 1-2: bucket offsets = exclusive scan of the counts of the keys' 2^(2b + 6)
// bins, in tiles of 1024 bins (one block each, WfLaunch::sort_tiles): step 1 sums every tile,
// step 2 scans its tile on top of the sums of the tiles before it and clears the counts for the
// next use

__device__ __forceinline__ unsigned block_exclusive_scan(unsigned v, unsigned* total) {
  __shared__ unsigned warp_sum[32];
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  unsigned x = v;
  for (int o = 1; o < 32; o <<= 1) {
    const unsigned y = __shfl_up_sync(0xffffffffu, x, o);
    if (lane >= o) x += y;
  }
  if (lane == 31) warp_sum[wid] = x;
  __syncthreads();
  if (wid == 0) {
    unsigned w = warp_sum[lane];
    for (int o = 1; o < 32; o <<= 1) {
      const unsigned y = __shfl_up_sync(0xffffffffu, w, o);
      if (lane >= o) w += y;
    }
    warp_sum[lane] = w;
  }
  __syncthreads();
  *total = warp_sum[31];
  return x - v + (wid ? warp_sum[wid - 1] : 0u);
}

__global__ void __launch_bounds__(1024) k_wf_sort_tiles(const WfParams* __restrict__ pp) {
  const WfParams& p = *pp;
  unsigned total;
  block_exclusive_scan(p.hist[blockIdx.x * 1024 + threadIdx.x], &total);
  if (threadIdx.x == 0) p.off[kSortBins + blockIdx.x] = total;  // tile sums after the offsets
}

__global__ void __launch_bounds__(1024) k_wf_sort_scan(const WfParams* __restrict__ pp) {
  const WfParams& p = *pp;
  __shared__ unsigned tile_base;
  if (threadIdx.x < 32) {
    unsigned b = 0;
    for (int t = threadIdx.x; t < static_cast<int>(blockIdx.x); t += 32) b += p.off[kSortBins + t];
    for (int o = 16; o > 0; o >>= 1) b += __shfl_down_sync(0xffffffffu, b, o);
    if (threadIdx.x == 0) tile_base = b;
  }
  const int i = blockIdx.x * 1024 + threadIdx.x;
  const unsigned c = p.hist[i];
  unsigned total;
  const unsigned x = block_exclusive_scan(c, &total);  // its barriers also publish tile_base
  p.off[i] = tile_base + x;
  p.hist[i] = 0u;
}

// counting sort, step 2: every queue entry to its bucket (order within a bucket is arbitrary;
// per-path results do not depend on it)
__global__ void __launch_bounds__(256) k_wf_sort_scatter(const WfParams* __restrict__ pp, int shadow_queue) {
  const WfParams& p = *pp;
  const int n = min(p.counters[shadow_queue ? kCntShadow : kCntActive], p.pool);
  const int* keys = shadow_queue ? p.sh_key : p.q_key;
  int* out = shadow_queue ? p.q_shadow : p.q_ray;
  const int stride = gridDim.x * blockDim.x;
  const int nw = (n + 31) & ~31;
  const int lane = threadIdx.x & 31;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < nw; i += stride) {
    const bool valid = i < n;
    const int key = valid ? keys[i] : -1;
    const unsigned peers = __match_any_sync(0xffffffffu, key);
    const int leader = __ffs(peers) - 1;
    unsigned base = 0;
    if (valid && lane == leader) base = atomicAdd(p.off + key, static_cast<unsigned>(__popc(peers)));
    base = __shfl_sync(peers, base, leader);
    if (valid) out[base + __popc(peers & ((1u << lane) - 1u))] = shadow_queue ? i : p.q_active[i];
  }
}

__global__ void k_wf_control(WfParams* pp, int use_graph) {
  WfParams& p = *pp;
  int* c = p.counters;
  const bool more_work = *p.work_next < static_cast<unsigned long long>(p.total_paths);
  // PSSMLT chains: the chain regen counted the chains that are not finished into kCntDone
  bool again = p.mlt ? c[kCntDone] > 0 : (c[kCntCont] > 0 || c[kCntDone] > 0 || more_work);
  const int iter = ++c[kCntIter];
  if (again && iter >= p.max_iters) {
    atomicOr(p.scene.error_word, BN_DEVERR_WATCHDOG);
    again = false;
  }
  if (p.mlt) {
    // the chains' queues were filled this iteration for the next one
    c[kCntActive] = c[kCntActiveNext];
    c[kCntShadow] = c[kCntShadowNext];
    c[kCntActiveNext] = 0;
    c[kCntShadowNext] = 0;
  } else {
    c[kCntActive] = 0;
    c[kCntShadow] = 0;
  }
  c[kCntFetchRay] = 0;
  c[kCntFetchShadow] = 0;
  c[kCntCont] = 0;
  c[kCntDone] = 0;
  for (int b = 0; b < kNumBins; ++b) c[kCntBin0 + b] = 0;
  c[kCntAgain] = again ? 1 : 0;
  if (use_graph) cudaGraphSetConditional(p.cond, again ? 1u : 0u);
}

// FP64 film -> FP32 film (the rows were flipped when the pixel index was formed)
__global__ void k_wf_resolve(const WfParams* __restrict__ pp) {
  const WfParams& p = *pp;
  const long long n = 3LL * p.n_pixels;
  for (long long i = static_cast<long long>(blockIdx.x) * blockDim.x + threadIdx.x; i < n;
       i += static_cast<long long>(gridDim.x) * blockDim.x)
    p.film_out[i] = static_cast<float>(p.film_acc[i]);
}

template <class K>
int resident_grid(K kernel, int block) {
  int dev = 0, sms = 0, per = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, kernel, block, 0);
  return sms * (per > 0 ? per : 1);
}

}  // namespace

cudaError_t wf_launch_iteration(WfParams* dparams, const WfLaunch& l, bool use_graph, cudaStream_t st,
                                const WfFork* fk) {
  auto sort = [&](int shadow_queue) {
    if (!l.sort || (shadow_queue && !l.sort_shadow)) return;
    k_wf_sort_tiles<<<l.sort_tiles, 1024, 0, st>>>(dparams);
    k_wf_sort_scan<<<l.sort_tiles, 1024, 0, st>>>(dparams);
    k_wf_sort_scatter<<<l.grid_scatter, 256, 0, st>>>(dparams, shadow_queue);
  };
  cudaError_t e = cudaSuccess;
  auto go = [&](auto wt, auto walk) {
    constexpr bool kWT = decltype(wt)::value;
    constexpr int kWalk = decltype(walk)::value;
    if (l.mlt) {
      // PSSMLT chains: the shadow records of the last bounce are traced while the rays of the
      // next one are (they touch different fields of a slot: the shadow kernel adds to L, the
      // extension writes the hit), then shade, then the chains' Metropolis steps
      if (fk) {
        if ((e = cudaEventRecord(fk->fork, st)) != cudaSuccess) return;
        if ((e = cudaStreamWaitEvent(fk->side, fk->fork, 0)) != cudaSuccess) return;
      }
      k_wf_shadow<kWT, kWalk><<<l.grid_shadow, 128, 0, fk ? fk->side : st>>>(dparams);
      k_wf_extend<kWT, kWalk><<<l.grid_extend, 128, 0, st>>>(dparams);
      if (fk) {
        if ((e = cudaEventRecord(fk->join, fk->side)) != cudaSuccess) return;
        if ((e = cudaStreamWaitEvent(st, fk->join, 0)) != cudaSuccess) return;
      }
      mlt_launch_shade(dparams, l.grid_shade, kWT, l.mlt_kelemen, st);
      mlt_launch_regen(dparams, l.grid_regen, l.mlt_kelemen, st);
      return;
    }
    k_wf_regen<<<l.grid_regen, 256, 0, st>>>(dparams);
    sort(0);
    k_wf_extend<kWT, kWalk><<<l.grid_extend, 128, 0, st>>>(dparams);
    k_wf_shade<kWT><<<l.grid_shade, 128, 0, st>>>(dparams);
    sort(1);
    k_wf_shadow<kWT, kWalk><<<l.grid_shadow, 128, 0, st>>>(dparams);
  };
  using WT = std::integral_constant<bool, true>;
  using MT = std::integral_constant<bool, false>;
  using Bin = std::integral_constant<int, kWalkBinary>;
  using Cnt = std::integral_constant<int, kWalkCount>;
  using Wide = std::integral_constant<int, kWalkWide>;
  if (l.watertight) {
    if (l.count) go(WT{}, Cnt{});
    else if (l.wide) go(WT{}, Wide{});
    else go(WT{}, Bin{});
  } else {
    if (l.count) go(MT{}, Cnt{});
    else if (l.wide) go(MT{}, Wide{});
    else go(MT{}, Bin{});
  }
  if (e != cudaSuccess) return e;
  k_wf_control<<<1, 1, 0, st>>>(dparams, use_graph ? 1 : 0);
  return cudaGetLastError();
}

cudaError_t wf_launch_resolve(WfParams* dparams, cudaStream_t st) {
  k_wf_resolve<<<152 * 8, 256, 0, st>>>(dparams);
  return cudaGetLastError();
}

WfLaunch wf_launch_shape(bool watertight, bool wide, bool sort, bool sort_shadow, bool count, int blocks_per_sm_cap,
                         bool mlt, bool mlt_kelemen, long long mlt_chains, int key_bits) {
  WfLaunch l{};
  l.sort_tiles = (1 << (2 * key_bits + 6)) / 1024;
  l.mlt = mlt;
  l.mlt_kelemen = mlt_kelemen;
  l.watertight = watertight;
  l.wide = wide;
  l.count = count;
  l.sort = sort;
  l.sort_shadow = sort && sort_shadow;
  auto sms = [] {
    int n = 0, dev = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev);
    return n;
  };
  auto cap = [&](int g) { return blocks_per_sm_cap > 0 ? std::min(g, sms() * blocks_per_sm_cap) : g; };
  l.grid_regen = cap(mlt ? mlt_grid_regen() : resident_grid(k_wf_regen, 256));
  l.grid_scatter = resident_grid(k_wf_sort_scatter, 256);
  auto shape = [&](auto wt, auto walk) {
    constexpr bool kWT = decltype(wt)::value;
    constexpr int kWalk = decltype(walk)::value;
    l.grid_extend = cap(resident_grid(k_wf_extend<kWT, kWalk>, 128));
    l.grid_shade = cap(mlt ? mlt_grid_shade(kWT) : resident_grid(k_wf_shade<kWT>, 128));
    l.grid_shadow = cap(resident_grid(k_wf_shadow<kWT, kWalk>, 128));
    if (mlt_chains > 0) {
      // the two traversals run side by side, each with one lane per chain (a queue holds at most
      // one ray per chain): for 65,536 chains 512 blocks each, 512 x 128 x (72 + 64) registers,
      // 90 % of the SMs' together
      const int blocks = static_cast<int>(std::min<long long>((mlt_chains + 127) / 128, 1 << 30));
      l.grid_extend = std::min(l.grid_extend, blocks);
      l.grid_shadow = std::min(l.grid_shadow, blocks);
    }
  };
  using WT = std::integral_constant<bool, true>;
  using MT = std::integral_constant<bool, false>;
  using Bin = std::integral_constant<int, kWalkBinary>;
  using Cnt = std::integral_constant<int, kWalkCount>;
  using Wide = std::integral_constant<int, kWalkWide>;
  if (watertight) {
    if (count) shape(WT{}, Cnt{});
    else if (wide) shape(WT{}, Wide{});
    else shape(WT{}, Bin{});
  } else {
    if (count) shape(MT{}, Cnt{});
    else if (wide) shape(MT{}, Wide{});
    else shape(MT{}, Bin{});
  }
  return l;
}

}  // namespace bn
