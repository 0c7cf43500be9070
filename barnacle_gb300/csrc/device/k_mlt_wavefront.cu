// PSSMLT chains in the wavefront (PSSMLTIntegrator.RenderSingleChain, Extensions/Integrator/
// PSSMLT.fs:275-377, with PSSMLTIntegrator.Li, :172-245, one bounce per iteration).
//
// One path slot per Markov chain.  An iteration of the bounce loop is
//   shadow      any hit for the shadow records of the last iteration's bounce (the path tracer's
//   + extend    kernels), on a second stream alongside the closest hit for the rays queued by the
//               last iteration: a bounce waits for one walk instead of two in a row
//   mlt shade   PSSMLTIntegrator.Li's bounce with its fixed 7 draws from the chain's MLTSampler:
//               emission with MIS, a shadow record for the light sample when it can change the
//               radiance, the BSDF sample, Russian roulette
//   mlt regen   every chain whose path has ended (and whose last shadow record has been traced)
//               takes its Metropolis step (acceptance, the expected-value splats, Accept/Reject
//               of the primary samples) and starts its next mutation (StartIteration, the pixel and
//               lens draws, the camera ray); chains whose path goes on are queued as they are.  A
//               chain that has run all its mutations splats its last state and stops.
//   control     moves the queues filled this iteration into place; another iteration while any
//               chain is not finished.
// A chain whose path is short starts its next mutation at once instead of waiting for the
// longest path of its warp, and every traversal runs compacted and binned by material.  Each
// chain draws exactly the random numbers of the lockstep kernel (k_mlt_chains) in the same order
// and adds its path's terms to L in the same order (a bounce's emission, then its shadow term),
// so both forms give every chain the same mutations and decisions; only the film's summation
// order differs.  Primary samples are chain-major here: the 7 draws of a bounce read one chain's
// consecutive 16-byte records, which a lane fetches in a few sectors whatever its neighbours do.
#include "launch.hpp"
#include "mlt_sampler.cuh"
#include "wavefront.hpp"

namespace bn {
namespace {

// kChainWait: the path ended with a shadow record not yet traced; the chain steps one iteration
// later
constexpr int kChainFree = 0, kChainPath = 1, kChainStep = 2, kChainDone = 3, kChainWait = 4;
constexpr int kBinMiss = 4;

__device__ __forceinline__ int append(int* counter, bool pred) {
  const unsigned mask = __ballot_sync(0xffffffffu, pred);
  const int lane = threadIdx.x & 31;
  const int leader = __ffs(mask) - 1;
  int base = 0;
  if (lane == leader && mask) base = atomicAdd(counter, __popc(mask));
  base = __shfl_sync(0xffffffffu, base, leader < 0 ? 0 : leader);
  return base + __popc(mask & ((1u << lane) - 1u));
}

// kKelemen: the mutation strategy fixed at compile time (1 Kelemen, 0 Gaussian), so each kernel
// holds one strategy's code
template <int kKelemen>
__device__ __forceinline__ MltSampler chain_sampler(const MltWf& q, int chain) {
  MltSampler m;
  m.p_large = q.p_large;
  m.kelemen = kKelemen;
  m.sigma = q.sigma;
  m.eps_min = q.eps_min;
  m.eps_max = q.eps_max;
  m.log_eps = logf(__fdiv_rn(m.eps_max, m.eps_min));
  m.X = q.X + static_cast<long long>(chain) * q.n_dims;
  m.stride = 1;
  m.max_dims = q.n_dims;
  return m;
}

template <int kKelemen>
__global__ void __launch_bounds__(256) k_mlt_regen(const WfParams* __restrict__ pp) {
  const WfParams& p = *pp;
  const MltWf& q = p.mlt_p;
  const DevView& v = p.views[0];
  const int W = v.width, H = v.height;
  const float inv_b = __frcp_rn(q.b);
  unsigned long long accepted = 0;
  const int nw = (q.n_chains + 31) & ~31;
  // whole warps: the splats and the queue appends are warp-wide
  for (int chain = blockIdx.x * blockDim.x + threadIdx.x; chain < nw; chain += gridDim.x * blockDim.x) {
    const bool valid = chain < q.n_chains;
    int4 st = valid ? p.meta[chain] : make_int4(0, 0, 0, kChainDone);
    bool queued = valid && st.w == kChainPath;
    Splat step{-1, mk(0.f, 0.f, 0.f)}, last{-1, mk(0.f, 0.f, 0.f)};
    if (valid && (st.w == kChainFree || st.w == kChainStep)) {
      MltSampler m = chain_sampler<kKelemen>(q, chain);
      float4* cr = q.chain + 3LL * chain;
      float4 c0, c1, c2;
      if (st.w == kChainFree) {
        // the chain's start: AliasTable.Sample over the bootstrap weights (Util/AliasTable.fs:52-62)
        IndepSampler cs{xxhash32_two(static_cast<uint32_t>(p.frame_id), static_cast<uint32_t>(chain))};
        const float u = __fmul_rn(cs.next(), static_cast<float>(q.n_bootstrap));
        int bid = min(static_cast<int>(u), q.n_bootstrap - 1);
        if (q.alias_prob) {
          const float frac = __fsub_rn(u, static_cast<float>(bid));
          if (frac >= q.alias_prob[bid]) bid = q.alias_idx[bid];
        }
        m.inner = xxhash32_two(static_cast<uint32_t>(p.frame_id), static_cast<uint32_t>(bid));
        m.large_step = false;
        m.last_large = 0;
        m.cur_iter = 0;
        m.index = 0;
        m.initialized = 0;
        c0 = make_float4(0.f, 0.f, 0.f, 0.f);
        c1 = make_float4(0.f, 0.f, 0.f, __int_as_float(0));
        c2 = make_float4(__uint_as_float(cs.state), __int_as_float(-1), __int_as_float(0), __int_as_float(bid));
      } else {
        m.unpack(q.smp[chain]);
        c0 = cr[0];
        c1 = cr[1];
        c2 = cr[2];
        const float4 l4 = p.bl[2 * chain + 1];
        const V3 Ln = mk(l4.x, l4.y, l4.z);
        const float yn = luminance(Ln);
        const int it = __float_as_int(c2.y), npix = __float_as_int(c2.z);
        V3 L = mk(c0.x, c0.y, c0.z), radiance = mk(c1.x, c1.y, c1.z);
        float y = c0.w;
        int pix = __float_as_int(c1.w);
        if (it < 0) {
          // the starting path (the bootstrap sample the chain was drawn from)
          L = Ln;
          y = yn;
          m.accept();
          m.inner = xxhash32_three(static_cast<uint32_t>(chain), static_cast<uint32_t>(__float_as_int(c2.w)),
                                   static_cast<uint32_t>(p.frame_id));
          pix = npix;
        } else {
          IndepSampler cs{__float_as_uint(c2.x)};
          const float ratio = __fdiv_rn(yn, y);
          const float acc = ratio != ratio ? ratio : fminf(1.f, ratio);  // MathF.Min propagates NaN
          const float w_old = __fdiv_rn(__fsub_rn(1.f, acc), fmaf(y, inv_b, q.p_large));
          radiance = add(radiance, scale(w_old, L));
          const float w_new = __fdiv_rn(__fadd_rn(acc, m.large_step ? 1.f : 0.f), fmaf(yn, inv_b, q.p_large));
          if (cs.next() < acc) {
            ++accepted;
            step.pix = pix;
            step.c = scale(q.inv_eff_spp, radiance);
            radiance = scale(w_new, Ln);
            pix = npix;
            L = Ln;
            y = yn;
            m.accept();
          } else {
            if (acc > 0.f) {
              step.pix = npix;
              step.c = scale(__fmul_rn(w_new, q.inv_eff_spp), Ln);
            }
            m.reject();
          }
          c2.x = __uint_as_float(cs.state);
        }
        c0 = make_float4(L.x, L.y, L.z, y);
        c1 = make_float4(radiance.x, radiance.y, radiance.z, __int_as_float(pix));
        c2.y = __int_as_float(it + 1);
      }
      if (__float_as_int(c2.y) < q.mutations) {
        // the next mutation: StartIteration, then the pixel and lens draws of its camera ray
        m.start_iteration();
        int nx, ny;
        const Ray ray = mlt_camera(v, m, &nx, &ny);
        c2.z = __int_as_float((H - ny - 1) * W + nx);
        p.ray[2 * chain] = make_float4(ray.o.x, ray.o.y, ray.o.z, 0.f);
        p.ray[2 * chain + 1] = make_float4(ray.d.x, ray.d.y, ray.d.z, 0.f);
        p.bl[2 * chain] = make_float4(1.f, 1.f, 1.f, 0.f);
        p.bl[2 * chain + 1] = make_float4(0.f, 0.f, 0.f, 0.f);
        st = make_int4(0, 0, 0, kChainPath);
        if (p.max_depth <= 0) st.w = kChainStep;  // while (depth < maxDepth) never runs
        else queued = true;
      } else {
        last.pix = __float_as_int(c1.w);
        last.c = scale(q.inv_eff_spp, mk(c1.x, c1.y, c1.z));
        st.w = kChainDone;
      }
      q.smp[chain] = m.pack();
      cr[0] = c0;
      cr[1] = c1;
      cr[2] = c2;
    }
    warp_splat(q.film, step);
    warp_splat(q.film, last);
    // the shadow record of a waiting chain is traced in the next iteration: it steps in the one after
    if (valid && st.w == kChainWait) st.w = kChainStep;
    const int qi = append(&p.counters[kCntActiveNext], queued);
    if (queued && qi < p.pool) p.q_active[qi] = chain;
    else if (queued) flag_error(p.scene, BN_DEVERR_QUEUE_OVERFLOW);
    if (valid) p.meta[chain] = st;
    // chains not finished keep the loop going (k_wf_control reads the count)
    const unsigned pending = __ballot_sync(0xffffffffu, valid && st.w != kChainDone);
    if ((threadIdx.x & 31) == 0 && pending) atomicAdd(&p.counters[kCntDone], __popc(pending));
  }
  unsigned long long a = accepted;
  for (int o = 16; o > 0; o >>= 1) a += __shfl_down_sync(0xffffffffu, a, o);
  if ((threadIdx.x & 31) == 0 && a) atomicAdd(q.accepted, a);
}

template <bool kWT, int kKelemen>
__global__ void __launch_bounds__(128) k_mlt_shade(const WfParams* __restrict__ pp) {
  const WfParams& p = *pp;
  const MltWf& q = p.mlt_p;
  const DevScene& s = p.scene;
  int cnt[kNumBins], total = 0;
  for (int b = 0; b < kNumBins; ++b) { cnt[b] = min(p.counters[kCntBin0 + b], p.pool); total += cnt[b]; }
  const int stride = gridDim.x * blockDim.x;
  const int nw = (total + 31) & ~31;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < nw; i += stride) {
    const bool valid = i < total;
    bool done = false, cont = false, shadow = false;
    float4 sh_o, sh_d, sh_a, sh_b;
    if (valid) {
      int b = 0, off = i;
      while (off >= cnt[b]) { off -= cnt[b]; ++b; }
      const int slot = p.q_bins[static_cast<long long>(b) * p.pool + off];
      int4 st = p.meta[slot];
      const float4 hf = p.hit[2 * slot];
      const int hinst = __float_as_int(hf.w);
      if (b == kBinMiss || hinst < 0) {
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
        const float4 L4 = p.bl[2 * slot + 1];
        V3 L = mk(L4.x, L4.y, L4.z);
        const int depth = st.y;
        MltSampler m = chain_sampler<kKelemen>(q, slot);
        m.unpack(q.smp[slot]);
        if (__ldg(&s.inst[it.inst].light) >= 0) {
          V3 le;
          float pdf_l;
          eval_light(s, ray.o, it, &le, &pdf_l);
          const float mis = depth == 0 ? 1.f : __fmul_rn(pdf_bsdf, __frcp_rn(__fadd_rn(pdf_l, pdf_bsdf)));
          L = fma3(beta, scale(mis, le), L);
        }
        const int mat = hit_material(s, it);
        // PSSMLT.fs:201-205: seven draws per bounce whatever happens next
        float u7[7];
        m.next_n<7>(u7);
        const float u_sel = u7[0], ulx = u7[1], uly = u7[2];
        const float u_lobe = u7[3], ubx = u7[4], uby = u7[5], u_rr = u7[6];
        if (mat < 0) {
          done = true;
        } else {
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
          const BsdfSample bs = bsdf_sample(mt, to_local(it.f, wo_w), u_lobe, ubx, uby);
          if (bs.pdf == 0.f) {
            done = true;
          } else {
            const V3 nd = to_world(it.f, bs.wi);
            beta = scale(__frcp_rn(bs.pdf), mul(beta, bs.f));
            bool alive = true;
            if (depth >= p.rr_depth) {
              const float qq = fminf(1.f, fmaxf(beta.x, fmaxf(beta.y, beta.z)));
              if (u_rr < qq) beta = scale(__frcp_rn(qq), beta);
              else alive = false;
            }
            if (alive && depth + 1 < p.max_depth) {
              cont = true;
              p.ray[2 * slot] = make_float4(it.p.x, it.p.y, it.p.z, 0.f);
              p.ray[2 * slot + 1] = make_float4(nd.x, nd.y, nd.z, bs.pdf);
              p.bl[2 * slot] = make_float4(beta.x, beta.y, beta.z, 0.f);
              st.y = depth + 1;
            } else {
              done = true;
            }
          }
        }
        p.bl[2 * slot + 1] = make_float4(L.x, L.y, L.z, 0.f);
        q.smp[slot] = m.pack();
      }
      st.w = done ? (shadow ? kChainWait : kChainStep) : kChainPath;
      p.meta[slot] = st;
    }
    const int si = append(&p.counters[kCntShadowNext], shadow);
    if (shadow && si >= p.pool) {
      flag_error(s, BN_DEVERR_QUEUE_OVERFLOW);
      shadow = false;
    }
    if (shadow) {
      float4* r = p.shadow + 4LL * si;
      r[0] = sh_o; r[1] = sh_d; r[2] = sh_a; r[3] = sh_b;
    }
  }
}

template <class K>
int resident(K kernel, int block) {
  int dev = 0, sms = 0, per = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, kernel, block, 0);
  return sms * (per > 0 ? per : 1);
}

}  // namespace

cudaError_t mlt_launch_regen(WfParams* dparams, int grid, bool kelemen, cudaStream_t st) {
  if (kelemen) k_mlt_regen<1><<<grid, 256, 0, st>>>(dparams);
  else k_mlt_regen<0><<<grid, 256, 0, st>>>(dparams);
  return cudaGetLastError();
}

cudaError_t mlt_launch_shade(WfParams* dparams, int grid, bool watertight, bool kelemen, cudaStream_t st) {
  if (watertight) {
    if (kelemen) k_mlt_shade<true, 1><<<grid, 128, 0, st>>>(dparams);
    else k_mlt_shade<true, 0><<<grid, 128, 0, st>>>(dparams);
  } else {
    if (kelemen) k_mlt_shade<false, 1><<<grid, 128, 0, st>>>(dparams);
    else k_mlt_shade<false, 0><<<grid, 128, 0, st>>>(dparams);
  }
  return cudaGetLastError();
}

int mlt_grid_regen() { return resident(k_mlt_regen<1>, 256); }
int mlt_grid_shade(bool watertight) {
  return watertight ? resident(k_mlt_shade<true, 1>, 128) : resident(k_mlt_shade<false, 1>, 128);
}

}  // namespace bn
