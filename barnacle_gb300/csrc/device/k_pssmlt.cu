// Primary Sample Space Metropolis Light Transport (Extensions/Integrator/PSSMLT.fs).
//
//  k_mlt_bootstrap  BootstrapSingleChain (:247-273): one thread per bootstrap path, luminance y.
//                   A fresh MLTSampler's first iteration is a large step in which every
//                   dimension is drawn once from the inner sampler in order, so the bootstrap
//                   uses the inner sampler directly and stores no primary samples.
//  k_mlt_chains     RenderSingleChain (:275-377): one thread per chain.  The chain's primary
//                   samples live in HBM as [dimension][chain] float4 records
//                   (value, backup, last modification, backup of it), so a warp's 32 chains touch
//                   one 512-byte line per dimension.  Splats go through warp-aggregated atomics
//                   (lanes that splat to the same pixel are summed first) into the FP32 film.
// Kept from the reference: Reject restores every initialised dimension (:142-146); the
// acceptance min(1, y'/y) propagates NaN like MathF.Min; the chain's start is drawn from the
// AliasTable as built, which samples uniformly (Util/AliasTable.fs:20) unless the caller asks for
// the proportional table (BN_RENDER_FIXED_ALIAS).
#include "launch.hpp"
#include "mlt_sampler.cuh"
#include "pssmlt.hpp"

namespace bn {
namespace {

template <bool kWT, int kWalk>
__global__ void __launch_bounds__(128) k_mlt_bootstrap(MltParams p) {
  const int id = blockIdx.x * blockDim.x + threadIdx.x;
  if (id >= p.n_bootstrap) return;
  IndepSampler smp{xxhash32_two(static_cast<uint32_t>(p.frame_id), static_cast<uint32_t>(id))};
  int x, y;
  const Ray ray = mlt_camera(*p.view, smp, &x, &y);
  PathCounters pc{};
  const V3 L = li_path<kWT, true, kWalk, IndepSampler, false, false, true>(p.scene, ray, smp, p.max_depth, p.rr_depth, &pc);
  p.weights[id] = luminance(L);
}

// kKelemen: the mutation strategy fixed at compile time (1 Kelemen, 0 Gaussian), so the kernel
// holds one strategy's code
template <bool kWT, int kWalk, int kKelemen>
__global__ void __launch_bounds__(128) k_mlt_chains(MltParams p) {
  const int chain = blockIdx.x * blockDim.x + threadIdx.x;
  const bool valid = chain < p.n_chains;
  const DevView& v = *p.view;
  const int W = v.width, H = v.height;
  unsigned long long accepted = 0;
  if (valid) {
    IndepSampler cs{xxhash32_two(static_cast<uint32_t>(p.frame_id), static_cast<uint32_t>(chain))};
    // AliasTable.Sample over the bootstrap weights (Util/AliasTable.fs:52-62)
    float u = __fmul_rn(cs.next(), static_cast<float>(p.n_bootstrap));
    int bid = min(static_cast<int>(u), p.n_bootstrap - 1);
    if (p.alias_prob) {
      const float frac = __fsub_rn(u, static_cast<float>(bid));
      if (frac >= p.alias_prob[bid]) bid = p.alias_idx[bid];
    }
    MltSampler m;
    m.inner = xxhash32_two(static_cast<uint32_t>(p.frame_id), static_cast<uint32_t>(bid));
    m.large_step = false;
    m.last_large = 0;
    m.cur_iter = 0;
    m.index = 0;
    m.initialized = 0;
    m.p_large = p.large_step_prob;
    m.kelemen = kKelemen;
    m.sigma = p.sigma;
    m.eps_min = p.eps_min;
    m.eps_max = p.eps_max;
    m.log_eps = logf(__fdiv_rn(m.eps_max, m.eps_min));
    m.X = p.X + chain;
    m.stride = p.n_chains;
    m.max_dims = p.n_dims;
    PathCounters pc{};
    const float inv_b = __frcp_rn(p.b);
    const float inv_spp = p.inv_eff_spp;
    V3 radiance = mk(0.f, 0.f, 0.f), L = mk(0.f, 0.f, 0.f);
    float y = 0.f;
    int pix = 0;
    // iteration -1 evaluates the chain's starting path (the bootstrap sample it was drawn from);
    // one call site of the path loop keeps the kernel's code small
    for (int it = -1; it < p.mutations_per_chain; ++it) {
      m.start_iteration();
      int nx, ny;
      const Ray ray = mlt_camera(v, m, &nx, &ny);
      const V3 Ln = li_path<kWT, true, kWalk, MltSampler, false, false, true>(p.scene, ray, m, p.max_depth, p.rr_depth, &pc);
      const float yn = luminance(Ln);
      if (it < 0) {
        L = Ln;
        y = yn;
        m.accept();
        m.inner = xxhash32_three(static_cast<uint32_t>(chain), static_cast<uint32_t>(bid),
                                 static_cast<uint32_t>(p.frame_id));
        pix = (H - ny - 1) * W + nx;
        continue;
      }
      const float ratio = __fdiv_rn(yn, y);
      const float acc = ratio != ratio ? ratio : fminf(1.f, ratio);  // MathF.Min propagates NaN
      const float w_old = __fdiv_rn(__fsub_rn(1.f, acc), fmaf(y, inv_b, p.large_step_prob));
      radiance = add(radiance, scale(w_old, L));
      const float w_new = __fdiv_rn(__fadd_rn(acc, m.large_step ? 1.f : 0.f), fmaf(yn, inv_b, p.large_step_prob));
      const int npix = (H - ny - 1) * W + nx;
      Splat sp{-1, mk(0.f, 0.f, 0.f)};
      if (cs.next() < acc) {
        ++accepted;
        sp.pix = pix;
        sp.c = scale(inv_spp, radiance);
        radiance = scale(w_new, Ln);
        pix = npix;
        L = Ln;
        y = yn;
        m.accept();
      } else {
        if (acc > 0.f) {
          sp.pix = npix;
          sp.c = scale(__fmul_rn(w_new, inv_spp), Ln);
        }
        m.reject();
      }
      warp_splat(p.film, sp);
    }
    Splat last{pix, scale(inv_spp, radiance)};
    warp_splat(p.film, last);
  }
  unsigned long long a = accepted;
  for (int o = 16; o > 0; o >>= 1) a += __shfl_down_sync(0xffffffffu, a, o);
  if ((threadIdx.x & 31) == 0 && a) atomicAdd(p.accepted, a);
}

}  // namespace

cudaError_t launch_mlt_bootstrap(const MltParams& p, cudaStream_t st) {
  const int grid = (p.n_bootstrap + 127) / 128;
  dispatch_walk<false>(p.scene, p.watertight, false, [&](auto wt, auto walk) {
    k_mlt_bootstrap<decltype(wt)::value, decltype(walk)::value><<<grid, 128, 0, st>>>(p);
  });
  return cudaGetLastError();
}

cudaError_t launch_mlt_chains(const MltParams& p, cudaStream_t st) {
  const int grid = (p.n_chains + 127) / 128;
  dispatch_walk<false>(p.scene, p.watertight, false, [&](auto wt, auto walk) {
    if (p.kelemen) k_mlt_chains<decltype(wt)::value, decltype(walk)::value, 1><<<grid, 128, 0, st>>>(p);
    else k_mlt_chains<decltype(wt)::value, decltype(walk)::value, 0><<<grid, 128, 0, st>>>(p);
  });
  return cudaGetLastError();
}

}  // namespace bn
