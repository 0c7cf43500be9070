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
#include "dev_shading.cuh"
#include "launch.hpp"
#include "pssmlt.hpp"

namespace bn {
namespace {

// Giles' single-precision inverse error function ("Approximating the erfinv function", GPU
// Computing Gems Jade Edition, 2011), as the reference evaluates it (PSSMLT.fs:69-94)
__device__ __forceinline__ float erfinv_giles(float x) {
  x = fminf(fmaxf(x, -0.99999f), 0.99999f);
  float w = -logf(fmaf(x, -x, 1.f));
  float p;
  if (w < 5.f) {
    w = w - 2.5f;
    p = 2.81022636e-08f;
    p = fmaf(p, w, 3.43273939e-07f);
    p = fmaf(p, w, -3.5233877e-06f);
    p = fmaf(p, w, -4.39150654e-06f);
    p = fmaf(p, w, 0.00021858087f);
    p = fmaf(p, w, -0.00125372503f);
    p = fmaf(p, w, -0.00417768164f);
    p = fmaf(p, w, 0.246640727f);
    return __fmul_rn(fmaf(p, w, 1.50140941f), x);
  }
  w = __fsub_rn(sqrtf(w), 3.f);
  p = -0.000200214257f;
  p = fmaf(p, w, 0.000100950558f);
  p = fmaf(p, w, 0.00134934322f);
  p = fmaf(p, w, -0.00367342844f);
  p = fmaf(p, w, 0.00573950773f);
  p = fmaf(p, w, -0.0076224613f);
  p = fmaf(p, w, 0.00943887047f);
  p = fmaf(p, w, 1.00167406f);
  return __fmul_rn(fmaf(p, w, 2.83297682f), x);
}

// MLTSampler (PSSMLT.fs:36-150); primary samples at X[dim * stride + chain]
struct MltSampler {
  uint32_t inner;
  bool large_step;
  int last_large;
  int cur_iter;
  int index;
  int initialized;
  float p_large;
  int kelemen;
  float sigma, eps_min, eps_max;
  float4* X;
  long long stride;
  int max_dims;

  __device__ __forceinline__ void start_iteration() {
    large_step = cur_iter == 0 || lcg_next(inner) < p_large;
    cur_iter += 1;
    index = 0;
  }
  __device__ __forceinline__ float next() {
    const int i = index++;
    float4* xp = X + static_cast<long long>(min(i, max_dims - 1)) * stride;
    float4 x;
    if (initialized <= i) {
      x = make_float4(0.f, 0.f, __int_as_float(0), __int_as_float(0));
      initialized = i + 1;
    } else {
      x = *xp;
    }
    int last_mod = __float_as_int(x.z);
    if (last_mod < last_large) {
      x.x = lcg_next(inner);
      last_mod = last_large;
    }
    x.y = x.x;                       // BackUp
    x.w = __int_as_float(last_mod);
    float v;
    if (large_step) {
      v = lcg_next(inner);
    } else if (kelemen) {
      v = x.x;
      const float a = logf(__fdiv_rn(eps_max, eps_min));
      for (int k = last_mod; k < cur_iter; ++k) {
        const float u1 = __fsub_rn(lcg_next(inner), 0.5f);
        const float u2 = u1 < 0.f ? __fadd_rn(1.f, __fmul_rn(2.f, u1)) : __fmul_rn(2.f, u1);
        v = __fadd_rn(v, copysignf(__fmul_rn(eps_max, expf(__fmul_rn(-a, u2))), u1));
      }
    } else {
      const float normal = __fmul_rn(sqrtf(2.f), erfinv_giles(fmaf(2.f, lcg_next(inner), -1.f)));
      const float eff = __fmul_rn(sigma, sqrtf(static_cast<float>(cur_iter - last_mod)));
      v = fmaf(normal, eff, x.x);
    }
    v = __fsub_rn(v, floorf(v));
    x.x = v;
    x.z = __int_as_float(cur_iter);
    if (i < max_dims) *xp = x;
    return v;
  }
  __device__ __forceinline__ void reject() {
    for (int i = 0; i < min(initialized, max_dims); ++i) {
      float4* xp = X + static_cast<long long>(i) * stride;
      float4 x = *xp;
      x.x = x.y;
      x.z = x.w;
      *xp = x;
    }
    cur_iter -= 1;
  }
  __device__ __forceinline__ void accept() {
    if (large_step) last_large = cur_iter;
  }
};

__device__ __forceinline__ float luminance(V3 L) {
  return __fadd_rn(__fadd_rn(__fmul_rn(L.x, 0.2126f), __fmul_rn(L.y, 0.7152f)), __fmul_rn(L.z, 0.0722f));
}

// uPixel = Next2D * (W, H); pixel = min(W-1, int(u)); the pixel offset is u - pixel
template <class Smp>
__device__ __forceinline__ Ray mlt_camera(const DevView& v, Smp& smp, int* px, int* py) {
  const float ux = __fmul_rn(smp.next(), static_cast<float>(v.width));
  const float uy = __fmul_rn(smp.next(), static_cast<float>(v.height));
  const int x = min(v.width - 1, static_cast<int>(ux)), y = min(v.height - 1, static_cast<int>(uy));
  const float fx = __fsub_rn(ux, static_cast<float>(x)), fy = __fsub_rn(uy, static_cast<float>(y));
  const float lx = smp.next(), ly = smp.next();
  *px = x;
  *py = y;
  return camera_ray(v, x, y, fx, fy, lx, ly);
}

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

struct Splat {
  int pix;  // -1 = none
  V3 c;
};

// warp-aggregated splat: lanes with the same pixel add their colours, one atomic per pixel
__device__ __forceinline__ void warp_splat(float* film, Splat s) {
  const unsigned active = __activemask();
  const unsigned peers = __match_any_sync(active, s.pix);
  if (s.pix < 0) return;
  const int lane = threadIdx.x & 31;
  const int leader = __ffs(peers) - 1;
  float r = 0.f, g = 0.f, b = 0.f;
  // sum over the peer group in lane order (each lane reads every peer's value)
  for (unsigned m = peers; m; m &= m - 1) {
    const int src = __ffs(m) - 1;
    r += __shfl_sync(peers, s.c.x, src);
    g += __shfl_sync(peers, s.c.y, src);
    b += __shfl_sync(peers, s.c.z, src);
  }
  if (lane == leader) {
    atomicAdd(film + 3LL * s.pix, r);
    atomicAdd(film + 3LL * s.pix + 1, g);
    atomicAdd(film + 3LL * s.pix + 2, b);
  }
}

template <bool kWT, int kWalk>
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
    m.kelemen = p.kelemen;
    m.sigma = p.sigma;
    m.eps_min = p.eps_min;
    m.eps_max = p.eps_max;
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
    k_mlt_chains<decltype(wt)::value, decltype(walk)::value><<<grid, 128, 0, st>>>(p);
  });
  return cudaGetLastError();
}

}  // namespace bn
