// The PSSMLT sampler and splats shared by the lockstep chain kernel (k_pssmlt.cu) and the
// wavefront chains (k_mlt_wavefront.cu): MLTSampler (Extensions/Integrator/PSSMLT.fs:36-150) over
// primary samples at X[dim * stride] (float4: value, backup, last modification, its backup),
// the luminance and camera draws of PSSMLTIntegrator, and warp-aggregated film splats.
#pragma once
#include "dev_shading.cuh"

namespace bn {

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
  float log_eps;  // logf(eps_max / eps_min), set with them: Kelemen's exponent scale, once per chain
  float4* X;
  long long stride;
  int max_dims;

  __device__ __forceinline__ void start_iteration() {
    large_step = cur_iter == 0 || lcg_next(inner) < p_large;
    cur_iter += 1;
    index = 0;
  }
  // the draw of dimension i from its primary sample x (zeroes for a dimension drawn for the
  // first time): EnsureReady (PSSMLT.fs:98-134), the record written back
  __device__ __forceinline__ float draw(int i, float4 x) {
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
      const float a = log_eps;
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
    if (i < max_dims) X[static_cast<long long>(i) * stride] = x;
    return v;
  }
  __device__ __forceinline__ float next() {
    const int i = index++;
    float4 x = make_float4(0.f, 0.f, __int_as_float(0), __int_as_float(0));
    if (initialized <= i) initialized = i + 1;
    else x = X[static_cast<long long>(min(i, max_dims - 1)) * stride];
    return draw(i, x);
  }
  // the next N draws (Next1D N times), their primary samples loaded together first: one memory
  // round trip instead of N dependent ones, the same values in the same order
  template <int N>
  __device__ __forceinline__ void next_n(float* u) {
    const int i0 = index, init0 = initialized;
    if (i0 + N > max_dims) {  // past the vector's end: one at a time, as Next1D
#pragma unroll
      for (int k = 0; k < N; ++k) u[k] = next();
      return;
    }
    float4 x[N];
#pragma unroll
    for (int k = 0; k < N; ++k)
      x[k] = i0 + k < init0 ? X[static_cast<long long>(i0 + k) * stride]
                            : make_float4(0.f, 0.f, __int_as_float(0), __int_as_float(0));
#pragma unroll
    for (int k = 0; k < N; ++k) {
      const int i = index++;
      if (initialized <= i) initialized = i + 1;
      u[k] = draw(i, x[k]);
    }
  }
  // Reject restores every initialised dimension.  The records are read eight at a time before any
  // is written back: the stride is a runtime value, so record by record each load would wait for
  // the store before it, one memory round trip per dimension.
  __device__ __forceinline__ void reject() {
    const int n = min(initialized, max_dims);
    int i = 0;
    for (; i + 8 <= n; i += 8) {
      float4 x[8];
#pragma unroll
      for (int k = 0; k < 8; ++k) x[k] = X[static_cast<long long>(i + k) * stride];
#pragma unroll
      for (int k = 0; k < 8; ++k) {
        x[k].x = x[k].y;
        x[k].z = x[k].w;
        X[static_cast<long long>(i + k) * stride] = x[k];
      }
    }
    for (; i < n; ++i) {
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
  // the scalar state between the kernels of the wavefront chains: (inner sampler, current
  // iteration, last large step, sample index | initialised count << 12 | large step << 24)
  __device__ __forceinline__ int4 pack() const {
    return make_int4(static_cast<int>(inner), cur_iter, last_large,
                     index | (initialized << 12) | (large_step ? 1 << 24 : 0));
  }
  __device__ __forceinline__ void unpack(int4 q) {
    inner = static_cast<uint32_t>(q.x);
    cur_iter = q.y;
    last_large = q.z;
    index = q.w & 0xfff;
    initialized = (q.w >> 12) & 0xfff;
    large_step = (q.w >> 24) & 1;
  }
};

__device__ __forceinline__ float luminance(V3 L) {
  return __fadd_rn(__fadd_rn(__fmul_rn(L.x, 0.2126f), __fmul_rn(L.y, 0.7152f)), __fmul_rn(L.z, 0.0722f));
}

// uPixel = Next2D * (W, H); pixel = min(W-1, int(u)); the pixel offset is u - pixel
template <class Smp>
__device__ __forceinline__ Ray mlt_camera(const DevView& v, Smp& smp, int* px, int* py) {
  float u[4];
  smp.template next_n<4>(u);
  const float ux = __fmul_rn(u[0], static_cast<float>(v.width));
  const float uy = __fmul_rn(u[1], static_cast<float>(v.height));
  const int x = min(v.width - 1, static_cast<int>(ux)), y = min(v.height - 1, static_cast<int>(uy));
  const float fx = __fsub_rn(ux, static_cast<float>(x)), fy = __fsub_rn(uy, static_cast<float>(y));
  const float lx = u[2], ly = u[3];
  *px = x;
  *py = y;
  return camera_ray(v, x, y, fx, fy, lx, ly);
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

}  // namespace bn
