// Film output on the device: Film.PostProcess (Base/Film.fs:21-30) and the 8-bit packing that
// Film.Save (:55-66) gets from ImageSharp 3.1.6's Rgba32(Vector3) constructor.
#include <cstdint>

#include "dev_geometry.cuh"
#include "launch.hpp"

namespace bn {
namespace {

// Vector3.Clamp(x, 0, 1) = Min(Max(x, 0), 1); Math.Max/Min semantics keep a NaN
__device__ __forceinline__ float clamp01(float x) { return x != x ? x : fminf(fmaxf(x, 0.f), 1.f); }

// Rgba32.Pack: v * 255 + 0.5, clamped to [0, 255], converted by truncation (a NaN converts to 0)
__device__ __forceinline__ unsigned pack8(float v) {
  const float w = __fadd_rn(__fmul_rn(v, 255.f), 0.5f);
  if (w != w) return 0u;
  return static_cast<unsigned>(fminf(fmaxf(w, 0.f), 255.f));
}

__device__ __forceinline__ float post(float x, int tm) {
  if (tm == BN_TONE_ACES) {
    // x * (2.51 x + 0.03) / (x * (2.43 x + 0.59) + 0.14), per component in this order
    const float num = __fmul_rn(x, __fadd_rn(__fmul_rn(2.51f, x), 0.03f));
    const float den = __fadd_rn(__fmul_rn(x, __fadd_rn(__fmul_rn(2.43f, x), 0.59f)), 0.14f);
    x = __fdiv_rn(num, den);
  } else if (tm == BN_TONE_GAMMA) {
    x = powf(x, 1.f / 2.2f);  // MathF.Pow(x, 1f / 2.2f)
  }
  return clamp01(x);
}

__global__ void k_film_tonemap(const float* __restrict__ film, long long n, int tm, uchar4* __restrict__ out) {
  for (long long i = static_cast<long long>(blockIdx.x) * blockDim.x + threadIdx.x; i < n;
       i += static_cast<long long>(gridDim.x) * blockDim.x) {
    const float r = post(film[3 * i], tm), g = post(film[3 * i + 1], tm), b = post(film[3 * i + 2], tm);
    out[i] = make_uchar4(static_cast<unsigned char>(pack8(r)), static_cast<unsigned char>(pack8(g)),
                         static_cast<unsigned char>(pack8(b)), 255);
  }
}

}  // namespace

cudaError_t launch_film_tonemap(const float* film, long long n_pixels, int tone_mapping, void* rgba, cudaStream_t st) {
  if (n_pixels <= 0) return cudaSuccess;
  const long long blocks = (n_pixels + 255) / 256;
  k_film_tonemap<<<static_cast<unsigned>(blocks < 152 * 16 ? blocks : 152 * 16), 256, 0, st>>>(
      film, n_pixels, tone_mapping, static_cast<uchar4*>(rgba));
  return cudaGetLastError();
}

}  // namespace bn
