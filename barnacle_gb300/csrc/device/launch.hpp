// Host-side launchers of the device kernels (one translation unit per kernel family).
#pragma once
#include <cuda_runtime.h>

#include <type_traits>

#include "../../../include/barnacle_gpu.h"
#include "dev_types.cuh"

namespace bn {

// Compile-time walk and triangle test of a launch: f(std::integral_constant<bool, watertight>,
// std::integral_constant<int, walk>) with walk one of kWalkBinary / kWalkCount / kWalkWide
// (dev_traverse.cuh).  A counting launch walks the binary tree; otherwise the scene's choice.
template <bool kWithCount, class F>
void dispatch_walk(const DevScene& s, bool watertight, bool count, F&& f) {
  using WT = std::integral_constant<bool, true>;
  using MT = std::integral_constant<bool, false>;
  using Bin = std::integral_constant<int, 0>;
  using Cnt = std::integral_constant<int, 1>;
  using Wide = std::integral_constant<int, 2>;
  const int walk = (kWithCount && count) ? 1 : (s.wide ? 2 : 0);
  if (walk == 1) {
    if constexpr (kWithCount) {
      if (watertight) f(WT{}, Cnt{});
      else f(MT{}, Cnt{});
    }
  } else if (walk == 2) {
    if (watertight) f(WT{}, Wide{});
    else f(MT{}, Wide{});
  } else {
    if (watertight) f(WT{}, Bin{});
    else f(MT{}, Bin{});
  }
}

// per-launch counters written by kernels that count (BN_TRACE_COUNT, stats renders)
struct DevCounters {
  unsigned long long rays, nodes, tris, insts, paths, accepted, proposed, pad;
};

cudaError_t launch_trace(const DevScene& s, const bn_ray* rays, bn_hit* hits, long long n, unsigned flags,
                         DevCounters* counters, cudaStream_t st);
cudaError_t launch_bsdf(const DevScene& s, const bn_bsdf_query* q, bn_bsdf_result* out, long long n, bool sample,
                        cudaStream_t st);
cudaError_t launch_sampler_stream(const uint32_t* seeds, long long n_streams, int n_draws, float* out, cudaStream_t st);

// Plain megakernel: one thread per (view, pixel, sample chunk); partial sums per chunk, then a
// reduction in chunk order into the FP32 film (rows flipped as Film.SetPixel does).
struct MegaParams {
  const DevView* views;
  int n_views;
  long long n_items;         // sum over views of pixels * chunks
  const long long* item_offsets;  // per view: first item (device)
  int spp, chunks, spc;      // samples per pixel, chunks per pixel, samples per chunk
  int max_depth, rr_depth, frame_id;
  int integrator;            // bn_integrator_type: PATH, NORMAL or DIRECT
  bool simple;               // Lambertian meshes, uniform light sampler, pinhole views only
  bool watertight;
  bool count;
  bool cull;                 // trace a light sample's shadow ray only if it can change L
  float4* partial;           // n_items partial sums (scratch)
  float* film;               // concatenated views, 3 floats per pixel
  long long n_pixels;
  DevCounters* counters;
};
cudaError_t launch_megakernel(const DevScene& s, const MegaParams& p, cudaStream_t st);
cudaError_t launch_megakernel_simple(const DevScene& s, const MegaParams& p, cudaStream_t st);  // NORMAL, DIRECT
cudaError_t launch_megakernel_cull(const DevScene& s, const MegaParams& p, cudaStream_t st);    // PATH + cull
cudaError_t launch_mega_reduce(const MegaParams& p, cudaStream_t st);

// Film.PostProcess + Rgba32 packing over n_pixels RGB floats into 4-byte RGBA
cudaError_t launch_film_tonemap(const float* film, long long n_pixels, int tone_mapping, void* rgba, cudaStream_t st);

}  // namespace bn
