// The plain megakernel, one template per integrator (k_megakernel.cu instantiates the path
// tracer, k_integrators.cu the Normal and Direct integrators): ProgressiveIntegrator.RenderTile
// (Base/Integrator.fs:22-44), one thread per (view, pixel, sample chunk).
//
// Work item -> (view, chunk, pixel): items of one view are chunk-major, pixels row-major inside a
// chunk, so a warp holds 32 neighbouring pixels of one sample range (coherent primary rays,
// coalesced partial-sum stores).  Each thread runs samples [chunk*spc, (chunk+1)*spc) with the
// reference seeds Sampler(x, y, frame*spp + s) and accumulates fma(1/spp, L, acc) in sample
// order; the reduction then adds the chunks in chunk order in double precision, so the film is
// deterministic run to run.
//
// kCull (BN_RENDER_CULL_SHADOW): the light sample is evaluated before its shadow ray and the ray
// is traced only if it can change the radiance, as the wavefront does; the image is the same.
#pragma once
#include "dev_shading.cuh"
#include "launch.hpp"

namespace bn {
namespace {

__device__ __forceinline__ int find_view(const long long* __restrict__ offsets, int n_views, long long item) {
  int v = 0;
  while (v + 1 < n_views && __ldg(&offsets[v + 1]) <= item) ++v;
  return v;
}

template <bool kWT, int kWalk, int kInteg, bool kSimple = false, bool kCull = false>
__global__ void __launch_bounds__(128) k_pt_mega(DevScene s, MegaParams p) {
  constexpr bool kCount = kWalk == kWalkCount;
  // scenes walked binary are small and shading-bound: one out-of-line walk keeps the kernel in
  // the instruction cache (+9% on the Cornell box); large scenes keep inlined walks (the
  // out-of-line walk costs 7% on the 1,024-instance scene)
  constexpr bool kOutline = kWalk != kWalkWide;
  const long long item = static_cast<long long>(blockIdx.x) * blockDim.x + threadIdx.x;
  PathCounters pc{};
  unsigned long long paths = 0;
  if (item < p.n_items) {
    const int vi = find_view(p.item_offsets, p.n_views, item);
    const DevView& v = p.views[vi];
    const long long local = item - __ldg(&p.item_offsets[vi]);
    const long long npix = static_cast<long long>(v.width) * v.height;
    const int chunk = static_cast<int>(local / npix);
    const long long pix = local - chunk * npix;
    const int x = static_cast<int>(pix % v.width), y = static_cast<int>(pix / v.width);
    const float inv_spp = __frcp_rn(static_cast<float>(p.spp));
    V3 acc = mk(0.f, 0.f, 0.f);
    const int s0 = chunk * p.spc, s1 = min(p.spp, s0 + p.spc);
    for (int sid = s0; sid < s1; ++sid) {
      IndepSampler smp{xxhash32_three(static_cast<uint32_t>(x), static_cast<uint32_t>(y),
                                      static_cast<uint32_t>(p.frame_id * p.spp + sid))};
      const float upx = smp.next(), upy = smp.next();
      const float ulx = smp.next(), uly = smp.next();
      const Ray ray = camera_ray<kSimple>(v, x, y, upx, upy, ulx, uly);
      V3 L;
      if (kInteg == BN_INTEGRATOR_NORMAL) L = li_normal<kWT, kWalk, kOutline>(s, ray, &pc);
      else if (kInteg == BN_INTEGRATOR_DIRECT) L = li_direct<kWT, kWalk, IndepSampler, kOutline>(s, ray, smp, &pc);
      else L = li_path<kWT, false, kWalk, IndepSampler, kOutline, kSimple, kCull>(s, ray, smp, p.max_depth, p.rr_depth, &pc);
      acc = fma3(mk(inv_spp, inv_spp, inv_spp), L, acc);
      ++paths;
    }
    p.partial[item] = make_float4(acc.x, acc.y, acc.z, 0.f);
  }
  if (kCount) {
    unsigned long long r = pc.rays, nn = pc.tc.nodes, tt = pc.tc.tris, ii = pc.tc.insts, pp = paths;
    for (int o = 16; o > 0; o >>= 1) {
      r += __shfl_down_sync(0xffffffffu, r, o);
      nn += __shfl_down_sync(0xffffffffu, nn, o);
      tt += __shfl_down_sync(0xffffffffu, tt, o);
      ii += __shfl_down_sync(0xffffffffu, ii, o);
      pp += __shfl_down_sync(0xffffffffu, pp, o);
    }
    if ((threadIdx.x & 31) == 0) {
      atomicAdd(&p.counters->rays, r);
      atomicAdd(&p.counters->nodes, nn);
      atomicAdd(&p.counters->tris, tt);
      atomicAdd(&p.counters->insts, ii);
      atomicAdd(&p.counters->paths, pp);
    }
  }
}

}  // namespace
}  // namespace bn
