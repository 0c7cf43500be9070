// The plain path-tracing megakernel: ProgressiveIntegrator.RenderTile (Base/Integrator.fs:22-44)
// with PathTracingIntegrator.Li, one thread per (view, pixel, sample chunk).
//
// Work item -> (view, chunk, pixel): items of one view are chunk-major, pixels row-major inside a
// chunk, so a warp holds 32 neighbouring pixels of one sample range (coherent primary rays,
// coalesced partial-sum stores).  Each thread runs samples [chunk*spc, (chunk+1)*spc) with the
// reference seeds Sampler(x, y, frame*spp + s) and accumulates fma(1/spp, L, acc) in sample
// order; the reduction then adds the chunks in chunk order in double precision, so the film is
// deterministic run to run.
#include "dev_shading.cuh"
#include "launch.hpp"

namespace bn {
namespace {

__device__ __forceinline__ int find_view(const long long* __restrict__ offsets, int n_views, long long item) {
  int v = 0;
  while (v + 1 < n_views && __ldg(&offsets[v + 1]) <= item) ++v;
  return v;
}

template <bool kWT, int kWalk>
__global__ void __launch_bounds__(128) k_pt_mega(DevScene s, MegaParams p) {
  constexpr bool kCount = kWalk == kWalkCount;
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
      const Ray ray = camera_ray(v, x, y, upx, upy, ulx, uly);
      // scenes walked binary are small and shading-bound: one out-of-line walk keeps the kernel
      // in the instruction cache (+9% on the Cornell box); large scenes keep inlined walks
      // (the out-of-line walk costs 7% on the 1,024-instance scene)
      const V3 L = li_path<kWT, false, kWalk, IndepSampler, kWalk != kWalkWide>(s, ray, smp, p.max_depth, p.rr_depth, &pc);
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

// one thread per pixel: sum the chunk partials in order, store at the flipped row (Film.fs:41-46)
__global__ void k_mega_reduce(MegaParams p) {
  const long long gp = static_cast<long long>(blockIdx.x) * blockDim.x + threadIdx.x;
  if (gp >= p.n_pixels) return;
  int vi = 0;
  while (vi + 1 < p.n_views && p.views[vi + 1].pixel_offset <= gp) ++vi;
  const DevView& v = p.views[vi];
  const long long pix = gp - v.pixel_offset;
  const long long npix = static_cast<long long>(v.width) * v.height;
  const int x = static_cast<int>(pix % v.width), y = static_cast<int>(pix / v.width);
  const long long base = __ldg(&p.item_offsets[vi]) + pix;
  double r = 0.0, g = 0.0, b = 0.0;
  for (int c = 0; c < p.chunks; ++c) {
    const float4 q = p.partial[base + c * npix];
    r += q.x; g += q.y; b += q.z;
  }
  const long long out = v.pixel_offset + static_cast<long long>(v.height - y - 1) * v.width + x;
  p.film[3 * out] = static_cast<float>(r);
  p.film[3 * out + 1] = static_cast<float>(g);
  p.film[3 * out + 2] = static_cast<float>(b);
}

}  // namespace

cudaError_t launch_megakernel(const DevScene& s, const MegaParams& p, cudaStream_t st) {
  if (p.n_items <= 0) return cudaSuccess;
  const int bs = 128;
  const long long grid = (p.n_items + bs - 1) / bs;
  dispatch_walk<true>(s, p.watertight, p.count, [&](auto wt, auto walk) {
    k_pt_mega<decltype(wt)::value, decltype(walk)::value><<<grid, bs, 0, st>>>(s, p);
  });
  return cudaGetLastError();
}

cudaError_t launch_mega_reduce(const MegaParams& p, cudaStream_t st) {
  if (p.n_pixels <= 0) return cudaSuccess;
  k_mega_reduce<<<(p.n_pixels + 255) / 256, 256, 0, st>>>(p);
  return cudaGetLastError();
}

}  // namespace bn
