// The plain path-tracing megakernel (PathTracingIntegrator.Li, the kernel template is in
// dev_mega.cuh) and the chunk reduction shared by every integrator.
#include "dev_mega.cuh"

namespace bn {
namespace {

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
  if (p.integrator == BN_INTEGRATOR_NORMAL || p.integrator == BN_INTEGRATOR_DIRECT)
    return launch_megakernel_simple(s, p, st);
  if (p.cull && !p.count) return launch_megakernel_cull(s, p, st);
  if (p.simple && !p.count && !s.wide) {
    // Lambertian meshes, uniform lights, pinhole views: the specialised path loop
    if (p.watertight) k_pt_mega<true, kWalkBinary, BN_INTEGRATOR_PATH, true><<<grid, bs, 0, st>>>(s, p);
    else k_pt_mega<false, kWalkBinary, BN_INTEGRATOR_PATH, true><<<grid, bs, 0, st>>>(s, p);
    return cudaGetLastError();
  }
  dispatch_walk<true>(s, p.watertight, p.count, [&](auto wt, auto walk) {
    k_pt_mega<decltype(wt)::value, decltype(walk)::value, BN_INTEGRATOR_PATH><<<grid, bs, 0, st>>>(s, p);
  });
  return cudaGetLastError();
}

cudaError_t launch_mega_reduce(const MegaParams& p, cudaStream_t st) {
  if (p.n_pixels <= 0) return cudaSuccess;
  k_mega_reduce<<<(p.n_pixels + 255) / 256, 256, 0, st>>>(p);
  return cudaGetLastError();
}

}  // namespace bn
