// The plain path-tracing megakernel with shadow-ray culling (BN_RENDER_CULL_SHADOW): each light
// sample is evaluated first and its shadow ray traced only when it can change the radiance
// (shadow_contributes), the test the wavefront applies to every light sample.  Same images as the
// reference-order megakernel; it is the fair plain-form baseline for the wavefront's ray counts.
#include "dev_mega.cuh"

namespace bn {

cudaError_t launch_megakernel_cull(const DevScene& s, const MegaParams& p, cudaStream_t st) {
  if (p.n_items <= 0) return cudaSuccess;
  const int bs = 128;
  const long long grid = (p.n_items + bs - 1) / bs;
  if (p.simple && !s.wide) {
    if (p.watertight) k_pt_mega<true, kWalkBinary, BN_INTEGRATOR_PATH, true, true><<<grid, bs, 0, st>>>(s, p);
    else k_pt_mega<false, kWalkBinary, BN_INTEGRATOR_PATH, true, true><<<grid, bs, 0, st>>>(s, p);
    return cudaGetLastError();
  }
  dispatch_walk<false>(s, p.watertight, false, [&](auto wt, auto walk) {
    k_pt_mega<decltype(wt)::value, decltype(walk)::value, BN_INTEGRATOR_PATH, false, true><<<grid, bs, 0, st>>>(s, p);
  });
  return cudaGetLastError();
}

}  // namespace bn
