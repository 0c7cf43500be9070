// The plain megakernel with the Normal and Direct integrators (NormalIntegrator.Li,
// Extensions/Integrator/Normal.fs:10-17; DirectIntegrator.Li, Direct.fs:10-40), in their own
// translation unit so they compile in parallel with the path tracer.
#include "dev_mega.cuh"

namespace bn {

cudaError_t launch_megakernel_simple(const DevScene& s, const MegaParams& p, cudaStream_t st) {
  if (p.n_items <= 0) return cudaSuccess;
  const int bs = 128;
  const long long grid = (p.n_items + bs - 1) / bs;
  dispatch_walk<true>(s, p.watertight, p.count, [&](auto wt, auto walk) {
    constexpr bool kWT = decltype(wt)::value;
    constexpr int kWalk = decltype(walk)::value;
    if (p.integrator == BN_INTEGRATOR_NORMAL) k_pt_mega<kWT, kWalk, BN_INTEGRATOR_NORMAL><<<grid, bs, 0, st>>>(s, p);
    else k_pt_mega<kWT, kWalk, BN_INTEGRATOR_DIRECT><<<grid, bs, 0, st>>>(s, p);
  });
  return cudaGetLastError();
}

}  // namespace bn
