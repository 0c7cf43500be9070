// PSSMLT launch parameters (Extensions/Integrator/PSSMLT.fs:153-414).
#pragma once
#include <cuda_runtime.h>

#include "dev_types.cuh"

namespace bn {

struct MltParams {
  DevScene scene;
  const DevView* view;          // one film (the reference renders one camera)
  int n_bootstrap, n_chains;
  int max_depth, rr_depth, frame_id;
  int n_dims;                   // 4 + 7 * max_depth primary samples per chain (PSSMLT.fs:387)
  int mutations_per_chain;      // ceil(spp * W * H / n_chains) (:314-320)
  int kelemen;                  // 1 Kelemen(eps_min, eps_max), 0 Gaussian(sigma)
  float large_step_prob, sigma, eps_min, eps_max;
  float b;                      // mean bootstrap luminance (:394)
  float inv_eff_spp;            // 1 / (mutations * chains / pixels) (:322-326)
  bool watertight;
  float* weights;               // n_bootstrap luminances
  const float* alias_prob;      // proportional start table, or null: uniform as the reference
  const int* alias_idx;
  float4* X;                    // n_dims x n_chains primary samples
  float* film;                  // W * H * 3
  unsigned long long* accepted;
};

cudaError_t launch_mlt_bootstrap(const MltParams& p, cudaStream_t st);
cudaError_t launch_mlt_chains(const MltParams& p, cudaStream_t st);

}  // namespace bn
