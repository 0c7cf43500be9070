// Differentiable-material render (forward) and path-replay adjoint (backward) parameters.
#pragma once
#include <cuda_runtime.h>

#include "dev_types.cuh"

namespace bn {

constexpr int kSlotParams = 6;  // albedo r, g, b, roughness, metallic, emission scale

struct AdjParams {
  DevScene scene;
  const DevView* view;
  int n_slots, emissive_base;
  int spp, max_depth, rr_depth, frame_id;
  const float* params;        // values: n_slots * 6
  const float* sparams;       // sampling decisions: n_slots * 6 (== params unless frozen)
  float4* path_L;             // per (sample, pixel): radiance of the path
  float* image;               // W*H*3, Film.Pixels order
  const float* target;        // W*H*3
  double* grad;               // n_slots * 6
  double* loss;               // 1
  long long n_pixels;
};

cudaError_t launch_adj_forward(const AdjParams& p, cudaStream_t st);
cudaError_t launch_adj_image(const AdjParams& p, cudaStream_t st);
cudaError_t launch_adj_loss(const AdjParams& p, cudaStream_t st);
cudaError_t launch_adj_backward(const AdjParams& p, cudaStream_t st);

}  // namespace bn
