// bn_forward / bn_backward: differentiable material slots over the uploaded scene.
#include <string>
#include <vector>

#include "../device/adjoint.hpp"
#include "context.hpp"

namespace {

int prepare(bn_context* ctx, const bn_adjoint_desc* d, const float* params, const float* sparams, bn::AdjParams* p) {
  if (!ctx->has_scene) return ctx->fail(BN_ERR_NO_SCENE, "adjoint before bn_scene_upload");
  if (!d || !params) return ctx->fail(BN_ERR_INVALID_ARG, "adjoint: null descriptor or parameters");
  if (d->n_slots <= 0 || d->emissive_slot_base < 0 || d->emissive_slot_base > d->n_slots)
    return ctx->fail(BN_ERR_INVALID_ARG, "adjoint: bad slot counts");
  if (d->width <= 0 || d->height <= 0 || d->spp <= 0 || d->max_depth < 0 || d->rr_depth < 0)
    return ctx->fail(BN_ERR_INVALID_ARG, "adjoint: bad film, spp or depth");
  if (d->emissive_slot_base > ctx->scene.n_mats)
    return ctx->fail(BN_ERR_INVALID_ARG, "adjoint: material slots beyond the scene's materials");
  cudaError_t e;
  const size_t np = static_cast<size_t>(d->n_slots) * bn::kSlotParams;
  const long long pixels = static_cast<long long>(d->width) * d->height;
  if ((e = ctx->adj_params.reserve(2 * np * sizeof(float))) != cudaSuccess) return ctx->cuda_fail(e, "adjoint params");
  if ((e = ctx->adj_aux.reserve(static_cast<size_t>(pixels) * d->spp * sizeof(float4))) != cudaSuccess)
    return ctx->cuda_fail(e, "adjoint path radiance");
  if ((e = ctx->adj_image.reserve(static_cast<size_t>(pixels) * 3 * sizeof(float))) != cudaSuccess)
    return ctx->cuda_fail(e, "adjoint image");
  if ((e = ctx->views.reserve(sizeof(bn::DevView))) != cudaSuccess) return ctx->cuda_fail(e, "adjoint view");
  bn_view v{};
  v.camera = d->camera;
  v.width = d->width;
  v.height = d->height;
  const bn::DevView dv = bnc::make_dev_view(v, 0, 0);
  float* dparams = ctx->adj_params.as<float>();
  float* dsparams = dparams + np;
  cudaStream_t st = ctx->stream;
  cudaMemcpyAsync(ctx->views.ptr, &dv, sizeof(dv), cudaMemcpyHostToDevice, st);
  cudaMemcpyAsync(dparams, params, np * sizeof(float), cudaMemcpyHostToDevice, st);
  const float* sp = (d->freeze_sampling && sparams) ? sparams : params;
  cudaMemcpyAsync(dsparams, sp, np * sizeof(float), cudaMemcpyHostToDevice, st);
  *p = bn::AdjParams{};
  p->scene = ctx->scene;
  p->view = ctx->views.as<bn::DevView>();
  p->n_slots = d->n_slots;
  p->emissive_base = d->emissive_slot_base;
  p->spp = d->spp;
  p->max_depth = d->max_depth;
  p->rr_depth = d->rr_depth;
  p->frame_id = d->frame_id;
  p->params = dparams;
  p->sparams = dsparams;
  p->path_L = ctx->adj_aux.as<float4>();
  p->image = ctx->adj_image.as<float>();
  p->n_pixels = pixels;
  return BN_OK;
}

}  // namespace

extern "C" int bn_forward(bn_context* ctx, const bn_adjoint_desc* d, const float* params, const float* sampling_params,
                          float* out_image) {
  if (!ctx) return BN_ERR_INVALID_ARG;
  cudaSetDevice(ctx->device);
  bn::AdjParams p;
  int rc = prepare(ctx, d, params, sampling_params, &p);
  if (rc) return rc;
  cudaError_t e;
  cudaEventRecord(ctx->ev0, ctx->stream);
  if ((e = bn::launch_adj_forward(p, ctx->stream)) != cudaSuccess) return ctx->cuda_fail(e, "forward launch");
  cudaEventRecord(ctx->ev1, ctx->stream);
  if ((e = bn::launch_adj_image(p, ctx->stream)) != cudaSuccess) return ctx->cuda_fail(e, "image launch");
  cudaEventRecord(ctx->ev2, ctx->stream);
  if (out_image)
    cudaMemcpyAsync(out_image, p.image, static_cast<size_t>(p.n_pixels) * 3 * sizeof(float), cudaMemcpyDeviceToHost,
                    ctx->stream);
  if ((e = cudaStreamSynchronize(ctx->stream)) != cudaSuccess) return ctx->cuda_fail(e, "forward");
  float ms_main = 0.f, ms_all = 0.f;
  cudaEventElapsedTime(&ms_main, ctx->ev0, ctx->ev1);
  cudaEventElapsedTime(&ms_all, ctx->ev0, ctx->ev2);
  ctx->stats.last_dominant_ms = ms_main;
  ctx->stats.last_kernel_ms = ms_all;
  ctx->stats.last_launches = 2;
  ctx->stats.paths += static_cast<uint64_t>(p.n_pixels) * p.spp;
  return bnc::check_device_error(ctx);
}

extern "C" int bn_backward(bn_context* ctx, const bn_adjoint_desc* d, const float* params, const float* sampling_params,
                           const float* target_image, double* d_params, double* loss) {
  if (!ctx) return BN_ERR_INVALID_ARG;
  if (!target_image || !d_params) return ctx->fail(BN_ERR_INVALID_ARG, "bn_backward: null target or gradient");
  cudaSetDevice(ctx->device);
  bn::AdjParams p;
  int rc = prepare(ctx, d, params, sampling_params, &p);
  if (rc) return rc;
  cudaError_t e;
  const size_t np = static_cast<size_t>(d->n_slots) * bn::kSlotParams;
  if ((e = ctx->adj_target.reserve(static_cast<size_t>(p.n_pixels) * 3 * sizeof(float))) != cudaSuccess)
    return ctx->cuda_fail(e, "adjoint target");
  if ((e = ctx->adj_grad.reserve((np + 1) * sizeof(double))) != cudaSuccess) return ctx->cuda_fail(e, "adjoint gradient");
  cudaStream_t st = ctx->stream;
  cudaMemcpyAsync(ctx->adj_target.ptr, target_image, static_cast<size_t>(p.n_pixels) * 3 * sizeof(float),
                  cudaMemcpyHostToDevice, st);
  cudaMemsetAsync(ctx->adj_grad.ptr, 0, (np + 1) * sizeof(double), st);
  p.target = ctx->adj_target.as<float>();
  p.grad = ctx->adj_grad.as<double>();
  p.loss = p.grad + np;
  cudaEventRecord(ctx->ev0, st);
  if ((e = bn::launch_adj_forward(p, st)) != cudaSuccess) return ctx->cuda_fail(e, "adjoint forward launch");
  if ((e = bn::launch_adj_image(p, st)) != cudaSuccess) return ctx->cuda_fail(e, "adjoint image launch");
  if ((e = bn::launch_adj_loss(p, st)) != cudaSuccess) return ctx->cuda_fail(e, "loss launch");
  cudaEventRecord(ctx->ev1, st);
  if ((e = bn::launch_adj_backward(p, st)) != cudaSuccess) return ctx->cuda_fail(e, "backward launch");
  cudaEventRecord(ctx->ev2, st);
  std::vector<double> host(np + 1);
  cudaMemcpyAsync(host.data(), ctx->adj_grad.ptr, (np + 1) * sizeof(double), cudaMemcpyDeviceToHost, st);
  if ((e = cudaStreamSynchronize(st)) != cudaSuccess) return ctx->cuda_fail(e, "backward");
  for (size_t i = 0; i < np; ++i) d_params[i] = host[i];
  if (loss) *loss = host[np];
  float ms_replay = 0.f, ms_all = 0.f;
  cudaEventElapsedTime(&ms_replay, ctx->ev1, ctx->ev2);
  cudaEventElapsedTime(&ms_all, ctx->ev0, ctx->ev2);
  ctx->stats.last_dominant_ms = ms_replay;
  ctx->stats.last_kernel_ms = ms_all;
  ctx->stats.last_launches = 4;
  return bnc::check_device_error(ctx);
}
