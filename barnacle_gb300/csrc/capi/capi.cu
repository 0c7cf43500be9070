// The C-ABI: contexts, queries, render dispatch and statistics.
#include <cmath>
#include <cstring>
#include <string>
#include <vector>

#include "context.hpp"

namespace bnc {

bn::DevView make_dev_view(const bn_view& v, long long pixel_offset, long long path_offset) {
  // PinholeCamera.GenerateRay constants (Extensions/Camera/Pinhole.fs:16-22), float ops in
  // the reference order: vh = 2 tan(fov pi / 360), vw = vh * aspect, du = (vw, 0, 0) / W,
  // dv = (0, vh, 0) / H, upper-left = -UnitZ - 0.5 (viewportU + viewportV)
  bn::DevView d{};
  const float pi = 3.14159265f;
  const float vh = 2.f * std::tan(v.camera.fov_y_degrees * pi / 360.f);
  const float vw = vh * v.camera.aspect_ratio;
  const float W = static_cast<float>(v.width), H = static_cast<float>(v.height);
  const float vu[3] = {vw * 1.f, vw * 0.f, vw * 0.f};
  const float vv[3] = {vh * 0.f, vh * 1.f, vh * 0.f};
  const float mz[3] = {-0.f, -0.f, -1.f};
  for (int k = 0; k < 3; ++k) {
    d.du[k] = vu[k] / W;
    d.dv[k] = vv[k] / H;
    d.ul[k] = mz[k] - 0.5f * (vu[k] + vv[k]);
  }
  std::memcpy(d.c2w, v.camera.camera_to_world, sizeof(d.c2w));
  d.width = v.width;
  d.height = v.height;
  d.cam_type = v.camera.type;
  d.aperture = v.camera.aperture;
  d.focus_distance = v.camera.focus_distance;
  d.push_forward = v.camera.push_forward;
  d.pixel_offset = pixel_offset;
  d.path_offset = path_offset;
  return d;
}

MegaChunks mega_chunks(long long pixels, int spp, long long max_items) {
  // work items: pixels x chunks per view; enough threads to fill 152 SMs several times
  const long long target = 152LL * 2048 * 4;
  long long chunks = std::min<long long>(spp, std::max<long long>(1, (target + pixels - 1) / pixels));
  // a caller with a fixed scratch size: fewer, longer chunks until the partial sums fit
  if (max_items > 0) chunks = std::max<long long>(1, std::min<long long>(chunks, max_items / std::max(1LL, pixels)));
  const long long spc = (spp + chunks - 1) / chunks;
  MegaChunks c;
  c.spc = static_cast<int>(spc);
  c.chunks = static_cast<int>((spp + spc - 1) / spc);
  return c;
}

bn::MegaParams mega_params(const bn_context* ctx, const bn_render_desc* d, const std::vector<bn::DevView>& views,
                           const MegaChunks& ck, long long items, long long pixels) {
  bn::MegaParams p{};
  p.n_views = static_cast<int>(views.size());
  p.n_items = items;
  p.spp = d->spp;
  p.chunks = ck.chunks;
  p.spc = ck.spc;
  p.max_depth = d->max_depth;
  p.rr_depth = d->rr_depth;
  p.frame_id = d->frame_id;
  p.integrator = d->integrator;
  p.simple = ctx->scene_simple;
  for (const bn::DevView& v : views)
    if (v.cam_type == BN_CAM_THIN_LENS && v.aperture > 0.f) p.simple = false;
  p.watertight = d->flags & BN_RENDER_WATERTIGHT;
  p.n_pixels = pixels;
  p.counters = ctx->counters.as<bn::DevCounters>();
  return p;
}

int check_device_error(bn_context* ctx) {
  unsigned int w = 0;
  cudaError_t e = cudaMemcpyAsync(&w, ctx->error_word.ptr, sizeof(w), cudaMemcpyDeviceToHost, ctx->stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->stream);
  if (e != cudaSuccess) return ctx->cuda_fail(e, "kernel execution");
  ctx->stats.device_error = w;
  if (w) {
    cudaMemsetAsync(ctx->error_word.ptr, 0, sizeof(unsigned int), ctx->stream);
    cudaStreamSynchronize(ctx->stream);
    return ctx->fail(BN_ERR_DEVICE, "device error word 0x" + std::to_string(w) +
                                        " (1 stack overflow, 2 queue overflow, 4 watchdog, 8 bad index)");
  }
  return BN_OK;
}

}  // namespace bnc

namespace {

int read_counters(bn_context* ctx, bn::DevCounters* out) {
  cudaError_t e = cudaMemcpyAsync(out, ctx->counters.ptr, sizeof(bn::DevCounters), cudaMemcpyDeviceToHost, ctx->stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->stream);
  return e == cudaSuccess ? BN_OK : ctx->cuda_fail(e, "read counters");
}

int render_megakernel(bn_context* ctx, const bn_render_desc* d, const std::vector<bn::DevView>& views, bool count) {
  long long pixels = 0;
  for (const auto& v : views) pixels += static_cast<long long>(v.width) * v.height;
  const bnc::MegaChunks ck = bnc::mega_chunks(pixels, d->spp, 0);
  std::vector<long long> item_off(views.size());
  long long items = 0;
  for (size_t i = 0; i < views.size(); ++i) {
    item_off[i] = items;
    items += static_cast<long long>(views[i].width) * views[i].height * ck.chunks;
  }
  cudaError_t e;
  if ((e = ctx->item_offsets.reserve(item_off.size() * sizeof(long long))) != cudaSuccess)
    return ctx->cuda_fail(e, "alloc item offsets");
  if ((e = ctx->partial.reserve(static_cast<size_t>(items) * sizeof(float4))) != cudaSuccess)
    return ctx->cuda_fail(e, "alloc partial sums");
  cudaMemcpyAsync(ctx->item_offsets.ptr, item_off.data(), item_off.size() * sizeof(long long), cudaMemcpyHostToDevice,
                  ctx->stream);
  bn::MegaParams p = bnc::mega_params(ctx, d, views, ck, items, pixels);
  p.views = ctx->views.as<bn::DevView>();
  p.item_offsets = ctx->item_offsets.as<long long>();
  p.count = count;
  p.cull = d->flags & BN_RENDER_CULL_SHADOW;
  p.partial = ctx->partial.as<float4>();
  p.film = ctx->film.as<float>();
  cudaEventRecord(ctx->ev0, ctx->stream);
  if ((e = bn::launch_megakernel(ctx->scene, p, ctx->stream)) != cudaSuccess) return ctx->cuda_fail(e, "megakernel launch");
  cudaEventRecord(ctx->ev1, ctx->stream);
  if ((e = bn::launch_mega_reduce(p, ctx->stream)) != cudaSuccess) return ctx->cuda_fail(e, "reduce launch");
  cudaEventRecord(ctx->ev2, ctx->stream);
  if ((e = cudaEventSynchronize(ctx->ev2)) != cudaSuccess) return ctx->cuda_fail(e, "megakernel");
  float ms_main = 0.f, ms_all = 0.f;
  cudaEventElapsedTime(&ms_main, ctx->ev0, ctx->ev1);
  cudaEventElapsedTime(&ms_all, ctx->ev0, ctx->ev2);
  ctx->stats.last_dominant_ms = ms_main;
  ctx->stats.last_kernel_ms = ms_all;
  ctx->stats.last_launches = 2;
  ctx->stats.paths += static_cast<uint64_t>(pixels) * d->spp;
  return BN_OK;
}

}  // namespace

extern "C" {

const char* bn_version(void) { return "barnacle-gb300 1 (sm_103a)"; }

int bn_create(int device, bn_context** out) {
  if (!out) return BN_ERR_INVALID_ARG;
  *out = nullptr;
  int n = 0;
  cudaError_t e = cudaGetDeviceCount(&n);
  if (e != cudaSuccess || device < 0 || device >= n) return BN_ERR_CUDA;
  auto* ctx = new bn_context();
  ctx->device = device;
  if ((e = cudaSetDevice(device)) != cudaSuccess ||
      (e = cudaStreamCreateWithFlags(&ctx->stream, cudaStreamNonBlocking)) != cudaSuccess ||
      (e = cudaEventCreate(&ctx->ev0)) != cudaSuccess || (e = cudaEventCreate(&ctx->ev1)) != cudaSuccess ||
      (e = cudaEventCreate(&ctx->ev2)) != cudaSuccess || (e = ctx->error_word.reserve(256)) != cudaSuccess ||
      (e = ctx->counters.reserve(sizeof(bn::DevCounters))) != cudaSuccess) {
    delete ctx;
    return BN_ERR_CUDA;
  }
  cudaMemset(ctx->error_word.ptr, 0, 256);
  cudaMemset(ctx->counters.ptr, 0, sizeof(bn::DevCounters));
  *out = ctx;
  return BN_OK;
}

int bn_destroy(bn_context* ctx) {
  if (!ctx) return BN_OK;
  cudaSetDevice(ctx->device);
  cudaStreamSynchronize(ctx->stream);
  DevBuf* bufs[] = {&ctx->nodes, &ctx->nodes4, &ctx->rgba, &ctx->tris, &ctx->inst, &ctx->mats, &ctx->lights, &ctx->light_inst,
                    &ctx->tri_pdf, &ctx->tri_lights, &ctx->error_word, &ctx->counters, &ctx->q_in, &ctx->q_out,
                    &ctx->views, &ctx->item_offsets, &ctx->partial, &ctx->film, &ctx->wf_state, &ctx->mlt_state,
                    &ctx->mlt_boot, &ctx->mlt_chain, &ctx->adj_params, &ctx->adj_image, &ctx->adj_target,
                    &ctx->adj_grad, &ctx->adj_aux};
  for (DevBuf* b : bufs) b->release();
  if (ctx->wf && ctx->wf_release) ctx->wf_release(ctx->wf);
  cudaEventDestroy(ctx->ev0);
  cudaEventDestroy(ctx->ev1);
  cudaEventDestroy(ctx->ev2);
  cudaStreamDestroy(ctx->stream);
  delete ctx;
  return BN_OK;
}

int bn_last_error(const bn_context* ctx, char* buf, size_t len) {
  if (!ctx) return BN_ERR_INVALID_ARG;
  if (buf && len) {
    std::strncpy(buf, ctx->err.c_str(), len - 1);
    buf[len - 1] = '\0';
  }
  return static_cast<int>(ctx->err.size());
}

int bn_scene_instance_order(const bn_context* ctx, int32_t* out, int32_t n) {
  if (!ctx || !out) return BN_ERR_INVALID_ARG;
  if (!ctx->has_scene) return BN_ERR_NO_SCENE;
  if (n < static_cast<int32_t>(ctx->inst_order.size())) return BN_ERR_INVALID_ARG;
  std::memcpy(out, ctx->inst_order.data(), ctx->inst_order.size() * sizeof(int32_t));
  return BN_OK;
}

int bn_trace(bn_context* ctx, const bn_ray* rays, int64_t n, uint32_t flags, bn_hit* hits) {
  if (!ctx) return BN_ERR_INVALID_ARG;
  if (!ctx->has_scene) return ctx->fail(BN_ERR_NO_SCENE, "bn_trace before bn_scene_upload");
  if (n < 0 || (n > 0 && (!rays || !hits))) return ctx->fail(BN_ERR_INVALID_ARG, "bn_trace: bad arrays");
  if (n == 0) return BN_OK;
  cudaSetDevice(ctx->device);
  cudaError_t e;
  if ((e = ctx->q_in.reserve(n * sizeof(bn_ray))) != cudaSuccess) return ctx->cuda_fail(e, "alloc rays");
  if ((e = ctx->q_out.reserve(n * sizeof(bn_hit))) != cudaSuccess) return ctx->cuda_fail(e, "alloc hits");
  cudaMemcpyAsync(ctx->q_in.ptr, rays, n * sizeof(bn_ray), cudaMemcpyHostToDevice, ctx->stream);
  if (flags & BN_TRACE_COUNT) cudaMemsetAsync(ctx->counters.ptr, 0, sizeof(bn::DevCounters), ctx->stream);
  cudaEventRecord(ctx->ev0, ctx->stream);
  if ((e = bn::launch_trace(ctx->scene, ctx->q_in.as<bn_ray>(), ctx->q_out.as<bn_hit>(), n, flags,
                            ctx->counters.as<bn::DevCounters>(), ctx->stream)) != cudaSuccess)
    return ctx->cuda_fail(e, "trace launch");
  cudaEventRecord(ctx->ev1, ctx->stream);
  cudaMemcpyAsync(hits, ctx->q_out.ptr, n * sizeof(bn_hit), cudaMemcpyDeviceToHost, ctx->stream);
  if ((e = cudaStreamSynchronize(ctx->stream)) != cudaSuccess) return ctx->cuda_fail(e, "trace");
  float ms = 0.f;
  cudaEventElapsedTime(&ms, ctx->ev0, ctx->ev1);
  ctx->stats.last_kernel_ms = ms;
  ctx->stats.last_dominant_ms = ms;
  ctx->stats.last_launches = 1;
  if (flags & BN_TRACE_COUNT) {
    bn::DevCounters c{};
    int rc = read_counters(ctx, &c);
    if (rc) return rc;
    ctx->stats.rays += c.rays;
    ctx->stats.nodes_visited += c.nodes;
    ctx->stats.tris_tested += c.tris;
    ctx->stats.instances_visited += c.insts;
  } else {
    ctx->stats.rays += static_cast<uint64_t>(n);
  }
  return bnc::check_device_error(ctx);
}

static int bsdf_common(bn_context* ctx, const bn_bsdf_query* q, int64_t n, bn_bsdf_result* out, bool sample) {
  if (!ctx) return BN_ERR_INVALID_ARG;
  if (!ctx->has_scene) return ctx->fail(BN_ERR_NO_SCENE, "BSDF query before bn_scene_upload");
  if (n < 0 || (n > 0 && (!q || !out))) return ctx->fail(BN_ERR_INVALID_ARG, "BSDF query: bad arrays");
  if (n == 0) return BN_OK;
  cudaSetDevice(ctx->device);
  cudaError_t e;
  if ((e = ctx->q_in.reserve(n * sizeof(bn_bsdf_query))) != cudaSuccess) return ctx->cuda_fail(e, "alloc queries");
  if ((e = ctx->q_out.reserve(n * sizeof(bn_bsdf_result))) != cudaSuccess) return ctx->cuda_fail(e, "alloc results");
  cudaMemcpyAsync(ctx->q_in.ptr, q, n * sizeof(bn_bsdf_query), cudaMemcpyHostToDevice, ctx->stream);
  if ((e = bn::launch_bsdf(ctx->scene, ctx->q_in.as<bn_bsdf_query>(), ctx->q_out.as<bn_bsdf_result>(), n, sample,
                           ctx->stream)) != cudaSuccess)
    return ctx->cuda_fail(e, "bsdf launch");
  cudaMemcpyAsync(out, ctx->q_out.ptr, n * sizeof(bn_bsdf_result), cudaMemcpyDeviceToHost, ctx->stream);
  if ((e = cudaStreamSynchronize(ctx->stream)) != cudaSuccess) return ctx->cuda_fail(e, "bsdf");
  return bnc::check_device_error(ctx);
}

int bn_bsdf_eval(bn_context* ctx, const bn_bsdf_query* q, int64_t n, bn_bsdf_result* out) {
  return bsdf_common(ctx, q, n, out, false);
}
int bn_bsdf_sample(bn_context* ctx, const bn_bsdf_query* q, int64_t n, bn_bsdf_result* out) {
  return bsdf_common(ctx, q, n, out, true);
}

int bn_sampler_stream(bn_context* ctx, const uint32_t* seeds, int64_t n_streams, int32_t n_draws, float* out) {
  if (!ctx) return BN_ERR_INVALID_ARG;
  if (n_streams < 0 || n_draws < 0 || (n_streams > 0 && (!seeds || !out)))
    return ctx->fail(BN_ERR_INVALID_ARG, "bn_sampler_stream: bad arrays");
  if (n_streams == 0 || n_draws == 0) return BN_OK;
  cudaSetDevice(ctx->device);
  cudaError_t e;
  if ((e = ctx->q_in.reserve(n_streams * 3 * sizeof(uint32_t))) != cudaSuccess) return ctx->cuda_fail(e, "alloc seeds");
  if ((e = ctx->q_out.reserve(n_streams * n_draws * sizeof(float))) != cudaSuccess) return ctx->cuda_fail(e, "alloc draws");
  cudaMemcpyAsync(ctx->q_in.ptr, seeds, n_streams * 3 * sizeof(uint32_t), cudaMemcpyHostToDevice, ctx->stream);
  if ((e = bn::launch_sampler_stream(ctx->q_in.as<uint32_t>(), n_streams, n_draws, ctx->q_out.as<float>(), ctx->stream)) !=
      cudaSuccess)
    return ctx->cuda_fail(e, "sampler launch");
  cudaMemcpyAsync(out, ctx->q_out.ptr, n_streams * n_draws * sizeof(float), cudaMemcpyDeviceToHost, ctx->stream);
  if ((e = cudaStreamSynchronize(ctx->stream)) != cudaSuccess) return ctx->cuda_fail(e, "sampler");
  return BN_OK;
}

int bn_render(bn_context* ctx, const bn_render_desc* d, const bn_view* views, int32_t n_views, float* out_rgb) {
  if (!ctx) return BN_ERR_INVALID_ARG;
  if (!ctx->has_scene) return ctx->fail(BN_ERR_NO_SCENE, "bn_render before bn_scene_upload");
  if (!d || !views || n_views <= 0) return ctx->fail(BN_ERR_INVALID_ARG, "bn_render: bad descriptor or views");
  if (d->spp <= 0 || d->max_depth < 0 || d->rr_depth < 0)
    return ctx->fail(BN_ERR_INVALID_ARG, "bn_render: spp must be positive, depths non-negative");
  cudaSetDevice(ctx->device);
  std::vector<bn::DevView> dv;
  long long pix = 0, paths = 0;
  for (int i = 0; i < n_views; ++i) {
    if (views[i].width <= 0 || views[i].height <= 0) return ctx->fail(BN_ERR_INVALID_ARG, "view with empty film");
    dv.push_back(bnc::make_dev_view(views[i], pix, paths));
    pix += static_cast<long long>(views[i].width) * views[i].height;
    paths += static_cast<long long>(views[i].width) * views[i].height * d->spp;
  }
  cudaError_t e;
  if ((e = ctx->views.reserve(dv.size() * sizeof(bn::DevView))) != cudaSuccess) return ctx->cuda_fail(e, "alloc views");
  if ((e = ctx->film.reserve(static_cast<size_t>(pix) * 3 * sizeof(float))) != cudaSuccess)
    return ctx->cuda_fail(e, "alloc film");
  ctx->film_floats = pix * 3;
  cudaMemcpyAsync(ctx->views.ptr, dv.data(), dv.size() * sizeof(bn::DevView), cudaMemcpyHostToDevice, ctx->stream);
  const bool count = d->flags & BN_RENDER_COUNT;
  if (count) cudaMemsetAsync(ctx->counters.ptr, 0, sizeof(bn::DevCounters), ctx->stream);
  int rc;
  if (d->integrator == BN_INTEGRATOR_PSSMLT) {
    rc = bnc::render_pssmlt(ctx, d, dv);
  } else if (d->integrator == BN_INTEGRATOR_PATH || d->integrator == BN_INTEGRATOR_NORMAL ||
             d->integrator == BN_INTEGRATOR_DIRECT) {
    if (d->mode == BN_MODE_WAVEFRONT) rc = bnc::render_wavefront(ctx, d, dv);
    else if (d->mode == BN_MODE_MEGAKERNEL) rc = render_megakernel(ctx, d, dv, count);
    else return ctx->fail(BN_ERR_INVALID_ARG, "unknown render mode");
  } else {
    return ctx->fail(BN_ERR_INVALID_ARG, "unknown integrator");
  }
  if (rc) return rc;
  if ((rc = bnc::check_device_error(ctx)) != BN_OK) return rc;
  if (count) {
    bn::DevCounters c{};
    if ((rc = read_counters(ctx, &c)) != BN_OK) return rc;
    ctx->stats.rays += c.rays;
    ctx->stats.nodes_visited += c.nodes;
    ctx->stats.tris_tested += c.tris;
    ctx->stats.instances_visited += c.insts;
  }
  if (out_rgb) {
    e = cudaMemcpyAsync(out_rgb, ctx->film.ptr, static_cast<size_t>(pix) * 3 * sizeof(float), cudaMemcpyDeviceToHost,
                        ctx->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->stream);
    if (e != cudaSuccess) return ctx->cuda_fail(e, "film download");
  }
  return BN_OK;
}

int bn_film_download(bn_context* ctx, float* out_rgb, int64_t n_floats) {
  if (!ctx || !out_rgb) return BN_ERR_INVALID_ARG;
  if (n_floats > ctx->film_floats) return ctx->fail(BN_ERR_INVALID_ARG, "bn_film_download: more floats than the film holds");
  cudaSetDevice(ctx->device);
  cudaError_t e = cudaMemcpyAsync(out_rgb, ctx->film.ptr, n_floats * sizeof(float), cudaMemcpyDeviceToHost, ctx->stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->stream);
  return e == cudaSuccess ? BN_OK : ctx->cuda_fail(e, "film download");
}

int bn_film_tonemap(bn_context* ctx, int32_t tone_mapping, uint8_t* rgba, int64_t n_pixels) {
  if (!ctx || !rgba) return BN_ERR_INVALID_ARG;
  if (tone_mapping != BN_TONE_IDENTITY && tone_mapping != BN_TONE_ACES && tone_mapping != BN_TONE_GAMMA)
    return ctx->fail(BN_ERR_INVALID_ARG, "bn_film_tonemap: unknown tone mapping");
  if (n_pixels <= 0 || 3 * n_pixels > ctx->film_floats)
    return ctx->fail(BN_ERR_INVALID_ARG, "bn_film_tonemap: n_pixels must be 1 .. the last render's film pixels");
  cudaSetDevice(ctx->device);
  cudaError_t e = ctx->rgba.reserve(static_cast<size_t>(n_pixels) * 4);
  if (e != cudaSuccess) return ctx->cuda_fail(e, "alloc tone-mapped film");
  if ((e = bn::launch_film_tonemap(ctx->film.as<float>(), n_pixels, tone_mapping, ctx->rgba.ptr, ctx->stream)) !=
      cudaSuccess)
    return ctx->cuda_fail(e, "tone-map launch");
  e = cudaMemcpyAsync(rgba, ctx->rgba.ptr, static_cast<size_t>(n_pixels) * 4, cudaMemcpyDeviceToHost, ctx->stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->stream);
  return e == cudaSuccess ? BN_OK : ctx->cuda_fail(e, "tone-mapped film download");
}

int bn_set_limits(bn_context* ctx, int32_t stack_entries, int32_t max_bounce_iterations) {
  if (!ctx) return BN_ERR_INVALID_ARG;
  if (stack_entries < 0 || stack_entries > bn::kStackSize || max_bounce_iterations < 0)
    return ctx->fail(BN_ERR_INVALID_ARG, "bn_set_limits: stack entries 0.." + std::to_string(bn::kStackSize) +
                                             ", iterations >= 0 (0 = default)");
  ctx->limit_stack = stack_entries;
  ctx->limit_iters = max_bounce_iterations;
  ctx->scene.stack_cap = stack_entries > 0 ? stack_entries : bn::kStackSize;
  return BN_OK;
}

int bn_get_stats(const bn_context* ctx, bn_stats* out) {
  if (!ctx || !out) return BN_ERR_INVALID_ARG;
  *out = ctx->stats;
  return BN_OK;
}

int bn_reset_stats(bn_context* ctx) {
  if (!ctx) return BN_ERR_INVALID_ARG;
  ctx->stats = bn_stats{};
  return BN_OK;
}

}  // extern "C"
