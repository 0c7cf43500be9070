// bn_render_noalloc: the plain megakernel render for callers that must not allocate device
// memory during the call.
//
// Who needs it: a host that owns every device byte through its own arena and forbids allocation
// inside its frame loop (cudaMalloc/cudaFree synchronise the device and can stall the loop), or a
// caller with a fixed memory budget on a shared GPU.  Such a caller uploads the scene once at
// set-up time (bn_scene_upload allocates then) and afterwards renders into a film buffer it owns.
//
// bn_render keeps its per-call scratch (view records, per-view item offsets, the partial sums of
// each sample chunk) in buffers it grows with cudaMalloc.  This entry point keeps the same scratch
// in one file-scope __device__ array of fixed size instead, so the call itself allocates nothing:
// it copies the view records into the array, launches the same two kernels as bn_render's
// megakernel mode (k_pt_mega, k_mega_reduce) and writes the caller's film.
//
//  * limits: at most kMaxViews (64) views and kMaxItems (1,048,576) partial sums, i.e. 16 MiB of
//    partial sums; every GPU that loads the library holds the array until the process exits.
//    A render with more than kMaxItems pixels in total is rejected.  While pixels x bn_render's
//    chunks per pixel fit the array the image is bit-identical to bn_render's; beyond that the
//    call uses fewer, longer sample chunks, so each chunk sums more samples and the image equals
//    bn_render's only up to float summation order (the per-path radiance is the same).
//  * not supported: BN_RENDER_COUNT (visit counting needs no scratch-free form); the context's own
//    film (bn_film_download, bn_film_tonemap) is not written, it keeps the last bn_render's image.
//  * set-up: the first call on a device resolves the array's device address with
//    cudaGetSymbolAddress (with that device current; this may load the library's device code on
//    that GPU).  Make the first call on each device before any stream capture.
//  * sharing: every call uses the same array and it keeps the last call's contents.  Each call
//    overwrites every view record, offset and partial sum it reads, so nothing is cleared; calls
//    that overlap on the GPU (two streams or two contexts on one device) race on the array.
#include <mutex>
#include <string>
#include <vector>

#include "context.hpp"

namespace {

constexpr int kMaxViews = 64;
constexpr long long kMaxItems = 1LL << 20;

struct NoAllocScratch {
  bn::DevView views[kMaxViews];
  long long item_offsets[kMaxViews];
  float4 partial[kMaxItems];
};

__device__ __align__(256) NoAllocScratch g_noalloc_scratch;

std::mutex g_setup_mu;
constexpr int kMaxDevices = 256;
NoAllocScratch* g_scratch_ptr[kMaxDevices] = {};

// once per device, with that device current: the array's device address (the host-side name is
// only a stand-in and must never reach a kernel)
int scratch_for_device(bn_context* ctx, NoAllocScratch** out) {
  if (ctx->device < 0 || ctx->device >= kMaxDevices) return ctx->fail(BN_ERR_UNSUPPORTED, "device index too large");
  std::lock_guard<std::mutex> lock(g_setup_mu);
  if (!g_scratch_ptr[ctx->device]) {
    void* p = nullptr;
    const cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
    if (e != cudaSuccess) return ctx->cuda_fail(e, "bn_render_noalloc: cudaGetSymbolAddress of the scratch array");
    g_scratch_ptr[ctx->device] = static_cast<NoAllocScratch*>(p);
  }
  *out = g_scratch_ptr[ctx->device];
  return BN_OK;
}

}  // namespace

extern "C" int bn_render_noalloc(bn_context* ctx, const bn_render_desc* d, const bn_view* views, int32_t n_views,
                                 float* film_device) {
  if (!ctx) return BN_ERR_INVALID_ARG;
  if (!ctx->has_scene) return ctx->fail(BN_ERR_NO_SCENE, "bn_render_noalloc before bn_scene_upload");
  if (!d || !views || !film_device) return ctx->fail(BN_ERR_INVALID_ARG, "bn_render_noalloc: null descriptor, views or film");
  if (n_views <= 0 || n_views > kMaxViews)
    return ctx->fail(BN_ERR_INVALID_ARG, "bn_render_noalloc: 1 to " + std::to_string(kMaxViews) + " views, got " +
                                             std::to_string(n_views));
  if (d->integrator != BN_INTEGRATOR_PATH || d->mode != BN_MODE_MEGAKERNEL)
    return ctx->fail(BN_ERR_UNSUPPORTED, "bn_render_noalloc renders the path-tracing megakernel mode only");
  if (d->flags & BN_RENDER_COUNT)
    return ctx->fail(BN_ERR_UNSUPPORTED, "bn_render_noalloc does not count visits (BN_RENDER_COUNT): use bn_render");
  if (d->spp <= 0 || d->max_depth < 0 || d->rr_depth < 0)
    return ctx->fail(BN_ERR_INVALID_ARG, "bn_render_noalloc: spp must be positive, depths non-negative");
  cudaError_t e = cudaSetDevice(ctx->device);
  if (e != cudaSuccess) return ctx->cuda_fail(e, "bn_render_noalloc: cudaSetDevice");
  // the film must be device memory of this context's GPU: a host pointer or another GPU's memory
  // would make the reduction kernel fault
  cudaPointerAttributes attr{};
  e = cudaPointerGetAttributes(&attr, film_device);
  if (e != cudaSuccess) {
    cudaGetLastError();  // clear the sticky-free error of an unknown pointer
    return ctx->fail(BN_ERR_INVALID_ARG, "bn_render_noalloc: film_device is not a CUDA pointer");
  }
  if ((attr.type != cudaMemoryTypeDevice && attr.type != cudaMemoryTypeManaged) || attr.device != ctx->device)
    return ctx->fail(BN_ERR_INVALID_ARG, "bn_render_noalloc: film_device must be device memory of GPU " +
                                             std::to_string(ctx->device));
  NoAllocScratch* scratch = nullptr;
  int rc = scratch_for_device(ctx, &scratch);
  if (rc) return rc;

  std::vector<bn::DevView> dv;
  long long pixels = 0;
  for (int i = 0; i < n_views; ++i) {
    if (views[i].width <= 0 || views[i].height <= 0) return ctx->fail(BN_ERR_INVALID_ARG, "view with empty film");
    dv.push_back(bnc::make_dev_view(views[i], pixels, pixels * d->spp));
    pixels += static_cast<long long>(views[i].width) * views[i].height;
  }
  if (pixels > kMaxItems)
    return ctx->fail(BN_ERR_INVALID_ARG, "bn_render_noalloc: " + std::to_string(pixels) + " pixels exceed the " +
                                             std::to_string(kMaxItems) + "-pixel limit of its static scratch");
  // bn_render's chunking, capped so that the partial sums fit the array
  const bnc::MegaChunks ck = bnc::mega_chunks(pixels, d->spp, kMaxItems);
  std::vector<long long> item_off(n_views);
  long long items = 0;
  for (int i = 0; i < n_views; ++i) {
    item_off[i] = items;
    items += static_cast<long long>(views[i].width) * views[i].height * ck.chunks;
  }
  if ((e = cudaMemcpyAsync(scratch->views, dv.data(), dv.size() * sizeof(bn::DevView), cudaMemcpyHostToDevice,
                           ctx->stream)) != cudaSuccess ||
      (e = cudaMemcpyAsync(scratch->item_offsets, item_off.data(), item_off.size() * sizeof(long long),
                           cudaMemcpyHostToDevice, ctx->stream)) != cudaSuccess)
    return ctx->cuda_fail(e, "bn_render_noalloc: view upload");

  bn::MegaParams p = bnc::mega_params(ctx, d, dv, ck, items, pixels);
  p.views = scratch->views;
  p.item_offsets = scratch->item_offsets;
  p.count = false;
  p.cull = d->flags & BN_RENDER_CULL_SHADOW;
  p.partial = scratch->partial;
  p.film = film_device;
  cudaEventRecord(ctx->ev0, ctx->stream);
  if ((e = bn::launch_megakernel(ctx->scene, p, ctx->stream)) != cudaSuccess)
    return ctx->cuda_fail(e, "bn_render_noalloc: megakernel launch");
  cudaEventRecord(ctx->ev1, ctx->stream);
  if ((e = bn::launch_mega_reduce(p, ctx->stream)) != cudaSuccess)
    return ctx->cuda_fail(e, "bn_render_noalloc: reduce launch");
  cudaEventRecord(ctx->ev2, ctx->stream);
  if ((e = cudaEventSynchronize(ctx->ev2)) != cudaSuccess) return ctx->cuda_fail(e, "bn_render_noalloc");
  float ms_main = 0.f, ms_all = 0.f;
  cudaEventElapsedTime(&ms_main, ctx->ev0, ctx->ev1);
  cudaEventElapsedTime(&ms_all, ctx->ev0, ctx->ev2);
  ctx->stats.last_dominant_ms = ms_main;
  ctx->stats.last_kernel_ms = ms_all;
  ctx->stats.last_launches = 2;
  ctx->stats.paths += static_cast<uint64_t>(pixels) * d->spp;
  return bnc::check_device_error(ctx);
}
