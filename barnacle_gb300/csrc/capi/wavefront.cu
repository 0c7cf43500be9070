// Wavefront render orchestration: path-state buffers, the CUDA graph whose while-node runs the
// whole bounce loop on the device, the host-driven fallback loop, and the launch autotuner.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <string>
#include <vector>

#include "../device/pssmlt.hpp"
#include "../device/wavefront.hpp"
#include "context.hpp"

namespace {

struct WfState {
  int pool = 0;
  DevBuf params, ray, bl, hit, meta, q_active, q_bins, shadow, counters, work_next, film_acc;
  DevBuf mlt_smp, mlt_chain;  // PSSMLT chains: sampler state and chain records
  DevBuf slot_key, q_key, q_ray, sh_key, q_shadow, hist, off;
  // captured graph (one per launch shape)
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t exec = nullptr;
  cudaGraphConditionalHandle cond = 0;
  bool graph_failed = false;
  bn::WfLaunch shape{};
  int shape_cap = -1;
  // autotuned choice per uploaded scene and triangle test (index: watertight)
  long long tuned_generation[2] = {-1, -1};
  int tuned_pool[2] = {0, 0}, tuned_cap[2] = {0, 0}, tuned_refill[2] = {16, 16};
  // the PSSMLT iteration's second stream and its fork / join events (made on first use)
  bn::WfFork fork{nullptr, nullptr, nullptr};

  cudaError_t ensure_fork() {
    cudaError_t e = cudaSuccess;
    if (!fork.side) e = cudaStreamCreateWithFlags(&fork.side, cudaStreamNonBlocking);
    if (e == cudaSuccess && !fork.fork) e = cudaEventCreateWithFlags(&fork.fork, cudaEventDisableTiming);
    if (e == cudaSuccess && !fork.join) e = cudaEventCreateWithFlags(&fork.join, cudaEventDisableTiming);
    return e;
  }

  void release() {
    DevBuf* b[] = {&params, &ray, &bl, &hit, &meta, &q_active, &q_bins, &shadow, &counters,
                   &work_next, &film_acc, &slot_key, &q_key, &q_ray, &sh_key, &q_shadow, &hist, &off,
                   &mlt_smp, &mlt_chain};
    for (DevBuf* x : b) x->release();
    if (exec) cudaGraphExecDestroy(exec);
    if (graph) cudaGraphDestroy(graph);
    exec = nullptr;
    graph = nullptr;
    if (fork.fork) cudaEventDestroy(fork.fork);
    if (fork.join) cudaEventDestroy(fork.join);
    if (fork.side) cudaStreamDestroy(fork.side);
    fork = bn::WfFork{nullptr, nullptr, nullptr};
  }
};

WfState* state(bn_context* ctx) {
  if (!ctx->wf) {
    ctx->wf = new WfState();
    ctx->wf_release = [](void* p) {
      auto* s = static_cast<WfState*>(p);
      s->release();
      delete s;
    };
  }
  return static_cast<WfState*>(ctx->wf);
}

cudaError_t ensure_pool(WfState* w, int pool) {
  if (w->pool == pool) return cudaSuccess;
  cudaError_t e;
  const size_t P = static_cast<size_t>(pool);
  if ((e = w->params.reserve(sizeof(bn::WfParams))) != cudaSuccess) return e;
  if ((e = w->ray.reserve(2 * P * sizeof(float4))) != cudaSuccess) return e;
  if ((e = w->bl.reserve(2 * P * sizeof(float4))) != cudaSuccess) return e;
  if ((e = w->hit.reserve(2 * P * sizeof(float4))) != cudaSuccess) return e;
  if ((e = w->meta.reserve(P * sizeof(int4))) != cudaSuccess) return e;
  if ((e = w->q_active.reserve(P * sizeof(int))) != cudaSuccess) return e;
  if ((e = w->q_bins.reserve(P * bn::kNumBins * sizeof(int))) != cudaSuccess) return e;
  if ((e = w->shadow.reserve(P * 4 * sizeof(float4))) != cudaSuccess) return e;
  if ((e = w->counters.reserve(bn::kCntSize * sizeof(int))) != cudaSuccess) return e;
  if ((e = w->work_next.reserve(sizeof(unsigned long long))) != cudaSuccess) return e;
  for (DevBuf* b : {&w->slot_key, &w->q_key, &w->q_ray, &w->sh_key, &w->q_shadow})
    if ((e = b->reserve(P * sizeof(int))) != cudaSuccess) return e;
  if ((e = w->hist.reserve(bn::kSortBins * sizeof(unsigned))) != cudaSuccess) return e;
  if ((e = w->off.reserve((bn::kSortBins + bn::kSortBins / 1024) * sizeof(unsigned))) != cudaSuccess) return e;
  w->pool = pool;
  return cudaSuccess;
}

// the while-node graph of the path tracer: body = one iteration (regen, extend, shade, shadow,
// control)
int build_graph(bn_context* ctx, WfState* w) {
  if (w->exec) {
    cudaGraphExecDestroy(w->exec);
    w->exec = nullptr;
  }
  if (w->graph) {
    cudaGraphDestroy(w->graph);
    w->graph = nullptr;
  }
  cudaError_t e;
  if ((e = cudaGraphCreate(&w->graph, 0)) != cudaSuccess) return ctx->cuda_fail(e, "cudaGraphCreate");
  if ((e = cudaGraphConditionalHandleCreate(&w->cond, w->graph, 1, cudaGraphCondAssignDefault)) != cudaSuccess)
    return ctx->cuda_fail(e, "cudaGraphConditionalHandleCreate");
  cudaGraphNodeParams np{};
  np.type = cudaGraphNodeTypeConditional;
  np.conditional.handle = w->cond;
  np.conditional.type = cudaGraphCondTypeWhile;
  np.conditional.size = 1;
  cudaGraphNode_t node;
  if ((e = cudaGraphAddNode(&node, w->graph, nullptr, nullptr, 0, &np)) != cudaSuccess)
    return ctx->cuda_fail(e, "cudaGraphAddNode(while)");
  cudaGraph_t body = np.conditional.phGraph_out[0];
  if ((e = cudaStreamBeginCaptureToGraph(ctx->stream, body, nullptr, nullptr, 0, cudaStreamCaptureModeRelaxed)) !=
      cudaSuccess)
    return ctx->cuda_fail(e, "cudaStreamBeginCaptureToGraph");
  cudaError_t le = bn::wf_launch_iteration(w->params.as<bn::WfParams>(), w->shape, true, ctx->stream);
  cudaGraph_t captured = body;
  e = cudaStreamEndCapture(ctx->stream, &captured);
  if (le != cudaSuccess) return ctx->cuda_fail(le, "capture of the bounce loop");
  if (e != cudaSuccess) return ctx->cuda_fail(e, "cudaStreamEndCapture");
  if ((e = cudaGraphInstantiate(&w->exec, w->graph, 0)) != cudaSuccess) return ctx->cuda_fail(e, "cudaGraphInstantiate");
  return BN_OK;
}

// One render (or a truncated tuning render) into w->film_acc / ctx->film.
int run(bn_context* ctx, WfState* w, const bn_render_desc* d, long long n_pixels, long long total_paths, int n_views,
        int pool, int cap, int refill, bool use_graph, float* ms_out) {
  cudaError_t e;
  if ((e = ensure_pool(w, pool)) != cudaSuccess) return ctx->cuda_fail(e, "wavefront path-state allocation");
  if ((e = w->film_acc.reserve(static_cast<size_t>(n_pixels) * 3 * sizeof(double))) != cudaSuccess)
    return ctx->cuda_fail(e, "wavefront film allocation");
  const bool wt = d->flags & BN_RENDER_WATERTIGHT;
  const bool wide = ctx->scene.wide != 0;
  // both queues sorted by ray key: on the 1,024-instance workload 111.5 M paths/s against 110.0
  // (ray queue only) and 107.9 (neither)
  const bool sort = true, sort_shadow = true;
  const bool count = d->flags & BN_RENDER_COUNT;
  const int key_bits = bn::sort_key_bits(pool);
  if (w->shape_cap != cap || w->shape.watertight != wt || w->shape.wide != wide || w->shape.sort != sort ||
      w->shape.sort_shadow != sort_shadow || w->shape.count != count || w->shape.mlt ||
      w->shape.sort_tiles != (1 << (2 * key_bits + 6)) / 1024) {
    w->shape = bn::wf_launch_shape(wt, wide, sort, sort_shadow, count, cap, false, false, 0, key_bits);
    w->shape_cap = cap;
    if (w->exec) {
      cudaGraphExecDestroy(w->exec);
      w->exec = nullptr;
    }
  }
  bn::WfParams p{};
  p.scene = ctx->scene;
  p.views = ctx->views.as<bn::DevView>();
  p.n_views = n_views;
  p.spp = d->spp;
  p.max_depth = d->max_depth;
  p.rr_depth = d->rr_depth;
  p.frame_id = d->frame_id;
  p.integrator = d->integrator;
  p.pool = pool;
  // refill thresholds (lanes of 32 still walking; autotuned, 16 unless told otherwise)
  p.refill_extend = refill;
  p.refill_shadow = refill;
  p.total_paths = total_paths;
  p.n_pixels = n_pixels;
  p.max_iters = static_cast<int>(std::min<long long>(1LL << 30, (total_paths / pool + 2) * (d->max_depth + 2) + 64));
  if (ctx->limit_iters > 0) p.max_iters = ctx->limit_iters;
  p.ray = w->ray.as<float4>();
  p.bl = w->bl.as<float4>();
  p.hit = w->hit.as<float4>();
  p.meta = w->meta.as<int4>();
  p.q_active = w->q_active.as<int>();
  p.sort = sort ? 1 : 0;
  p.sort_shadow = sort_shadow ? 1 : 0;
  {
    float lo[3], sc[3];
    for (int a = 0; a < 3; ++a) {
      const float ext = ctx->scene_hi[a] - ctx->scene_lo[a];
      lo[a] = ctx->scene_lo[a];
      sc[a] = ext > 0.f && std::isfinite(ext) ? (a == 1 ? 8.f : static_cast<float>(1 << key_bits)) / ext : 0.f;
    }
    p.key_lo = make_float4(lo[0], lo[1], lo[2], 0.f);
    p.key_scale = make_float4(sc[0], sc[1], sc[2], 0.f);
    p.key_bits = key_bits;
  }
  p.slot_key = w->slot_key.as<int>();
  p.q_key = w->q_key.as<int>();
  p.q_ray = sort ? w->q_ray.as<int>() : w->q_active.as<int>();
  p.sh_key = w->sh_key.as<int>();
  p.q_shadow = w->q_shadow.as<int>();
  p.hist = w->hist.as<unsigned>();
  p.off = w->off.as<unsigned>();
  p.q_bins = w->q_bins.as<int>();
  p.shadow = w->shadow.as<float4>();
  p.counters = w->counters.as<int>();
  p.trace_counters = ctx->counters.ptr;
  p.work_next = w->work_next.as<unsigned long long>();
  p.film_acc = w->film_acc.as<double>();
  p.film_out = ctx->film.as<float>();
  if (use_graph && !w->exec && !w->graph_failed) {
    if (build_graph(ctx, w) != BN_OK) {
      w->graph_failed = true;  // fall back to the host-driven loop; the message stays in ctx->err
      use_graph = false;
    }
  }
  if (use_graph && !w->exec) use_graph = false;
  p.cond = w->cond;
  cudaStream_t st = ctx->stream;
  cudaMemcpyAsync(w->params.ptr, &p, sizeof(p), cudaMemcpyHostToDevice, st);
  cudaMemsetAsync(w->counters.ptr, 0, bn::kCntSize * sizeof(int), st);
  cudaMemsetAsync(w->hist.ptr, 0, bn::kSortBins * sizeof(unsigned), st);
  cudaMemsetAsync(w->work_next.ptr, 0, sizeof(unsigned long long), st);
  cudaMemsetAsync(w->meta.ptr, 0, static_cast<size_t>(pool) * sizeof(int4), st);
  cudaMemsetAsync(w->film_acc.ptr, 0, static_cast<size_t>(n_pixels) * 3 * sizeof(double), st);
  cudaEventRecord(ctx->ev0, st);
  int launches = 0;
  if (use_graph) {
    if ((e = cudaGraphLaunch(w->exec, st)) != cudaSuccess) return ctx->cuda_fail(e, "cudaGraphLaunch");
  } else {
    for (int it = 0; it < p.max_iters + 1; ++it) {
      if ((e = bn::wf_launch_iteration(w->params.as<bn::WfParams>(), w->shape, false, st)) != cudaSuccess)
        return ctx->cuda_fail(e, "wavefront iteration launch");
      launches += 5 + (sort ? 3 : 0) + (sort_shadow ? 3 : 0);
      int again = 0;
      cudaMemcpyAsync(&again, w->counters.as<int>() + bn::kCntAgain, sizeof(int), cudaMemcpyDeviceToHost, st);
      if ((e = cudaStreamSynchronize(st)) != cudaSuccess) return ctx->cuda_fail(e, "wavefront iteration");
      if (!again) break;
    }
  }
  cudaEventRecord(ctx->ev1, st);
  if ((e = bn::wf_launch_resolve(w->params.as<bn::WfParams>(), st)) != cudaSuccess)
    return ctx->cuda_fail(e, "wavefront resolve");
  cudaEventRecord(ctx->ev2, st);
  if ((e = cudaEventSynchronize(ctx->ev2)) != cudaSuccess) return ctx->cuda_fail(e, "wavefront render");
  int counters[bn::kCntSize];
  cudaMemcpy(counters, w->counters.ptr, sizeof(counters), cudaMemcpyDeviceToHost);
  float ms_loop = 0.f, ms_all = 0.f;
  cudaEventElapsedTime(&ms_loop, ctx->ev0, ctx->ev1);
  cudaEventElapsedTime(&ms_all, ctx->ev0, ctx->ev2);
  if (use_graph) launches = (5 + (sort ? 3 : 0) + (sort_shadow ? 3 : 0)) * counters[bn::kCntIter];
  ctx->stats.last_kernel_ms = ms_all;
  ctx->stats.last_dominant_ms = ms_loop;
  ctx->stats.last_launches = launches + 1;
  if (ms_out) *ms_out = ms_all;
  return BN_OK;
}

// The bounce loop of PSSMLT chains (one slot per chain), enqueued on the context's stream after
// the bootstrap as host-driven iterations: a render of 65,536 chains runs about 2,100 short ones,
// and measured at 1024^2 they took 435-454 ms as launches from the host against 489-500 ms as the
// iterations of a conditional graph node.  Splats go straight into ctx->film.  Returns the
// iterations run through *iters.
int run_mlt(bn_context* ctx, WfState* w, const bn_render_desc* d, const bn::MltParams& mp, int* iters) {
  cudaError_t e;
  const int pool = mp.n_chains;
  if ((e = ensure_pool(w, pool)) != cudaSuccess) return ctx->cuda_fail(e, "wavefront chain-state allocation");
  if ((e = w->ensure_fork()) != cudaSuccess) return ctx->cuda_fail(e, "wavefront chain stream");
  if ((e = w->mlt_smp.reserve(static_cast<size_t>(pool) * sizeof(int4))) != cudaSuccess ||
      (e = w->mlt_chain.reserve(static_cast<size_t>(pool) * 3 * sizeof(float4))) != cudaSuccess)
    return ctx->cuda_fail(e, "wavefront chain records");
  const bool wt = d->flags & BN_RENDER_WATERTIGHT;
  const bool wide = ctx->scene.wide != 0;
  const bool kelemen = mp.kelemen != 0;
  // 65,536 chains are few rays per launch: the queues are traversed unsorted
  const bn::WfLaunch want = bn::wf_launch_shape(wt, wide, false, false, false, 0, true, kelemen, pool);
  if (!w->shape.mlt || w->shape.watertight != wt || w->shape.wide != wide || w->shape.mlt_kelemen != kelemen ||
      w->shape.grid_extend != want.grid_extend || w->shape.grid_shadow != want.grid_shadow) {
    w->shape = want;
    w->shape_cap = -1;
    if (w->exec) {
      cudaGraphExecDestroy(w->exec);
      w->exec = nullptr;
    }
  }
  bn::WfParams p{};
  p.scene = ctx->scene;
  p.views = mp.view;
  p.n_views = 1;
  p.spp = d->spp;
  p.max_depth = d->max_depth;
  p.rr_depth = d->rr_depth;
  p.frame_id = d->frame_id;
  p.integrator = BN_INTEGRATOR_PSSMLT;
  p.pool = pool;
  p.refill_extend = 16;
  p.refill_shadow = 16;
  p.total_paths = 0;
  p.n_pixels = 0;
  // a mutation's path takes at most max_depth iterations (at least one), and one more when its
  // last shadow record is traced after it ends
  p.max_iters = static_cast<int>(std::min<long long>(
      1LL << 30, (static_cast<long long>(mp.mutations_per_chain) + 1) * (std::max(1, d->max_depth) + 1) + 64));
  if (ctx->limit_iters > 0) p.max_iters = ctx->limit_iters;
  p.ray = w->ray.as<float4>();
  p.bl = w->bl.as<float4>();
  p.hit = w->hit.as<float4>();
  p.meta = w->meta.as<int4>();
  p.q_active = w->q_active.as<int>();
  p.sort = 0;
  p.sort_shadow = 0;
  p.key_bits = 5;
  p.q_ray = w->q_active.as<int>();
  p.q_bins = w->q_bins.as<int>();
  p.shadow = w->shadow.as<float4>();
  p.counters = w->counters.as<int>();
  p.trace_counters = ctx->counters.ptr;
  p.work_next = w->work_next.as<unsigned long long>();
  p.film_out = mp.film;
  p.mlt = 1;
  bn::MltWf& q = p.mlt_p;
  q.n_chains = mp.n_chains;
  q.n_bootstrap = mp.n_bootstrap;
  q.n_dims = mp.n_dims;
  q.mutations = mp.mutations_per_chain;
  q.kelemen = mp.kelemen;
  q.p_large = mp.large_step_prob;
  q.sigma = mp.sigma;
  q.eps_min = mp.eps_min;
  q.eps_max = mp.eps_max;
  q.b = mp.b;
  q.inv_eff_spp = mp.inv_eff_spp;
  q.alias_prob = mp.alias_prob;
  q.alias_idx = mp.alias_idx;
  q.smp = w->mlt_smp.as<int4>();
  q.chain = w->mlt_chain.as<float4>();
  q.X = mp.X;
  q.film = mp.film;
  q.accepted = mp.accepted;
  cudaStream_t st = ctx->stream;
  cudaMemcpyAsync(w->params.ptr, &p, sizeof(p), cudaMemcpyHostToDevice, st);
  cudaMemsetAsync(w->counters.ptr, 0, bn::kCntSize * sizeof(int), st);
  cudaMemsetAsync(w->meta.ptr, 0, static_cast<size_t>(pool) * sizeof(int4), st);  // every chain unstarted
  // (checking the loop condition every 4 or 16 iterations instead of every one measured slower:
  // 499 and 510 against 450 ms)
  for (int it = 0; it < p.max_iters + 1; ++it) {
    if ((e = bn::wf_launch_iteration(w->params.as<bn::WfParams>(), w->shape, false, st, &w->fork)) != cudaSuccess)
      return ctx->cuda_fail(e, "wavefront chain iteration launch");
    int again = 0;
    cudaMemcpyAsync(&again, w->counters.as<int>() + bn::kCntAgain, sizeof(int), cudaMemcpyDeviceToHost, st);
    if ((e = cudaStreamSynchronize(st)) != cudaSuccess) return ctx->cuda_fail(e, "wavefront chain iteration");
    if (!again) break;
  }
  int counters[bn::kCntSize];
  e = cudaMemcpyAsync(counters, w->counters.ptr, sizeof(counters), cudaMemcpyDeviceToHost, st);
  if (e == cudaSuccess) e = cudaStreamSynchronize(st);
  if (e != cudaSuccess) return ctx->cuda_fail(e, "wavefront chains");
  *iters = counters[bn::kCntIter];
  return BN_OK;
}

}  // namespace

namespace bnc {

int render_pssmlt_wavefront(bn_context* ctx, const bn_render_desc* d, const bn::MltParams& mp, int* launches) {
  int iters = 0;
  const int rc = run_mlt(ctx, state(ctx), d, mp, &iters);
  *launches = 5 * iters;
  return rc;
}

int render_wavefront(bn_context* ctx, const bn_render_desc* d, const std::vector<bn::DevView>& views) {
  WfState* w = state(ctx);
  long long pixels = 0, total = 0;
  for (const auto& v : views) {
    pixels += static_cast<long long>(v.width) * v.height;
    total += static_cast<long long>(v.width) * v.height * d->spp;
  }
  const bool use_graph = !(d->flags & BN_RENDER_NO_GRAPH);
  int pool = d->queue_capacity, cap = d->block_size;  // block_size doubles as the blocks/SM cap
  int refill = 16;
  if (pool <= 0 && cap <= 0 && !(d->flags & BN_RENDER_COUNT)) {  // a counting render is a one-off: no tuning
    const int wt = (d->flags & BN_RENDER_WATERTIGHT) ? 1 : 0;
    if (w->tuned_generation[wt] != ctx->scene_generation) {
      // autotune on a truncated render of the same views: pool size (the queue width) x
      // blocks-per-SM cap, then the lanes a traversal warp refills at (the width of its batch)
      const int pools[7] = {1 << 20, 1 << 21, 1 << 22, 1 << 23, 1 << 24, 1 << 25, 1 << 26};
      const int caps[2] = {0, 2};
      const int refills[3] = {16, 12, 20};
      const long long sample = std::min<long long>(total, 128LL << 20);  // two fills of the largest pool
      float best = 1e30f;
      w->tuned_refill[wt] = 16;
      for (int pi : pools)
        for (int ci : caps) {
          // a pool larger than the paths it would hold only adds slots to scan
          if (pi > (1 << 20) && pi > sample) continue;
          float ms = 0.f;
          const int rc = run(ctx, w, d, pixels, sample, static_cast<int>(views.size()), pi, ci, 16, use_graph, &ms);
          if (rc) return rc;
          if (ms < best) {
            best = ms;
            w->tuned_pool[wt] = pi;
            w->tuned_cap[wt] = ci;
          }
        }
      for (int k = 1; k < 3; ++k) {
        float ms = 0.f;
        const int rc = run(ctx, w, d, pixels, sample, static_cast<int>(views.size()), w->tuned_pool[wt],
                           w->tuned_cap[wt], refills[k], use_graph, &ms);
        if (rc) return rc;
        if (ms < best) {
          best = ms;
          w->tuned_refill[wt] = refills[k];
        }
      }
      w->tuned_generation[wt] = ctx->scene_generation;
    }
    pool = w->tuned_pool[wt];
    cap = w->tuned_cap[wt];
    refill = w->tuned_refill[wt];
  }
  if (pool <= 0) pool = 1 << 20;
  pool = std::max(pool, 1024);
  const int rc = run(ctx, w, d, pixels, total, static_cast<int>(views.size()), pool, cap, refill, use_graph, nullptr);
  if (rc) return rc;
  ctx->stats.paths += static_cast<uint64_t>(total);
  return BN_OK;
}

}  // namespace bnc
