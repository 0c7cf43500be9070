// PSSMLTIntegrator.Render (Extensions/Integrator/PSSMLT.fs:379-414): bootstrap, b, start table,
// chains.
#include <string>
#include <vector>

#include "../device/pssmlt.hpp"
#include "context.hpp"

namespace {

// Vose table over the bootstrap luminances (the proportional start distribution the reference's
// AliasTable intends; used with BN_RENDER_FIXED_ALIAS)
void vose(const std::vector<float>& w, std::vector<float>* prob, std::vector<int>* alias) {
  const size_t n = w.size();
  double sum = 0.0;
  for (float x : w) sum += x > 0.f ? x : 0.f;
  prob->assign(n, 1.f);
  alias->resize(n);
  std::vector<double> scaled(n);
  std::vector<size_t> small, large;
  for (size_t i = 0; i < n; ++i) {
    (*alias)[i] = static_cast<int>(i);
    scaled[i] = sum > 0 ? (w[i] > 0.f ? w[i] : 0.f) * n / sum : 1.0;
    (scaled[i] < 1.0 ? small : large).push_back(i);
  }
  while (!small.empty() && !large.empty()) {
    const size_t s = small.back(), l = large.back();
    small.pop_back();
    (*prob)[s] = static_cast<float>(scaled[s]);
    (*alias)[s] = static_cast<int>(l);
    scaled[l] = (scaled[l] + scaled[s]) - 1.0;
    if (scaled[l] < 1.0) {
      large.pop_back();
      small.push_back(l);
    }
  }
}

}  // namespace

namespace bnc {

int render_pssmlt(bn_context* ctx, const bn_render_desc* d, const std::vector<bn::DevView>& views) {
  if (views.size() != 1) return ctx->fail(BN_ERR_UNSUPPORTED, "PSSMLT renders one view per call");
  if (d->n_bootstrap <= 0 || d->n_chains <= 0) return ctx->fail(BN_ERR_INVALID_ARG, "PSSMLT needs bootstrap paths and chains");
  if (d->large_step_prob < 0.f || d->large_step_prob > 1.f) return ctx->fail(BN_ERR_INVALID_ARG, "large-step probability outside [0, 1]");
  if (d->mutation == BN_MUTATION_KELEMEN && !(d->eps_min > 0.f && d->eps_max > 0.f))
    return ctx->fail(BN_ERR_INVALID_ARG, "Kelemen mutation needs positive eps_min and eps_max");
  const bn::DevView& v = views[0];
  const long long pixels = static_cast<long long>(v.width) * v.height;
  const int dims = 4 + 7 * d->max_depth;
  if (d->mode == BN_MODE_WAVEFRONT && dims >= 4096)
    return ctx->fail(BN_ERR_UNSUPPORTED, "wavefront PSSMLT supports max_depth up to 584");
  const long long mpc_ll = (static_cast<long long>(d->spp) * pixels + d->n_chains - 1) / d->n_chains;
  if (mpc_ll > (1LL << 30)) return ctx->fail(BN_ERR_INVALID_ARG, "too many mutations per chain");
  cudaError_t e;
  cudaStream_t st = ctx->stream;
  if ((e = ctx->mlt_boot.reserve(static_cast<size_t>(d->n_bootstrap) * sizeof(float))) != cudaSuccess)
    return ctx->cuda_fail(e, "bootstrap weights");
  if ((e = ctx->mlt_state.reserve(static_cast<size_t>(dims) * d->n_chains * sizeof(float4))) != cudaSuccess)
    return ctx->cuda_fail(e, "primary-sample vectors");
  if ((e = ctx->mlt_chain.reserve(256 + 2 * static_cast<size_t>(d->n_bootstrap) * sizeof(float))) != cudaSuccess)
    return ctx->cuda_fail(e, "chain tables");
  bn::MltParams p{};
  p.scene = ctx->scene;
  p.view = ctx->views.as<bn::DevView>();
  p.n_bootstrap = d->n_bootstrap;
  p.n_chains = d->n_chains;
  p.max_depth = d->max_depth;
  p.rr_depth = d->rr_depth;
  p.frame_id = d->frame_id;
  p.n_dims = dims;
  p.mutations_per_chain = static_cast<int>(mpc_ll);
  p.kelemen = d->mutation == BN_MUTATION_KELEMEN;
  p.large_step_prob = d->large_step_prob;
  p.sigma = d->sigma;
  p.eps_min = d->eps_min;
  p.eps_max = d->eps_max;
  p.watertight = d->flags & BN_RENDER_WATERTIGHT;
  p.weights = ctx->mlt_boot.as<float>();
  p.X = ctx->mlt_state.as<float4>();  // [dimension][chain] (lockstep) or [chain][dimension] (wavefront)
  p.film = ctx->film.as<float>();
  p.accepted = reinterpret_cast<unsigned long long*>(ctx->mlt_chain.ptr);
  cudaMemsetAsync(ctx->film.ptr, 0, static_cast<size_t>(pixels) * 3 * sizeof(float), st);
  cudaMemsetAsync(ctx->mlt_chain.ptr, 0, 256, st);
  cudaEventRecord(ctx->ev0, st);
  if ((e = bn::launch_mlt_bootstrap(p, st)) != cudaSuccess) return ctx->cuda_fail(e, "bootstrap launch");
  // b = Array.average of the float32 weights: a float32 sum in order, then / n (PSSMLT.fs:394)
  std::vector<float> w(d->n_bootstrap);
  e = cudaMemcpyAsync(w.data(), p.weights, w.size() * sizeof(float), cudaMemcpyDeviceToHost, st);
  if (e == cudaSuccess) e = cudaStreamSynchronize(st);
  if (e != cudaSuccess) return ctx->cuda_fail(e, "bootstrap");
  float sum = 0.f;
  for (float x : w) sum = sum + x;
  const float b = sum / static_cast<float>(d->n_bootstrap);
  ctx->stats.bootstrap_b = b;
  ctx->stats.proposed += static_cast<uint64_t>(mpc_ll) * d->n_chains;
  int launches = 1;
  if (b != 0.f) {  // "all bootstrap samples are zero": nothing is rendered (:396-397)
    p.b = b;
    // ReciprocalEstimate(mutationPerChain * NChains / (W * H)), float32 operations in order
    p.inv_eff_spp = 1.f / ((static_cast<float>(mpc_ll) * static_cast<float>(d->n_chains)) / static_cast<float>(pixels));
    if (d->flags & BN_RENDER_FIXED_ALIAS) {
      std::vector<float> prob;
      std::vector<int> alias;
      vose(w, &prob, &alias);
      float* dprob = reinterpret_cast<float*>(static_cast<char*>(ctx->mlt_chain.ptr) + 256);
      int* didx = reinterpret_cast<int*>(dprob + d->n_bootstrap);
      cudaMemcpyAsync(dprob, prob.data(), prob.size() * sizeof(float), cudaMemcpyHostToDevice, st);
      cudaMemcpyAsync(didx, alias.data(), alias.size() * sizeof(int), cudaMemcpyHostToDevice, st);
      p.alias_prob = dprob;
      p.alias_idx = didx;
    }
    cudaEventRecord(ctx->ev1, st);
    if (d->mode == BN_MODE_WAVEFRONT) {
      // the chains compacted every bounce (wavefront.cu, k_mlt_wavefront.cu)
      int wl = 0;
      const int rc = bnc::render_pssmlt_wavefront(ctx, d, p, &wl);
      if (rc) return rc;
      launches += wl;
    } else {
      if ((e = bn::launch_mlt_chains(p, st)) != cudaSuccess) return ctx->cuda_fail(e, "chain launch");
      ++launches;
    }
  } else {
    cudaEventRecord(ctx->ev1, st);
  }
  cudaEventRecord(ctx->ev2, st);
  if ((e = cudaEventSynchronize(ctx->ev2)) != cudaSuccess) return ctx->cuda_fail(e, "PSSMLT");
  unsigned long long acc = 0;
  cudaMemcpy(&acc, p.accepted, sizeof(acc), cudaMemcpyDeviceToHost);
  float ms_chain = 0.f, ms_all = 0.f;
  cudaEventElapsedTime(&ms_chain, ctx->ev1, ctx->ev2);
  cudaEventElapsedTime(&ms_all, ctx->ev0, ctx->ev2);
  ctx->stats.accepted += acc;
  ctx->stats.paths += static_cast<uint64_t>(d->n_bootstrap) + (b != 0.f ? static_cast<uint64_t>(mpc_ll + 1) * d->n_chains : 0);
  ctx->stats.last_kernel_ms = ms_all;
  ctx->stats.last_dominant_ms = ms_chain;
  ctx->stats.last_launches = launches;
  return BN_OK;
}

}  // namespace bnc
