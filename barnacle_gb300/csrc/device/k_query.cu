// Query kernels: batched closest/any-hit tracing (the bit-exact parity path), batched BSDF
// eval/sample, and the hash-sampler stream.
#include "dev_shading.cuh"
#include "launch.hpp"

namespace bn {
namespace {

__device__ __forceinline__ void warp_add_counters(DevCounters* c, unsigned long long rays, const TraceCounters& tc) {
  // warp-aggregated: one atomic per warp per counter
  for (int o = 16; o > 0; o >>= 1) {
    rays += __shfl_down_sync(0xffffffffu, rays, o);
  }
  unsigned long long nn = tc.nodes, tt = tc.tris, ii = tc.insts;
  for (int o = 16; o > 0; o >>= 1) {
    nn += __shfl_down_sync(0xffffffffu, nn, o);
    tt += __shfl_down_sync(0xffffffffu, tt, o);
    ii += __shfl_down_sync(0xffffffffu, ii, o);
  }
  if ((threadIdx.x & 31) == 0) {
    atomicAdd(&c->rays, rays);
    atomicAdd(&c->nodes, nn);
    atomicAdd(&c->tris, tt);
    atomicAdd(&c->insts, ii);
  }
}

template <bool kAny, bool kWT, int kWalk>
__global__ void __launch_bounds__(128) k_trace(DevScene s, const bn_ray* __restrict__ rays, bn_hit* __restrict__ hits,
                                               long long n, DevCounters* counters) {
  constexpr bool kCount = kWalk == kWalkCount;
  const long long i = static_cast<long long>(blockIdx.x) * blockDim.x + threadIdx.x;
  TraceCounters tc{0, 0, 0};
  unsigned long long nr = 0;
  if (i < n) {
    const bn_ray r = rays[i];
    Ray ray;
    ray.o = mk(r.origin[0], r.origin[1], r.origin[2]);
    ray.d = mk(r.direction[0], r.direction[1], r.direction[2]);
    bn_hit out{};
    nr = 1;
    if (kAny) {
      const bool h = trace_any<kWT, kWalk>(s, ray, r.t_max, &tc);
      out.instance = h ? 0 : -1;
      out.t = r.t_max;
      out.primitive = -1;
    } else {
      HitRec h;
      if (trace_closest<kWT, kWalk>(s, ray, r.t_max, &h, &tc)) {
        const Interaction it = make_interaction(s, ray, h);
        out.t = h.t; out.u = it.u; out.v = it.v;
        out.instance = h.inst; out.primitive = h.tri;
        out.normal[0] = it.f.n.x; out.normal[1] = it.f.n.y; out.normal[2] = it.f.n.z;
        out.position[0] = it.p.x; out.position[1] = it.p.y; out.position[2] = it.p.z;
      } else {
        out.t = r.t_max;
        out.instance = -1;
        out.primitive = -1;
      }
    }
    hits[i] = out;
  }
  if (kCount) warp_add_counters(counters, nr, tc);
}

template <bool kAny>
cudaError_t launch_trace_t(const DevScene& s, const bn_ray* rays, bn_hit* hits, long long n, unsigned flags,
                           DevCounters* counters, cudaStream_t st) {
  const int bs = 128;
  const long long grid = (n + bs - 1) / bs;
  dispatch_walk<true>(s, flags & BN_TRACE_WATERTIGHT, flags & BN_TRACE_COUNT, [&](auto wt, auto walk) {
    k_trace<kAny, decltype(wt)::value, decltype(walk)::value><<<grid, bs, 0, st>>>(s, rays, hits, n, counters);
  });
  return cudaGetLastError();
}

__global__ void k_bsdf(DevScene s, const bn_bsdf_query* __restrict__ q, bn_bsdf_result* __restrict__ out, long long n,
                       bool sample) {
  const long long i = static_cast<long long>(blockIdx.x) * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const bn_bsdf_query a = q[i];
  bn_bsdf_result r{};
  if (a.material < 0 || a.material >= s.n_mats) {
    flag_error(s, BN_DEVERR_BAD_INDEX);
    out[i] = r;
    return;
  }
  const DevMaterial m = s.mats[a.material];
  const V3 wo = mk(a.wo[0], a.wo[1], a.wo[2]);
  if (sample) {
    const BsdfSample bs = bsdf_sample(m, wo, a.u_lobe, a.u_bsdf[0], a.u_bsdf[1]);
    r.bsdf[0] = bs.f.x; r.bsdf[1] = bs.f.y; r.bsdf[2] = bs.f.z; r.pdf = bs.pdf;
    r.wi[0] = bs.wi.x; r.wi[1] = bs.wi.y; r.wi[2] = bs.wi.z;
  } else {
    const BsdfEval e = bsdf_eval(m, wo, mk(a.wi[0], a.wi[1], a.wi[2]));
    r.bsdf[0] = e.f.x; r.bsdf[1] = e.f.y; r.bsdf[2] = e.f.z; r.pdf = e.pdf;
    r.wi[0] = a.wi[0]; r.wi[1] = a.wi[1]; r.wi[2] = a.wi[2];
  }
  out[i] = r;
}

__global__ void k_sampler_stream(const uint32_t* __restrict__ seeds, long long n_streams, int n_draws, float* __restrict__ out) {
  const long long i = static_cast<long long>(blockIdx.x) * blockDim.x + threadIdx.x;
  if (i >= n_streams) return;
  IndepSampler smp{xxhash32_three(seeds[3 * i], seeds[3 * i + 1], seeds[3 * i + 2])};
  for (int k = 0; k < n_draws; ++k) out[i * n_draws + k] = smp.next();
}

}  // namespace

cudaError_t launch_trace(const DevScene& s, const bn_ray* rays, bn_hit* hits, long long n, unsigned flags,
                         DevCounters* counters, cudaStream_t st) {
  if (n <= 0) return cudaSuccess;
  if (flags & BN_TRACE_ANY) return launch_trace_t<true>(s, rays, hits, n, flags, counters, st);
  return launch_trace_t<false>(s, rays, hits, n, flags, counters, st);
}

cudaError_t launch_bsdf(const DevScene& s, const bn_bsdf_query* q, bn_bsdf_result* out, long long n, bool sample,
                        cudaStream_t st) {
  if (n <= 0) return cudaSuccess;
  k_bsdf<<<(n + 127) / 128, 128, 0, st>>>(s, q, out, n, sample);
  return cudaGetLastError();
}

cudaError_t launch_sampler_stream(const uint32_t* seeds, long long n_streams, int n_draws, float* out, cudaStream_t st) {
  if (n_streams <= 0) return cudaSuccess;
  k_sampler_stream<<<(n_streams + 127) / 128, 128, 0, st>>>(seeds, n_streams, n_draws, out);
  return cudaGetLastError();
}

}  // namespace bn
