// Differentiable materials: a forward render whose PBR slots and light scales come from a
// parameter vector, and the path-replay adjoint of an L2 image loss (no counterpart in the
// reference; the path arithmetic is PathTracingIntegrator.Li, PathTracing.fs:14-81).
//
// Detached sampling: every sampling decision (BSDF direction and pdf, lobe choice, MIS weights,
// Russian roulette) is made with `sparams`; only BSDF values and emission use `params`.  With
// sparams == params this is the ordinary estimator.  The estimator is then a smooth function of
// params with the path fixed, and its exact derivative is what the backward pass computes:
//   backward = replay each path (same random stream, same rays) knowing its total radiance L;
//   at a vertex with sampled value f (per channel) every later contribution is proportional to
//   f, so d(later)/dtheta = L_remaining * (df/dtheta) / f; the vertex's own emission and NEE terms
//   are differentiated directly.  Nothing per vertex is stored, and the cost is one more pass.
// Gradients: lanes holding the same material slot are grouped (__match_any_sync), their FP32
// values summed by shuffles, and one FP64 atomicAdd per group and parameter lands in HBM.
#include "adjoint.hpp"
#include "launch.hpp"
#include "dev_shading.cuh"

namespace bn {
namespace {

__device__ __forceinline__ DevMaterial slot_material(const float* prm, int slot) {
  DevMaterial m;
  m.type = kMatPBR;
  m.base[0] = prm[kSlotParams * slot];
  m.base[1] = prm[kSlotParams * slot + 1];
  m.base[2] = prm[kSlotParams * slot + 2];
  const float r = prm[kSlotParams * slot + 3];
  const float a = __fmul_rn(r, r);
  m.alpha = a > 1e-3f ? a : 1e-3f;  // PBR.fs:106
  m.metallic = fminf(fmaxf(prm[kSlotParams * slot + 4], 0.f), 1.f);
  m.roughness = r;
  m.ior = 1.5f;
  return m;
}

__device__ __forceinline__ float light_scale(const AdjParams& p, const float* prm, int light) {
  const int slot = p.emissive_base + light;
  return (light >= 0 && slot < p.n_slots) ? prm[kSlotParams * slot + 5] : 1.f;
}

// d f / d (albedo, roughness, metallic) of the PBR value (per channel), f itself from pbr_eval
struct PbrGrad {
  V3 d_base;   // d f_c / d base_c
  V3 d_rough;
  V3 d_metal;
};
__device__ __forceinline__ PbrGrad pbr_grad(const DevMaterial& m, float rough_param, float metal_param, V3 wo, V3 wi) {
  PbrGrad g;
  const float a = m.alpha, a2 = a * a;
  const V3 h = mk(wo.x + wi.x, wo.y + wi.y, wo.z + wi.z);
  const float hl = sqrtf(h.x * h.x + h.y * h.y + h.z * h.z);
  const V3 wh = mk(h.x / hl, h.y / hl, h.z / hl);
  const float s2 = wh.x * wh.x + wh.y * wh.y, c2h = wh.z * wh.z;
  const float k = s2 + a2 * c2h;
  const float D = a2 / (kPi * k * k);
  const float dD = 2.f * a / (kPi * k * k * k) * (s2 - a2 * c2h);
  auto lam = [&](V3 w, float* dl) {
    const float sn = w.x * w.x + w.y * w.y;
    if (sn == 0.f) { *dl = 0.f; return 0.f; }
    const float t2 = sn / (w.z * w.z);
    const float q = sqrtf(1.f + a2 * t2);
    *dl = a * t2 / (2.f * q);
    return (q - 1.f) * 0.5f;
  };
  float dlo, dli;
  const float lo = lam(wo, &dlo), li = lam(wi, &dli);
  const float G = 1.f / (1.f + lo + li);
  const float dG = -G * G * (dlo + dli);
  const float inv4 = 1.f / (4.f * fabsf(wo.z));
  const float spec = D * G * inv4;
  const float dspec = (dD * G + D * dG) * inv4;
  const float coh = wo.x * wh.x + wo.y * wh.y + wo.z * wh.z;
  const float c = 1.f - coh, c5 = c * c * c * c * c;
  const float F = 0.04f + 0.96f * c5;
  const float mt = m.metallic;
  const float dmt = (metal_param > 0.f && metal_param < 1.f) ? 1.f : 0.f;
  const float dalpha = (rough_param * rough_param > 1e-3f) ? 2.f * rough_param : 0.f;
  const float cw = fabsf(wi.z) / kPi;
  const float base[3] = {m.base[0], m.base[1], m.base[2]};
  float db[3], dr[3], dm[3];
  for (int ch = 0; ch < 3; ++ch) {
    const float fc = base[ch] + (1.f - base[ch]) * c5;
    const float diff = base[ch] * cw;
    db[ch] = cw * (1.f - F) * (1.f - mt) + spec * (1.f - c5) * mt;
    dr[ch] = dspec * (F * (1.f - mt) + fc * mt) * dalpha;
    dm[ch] = (-(diff * (1.f - F) + spec * F) + spec * fc) * dmt;
  }
  g.d_base = mk(db[0], db[1], db[2]);
  g.d_rough = mk(dr[0], dr[1], dr[2]);
  g.d_metal = mk(dm[0], dm[1], dm[2]);
  return g;
}

__device__ __forceinline__ float dot3(V3 a, V3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }

// warp-aggregated gradient add: lanes with the same slot sum in FP32, one FP64 atomic per group
__device__ __forceinline__ void grad_add(double* grad, int slot, const float g[kSlotParams]) {
  const unsigned act = __activemask();
  const unsigned peers = __match_any_sync(act, slot);
  if (slot < 0) return;
  const int lane = threadIdx.x & 31;
  const int leader = __ffs(peers) - 1;
  for (int k = 0; k < kSlotParams; ++k) {
    float sum = 0.f;
    for (unsigned m = peers; m; m &= m - 1) sum += __shfl_sync(peers, g[k], __ffs(m) - 1);
    if (lane == leader && sum != 0.f) atomicAdd(grad + kSlotParams * slot + k, static_cast<double>(sum));
  }
}

// Li with value/sampling parameters; kGrad replays the path with its known total radiance
template <bool kGrad, int kWalk>
__device__ V3 li_adj(const AdjParams& p, Ray ray, IndepSampler& smp, V3 L_total, V3 delta) {
  const DevScene& s = p.scene;
  V3 L = mk(0.f, 0.f, 0.f), beta = mk(1.f, 1.f, 1.f), beta_s = mk(1.f, 1.f, 1.f);
  V3 L_rem = L_total;
  float pdf_bsdf = 0.f;
  int depth = 0;
  TraceCounters tc;
  while (depth < p.max_depth) {
    HitRec h;
    if (!trace_closest<false, kWalk, true>(s, ray, CUDART_INF_F, &h, &tc)) break;
    const Interaction it = make_interaction(s, ray, h);
    const DevInstance* I = s.inst + it.inst;
    const int light = __ldg(&I->light);
    if (light >= 0) {
      V3 le;
      float pdf_l;
      eval_light(s, ray.o, it, &le, &pdf_l);
      const float mis = depth == 0 ? 1.f : __fmul_rn(pdf_bsdf, __frcp_rn(__fadd_rn(pdf_l, pdf_bsdf)));
      const V3 le_v = scale(light_scale(p, p.params, light), le);
      L = fma3(beta, scale(mis, le_v), L);
      if (kGrad) {
        const V3 e = mul(beta, scale(mis, le_v));
        L_rem = sub(L_rem, e);
        float g[kSlotParams] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
        g[5] = dot3(delta, mul(beta, scale(mis, le)));
        const int slot = p.emissive_base + light < p.n_slots ? p.emissive_base + light : -1;
        grad_add(p.grad, slot, g);
      }
    }
    const int mat = hit_material(s, it);
    if (mat < 0) break;
    const float u_sel = smp.next(), ulx = smp.next(), uly = smp.next();
    const bool slotted = mat < p.emissive_base && mat < p.n_slots;
    const DevMaterial ms = slotted ? slot_material(p.sparams, mat) : s.mats[mat];
    const DevMaterial mv = slotted ? slot_material(p.params, mat) : ms;
    const V3 wo_w = neg(ray.d);
    const V3 wo = to_local(it.f, wo_w);
    const LightSample ls = sample_light(s, it.p, u_sel, ulx, uly);
    const float dist = length(sub(ls.p, it.p));
    if (ls.pdf != 0.f) {
      Ray sh;
      sh.o = it.p;
      sh.d = ls.wi;
      if (!trace_any<false, kWalk, true>(s, sh, __fsub_rn(dist, 1e-3f), &tc)) {
        const V3 wi = to_local(it.f, ls.wi);
        const BsdfEval bes = bsdf_eval(ms, wo, wi);
        const BsdfEval bev = slotted ? bsdf_eval(mv, wo, wi) : bes;
        const float r = __frcp_rn(__fadd_rn(bes.pdf, ls.pdf));
        const V3 le_v = scale(light_scale(p, p.params, ls.light), ls.L);
        const V3 a = mul(beta, bev.f);
        const V3 b = scale(r, le_v);
        L = fma3(a, b, L);
        if (kGrad) {
          L_rem = sub(L_rem, mul(a, b));
          if (slotted) {
            const PbrGrad dg = pbr_grad(mv, p.params[kSlotParams * mat + 3], p.params[kSlotParams * mat + 4], wo, wi);
            const V3 w = mul(delta, mul(beta, b));
            float g[kSlotParams] = {w.x * dg.d_base.x, w.y * dg.d_base.y, w.z * dg.d_base.z, dot3(w, dg.d_rough),
                                    dot3(w, dg.d_metal), 0.f};
            grad_add(p.grad, mat, g);
          }
          const int lslot = p.emissive_base + ls.light < p.n_slots ? p.emissive_base + ls.light : -1;
          float gl[kSlotParams] = {0.f, 0.f, 0.f, 0.f, 0.f, dot3(delta, mul(a, scale(r, ls.L)))};
          grad_add(p.grad, lslot, gl);
        }
      }
    }
    const float u_lobe = smp.next(), ubx = smp.next(), uby = smp.next();
    const BsdfSample bs = bsdf_sample(ms, wo, u_lobe, ubx, uby);
    if (bs.pdf == 0.f) break;
    const V3 fv = slotted ? bsdf_eval(mv, wo, bs.wi).f : bs.f;
    if (kGrad && slotted) {
      const PbrGrad dg = pbr_grad(mv, p.params[kSlotParams * mat + 3], p.params[kSlotParams * mat + 4], wo, bs.wi);
      // every later contribution carries fv per channel: d/dtheta = L_rem * dfv / fv
      const V3 w = mk(fv.x != 0.f ? delta.x * L_rem.x / fv.x : 0.f, fv.y != 0.f ? delta.y * L_rem.y / fv.y : 0.f,
                      fv.z != 0.f ? delta.z * L_rem.z / fv.z : 0.f);
      float g[kSlotParams] = {w.x * dg.d_base.x, w.y * dg.d_base.y, w.z * dg.d_base.z, dot3(w, dg.d_rough),
                              dot3(w, dg.d_metal), 0.f};
      grad_add(p.grad, mat, g);
    }
    pdf_bsdf = bs.pdf;
    ray.o = it.p;
    ray.d = to_world(it.f, bs.wi);
    beta = scale(__frcp_rn(bs.pdf), mul(beta, fv));
    beta_s = scale(__frcp_rn(bs.pdf), mul(beta_s, bs.f));
    if (depth >= p.rr_depth) {
      const float q = fminf(1.f, fmaxf(beta_s.x, fmaxf(beta_s.y, beta_s.z)));
      if (smp.next() < q) {
        beta = scale(__frcp_rn(q), beta);
        beta_s = scale(__frcp_rn(q), beta_s);
      } else {
        break;
      }
    }
    depth++;
  }
  return L;
}

__device__ __forceinline__ void path_pixel(const AdjParams& p, long long i, int* x, int* y, int* sid) {
  const long long npix = p.n_pixels;
  *sid = static_cast<int>(i / npix);
  const long long pix = i - *sid * npix;
  *x = static_cast<int>(pix % p.view->width);
  *y = static_cast<int>(pix / p.view->width);
}

__device__ __forceinline__ Ray adj_camera(const AdjParams& p, int x, int y, int sid, IndepSampler* smp) {
  *smp = IndepSampler{xxhash32_three(static_cast<uint32_t>(x), static_cast<uint32_t>(y),
                                     static_cast<uint32_t>(p.frame_id * p.spp + sid))};
  const float upx = smp->next(), upy = smp->next();
  const float ulx = smp->next(), uly = smp->next();
  return camera_ray(*p.view, x, y, upx, upy, ulx, uly);
}

template <int kWalk>
__global__ void __launch_bounds__(128) k_adj_forward(AdjParams p) {
  const long long i = static_cast<long long>(blockIdx.x) * blockDim.x + threadIdx.x;
  if (i >= p.n_pixels * p.spp) return;
  int x, y, sid;
  path_pixel(p, i, &x, &y, &sid);
  IndepSampler smp;
  const Ray ray = adj_camera(p, x, y, sid, &smp);
  const V3 L = li_adj<false, kWalk>(p, ray, smp, mk(0.f, 0.f, 0.f), mk(0.f, 0.f, 0.f));
  p.path_L[i] = make_float4(L.x, L.y, L.z, 0.f);
}

// per pixel: fma(1/spp, L_s, acc) in sample order (RenderTile, Base/Integrator.fs:34-44)
__global__ void k_adj_image(AdjParams p) {
  const long long pix = static_cast<long long>(blockIdx.x) * blockDim.x + threadIdx.x;
  if (pix >= p.n_pixels) return;
  const float inv = __frcp_rn(static_cast<float>(p.spp));
  V3 acc = mk(0.f, 0.f, 0.f);
  for (int s = 0; s < p.spp; ++s) {
    const float4 L = p.path_L[s * p.n_pixels + pix];
    acc = fma3(mk(inv, inv, inv), mk(L.x, L.y, L.z), acc);
  }
  const int W = p.view->width, H = p.view->height;
  const int x = static_cast<int>(pix % W), y = static_cast<int>(pix / W);
  const long long o = static_cast<long long>(H - y - 1) * W + x;
  p.image[3 * o] = acc.x;
  p.image[3 * o + 1] = acc.y;
  p.image[3 * o + 2] = acc.z;
}

// 0.5 * sum (image - target)^2, block reduction in double
__global__ void k_adj_loss(AdjParams p) {
  __shared__ double red[256];
  double v = 0.0;
  for (long long i = static_cast<long long>(blockIdx.x) * blockDim.x + threadIdx.x; i < 3 * p.n_pixels;
       i += static_cast<long long>(gridDim.x) * blockDim.x) {
    const double d = static_cast<double>(p.image[i]) - p.target[i];
    v += 0.5 * d * d;
  }
  red[threadIdx.x] = v;
  __syncthreads();
  for (int s = blockDim.x / 2; s > 0; s >>= 1) {
    if (threadIdx.x < s) red[threadIdx.x] += red[threadIdx.x + s];
    __syncthreads();
  }
  if (threadIdx.x == 0) atomicAdd(p.loss, red[0]);
}

template <int kWalk>
__global__ void __launch_bounds__(128) k_adj_backward(AdjParams p) {
  const long long i = static_cast<long long>(blockIdx.x) * blockDim.x + threadIdx.x;
  if (i >= p.n_pixels * p.spp) return;
  int x, y, sid;
  path_pixel(p, i, &x, &y, &sid);
  const int W = p.view->width, H = p.view->height;
  const long long o = static_cast<long long>(H - y - 1) * W + x;
  // d loss / d L_path = (image - target) / spp per channel
  const float inv = __frcp_rn(static_cast<float>(p.spp));
  const V3 delta = mk((p.image[3 * o] - p.target[3 * o]) * inv, (p.image[3 * o + 1] - p.target[3 * o + 1]) * inv,
                      (p.image[3 * o + 2] - p.target[3 * o + 2]) * inv);
  const float4 Lt = p.path_L[i];
  IndepSampler smp;
  const Ray ray = adj_camera(p, x, y, sid, &smp);
  li_adj<true, kWalk>(p, ray, smp, mk(Lt.x, Lt.y, Lt.z), delta);
}

}  // namespace

cudaError_t launch_adj_forward(const AdjParams& p, cudaStream_t st) {
  const long long n = p.n_pixels * p.spp;
  dispatch_walk<false>(p.scene, false, false, [&](auto, auto walk) {
    k_adj_forward<decltype(walk)::value><<<(n + 127) / 128, 128, 0, st>>>(p);
  });
  return cudaGetLastError();
}
cudaError_t launch_adj_image(const AdjParams& p, cudaStream_t st) {
  k_adj_image<<<(p.n_pixels + 255) / 256, 256, 0, st>>>(p);
  return cudaGetLastError();
}
cudaError_t launch_adj_loss(const AdjParams& p, cudaStream_t st) {
  k_adj_loss<<<152 * 4, 256, 0, st>>>(p);
  return cudaGetLastError();
}
cudaError_t launch_adj_backward(const AdjParams& p, cudaStream_t st) {
  const long long n = p.n_pixels * p.spp;
  dispatch_walk<false>(p.scene, false, false, [&](auto, auto walk) {
    k_adj_backward<decltype(walk)::value><<<(n + 127) / 128, 128, 0, st>>>(p);
  });
  return cudaGetLastError();
}

}  // namespace bn
