// Shading on the device: the hash sampler, cameras, BSDFs, light sampling and the path-tracing
// bounce loop, each following the reference's arithmetic (file:line cited per function).
#pragma once
#include "dev_geometry.cuh"

namespace bn {

constexpr float kPi = 3.14159265f;  // MathF.PI

// ------------------------------------------------------------------ sampler (Util/Hash.fs)
__device__ __forceinline__ uint32_t rotl32(uint32_t x, int r) { return (x << r) | (x >> (32 - r)); }
__host__ __device__ __forceinline__ uint32_t xxhash32_two(uint32_t x, uint32_t y) {
  uint32_t h = y + 374761393u + x * 3266489917u;
  h = 668265263u * ((h << 17) | (h >> 15));
  h = 2246822519u * (h ^ (h >> 15));
  h = 3266489917u * (h ^ (h >> 13));
  return h ^ (h >> 16);
}
__host__ __device__ __forceinline__ uint32_t xxhash32_three(uint32_t x, uint32_t y, uint32_t z) {
  uint32_t h = z + 374761393u + x * 3266489917u;
  h = 668265263u * ((h << 17) | (h >> 15));
  h = h + y * 3266489917u;
  h = 668265263u * ((h << 17) | (h >> 15));
  h = 2246822519u * (h ^ (h >> 15));
  h = 3266489917u * (h ^ (h >> 13));
  return h ^ (h >> 16);
}
// Hash.LCG: a = 0x343fd, c = 0x269ec3, 23 mantissa bits -> [0, 1)
__device__ __forceinline__ float lcg_next(uint32_t& s) {
  s = 0x00269ec3u + s * 0x000343fdu;
  return __fsub_rn(__uint_as_float((s >> 9) | 0x3f800000u), 1.f);
}

// Sampler (Base/Sampler.fs:7-16): independent per-path stream
struct IndepSampler {
  uint32_t state;
  __device__ __forceinline__ float next() { return lcg_next(state); }
  template <int N>
  __device__ __forceinline__ void next_n(float* u) {
#pragma unroll
    for (int k = 0; k < N; ++k) u[k] = lcg_next(state);
  }
};

// ------------------------------------------------------------------ camera (Base/Camera.fs:12-20)
__device__ __forceinline__ void concentric_disk(float ux, float uy, float* dx, float* dy) {
  // ThinLensCamera.SampleDiskConcentric (Extensions/Camera/ThinLens.fs:12-24)
  const float x = __fsub_rn(__fmul_rn(ux, 2.f), 1.f), y = __fsub_rn(__fmul_rn(uy, 2.f), 1.f);
  if (x == 0.f || y == 0.f) { *dx = 0.f; *dy = 0.f; return; }
  float r, theta;
  if (fabsf(x) > fabsf(y)) {
    r = x;
    theta = __fmul_rn(kPi / 4.f, __fdiv_rn(y, x));
  } else {
    r = y;
    theta = __fsub_rn(kPi / 2.f, __fmul_rn(kPi / 4.f, __fdiv_rn(x, y)));
  }
  *dx = __fmul_rn(r, cosf(theta));
  *dy = __fmul_rn(r, sinf(theta));
}

// kSimple (here and below): a scene of Lambertian triangle meshes, the uniform light sampler and
// pinhole views only; the specialised code leaves the other branches out, which keeps a path
// loop small enough for the instruction cache.
template <bool kSimple = false>
__device__ __forceinline__ Ray camera_ray(const DevView& v, int x, int y, float upx, float upy, float ulx, float uly) {
  // PinholeCamera.GenerateRay (Pinhole.fs:12-27): ((ul + (x + u.x) du) + (y + u.y) dv), normalised
  const float a = __fadd_rn(static_cast<float>(x), upx), b = __fadd_rn(static_cast<float>(y), upy);
  const V3 pl = {__fadd_rn(__fadd_rn(v.ul[0], __fmul_rn(a, v.du[0])), __fmul_rn(b, v.dv[0])),
                 __fadd_rn(__fadd_rn(v.ul[1], __fmul_rn(a, v.du[1])), __fmul_rn(b, v.dv[1])),
                 __fadd_rn(__fadd_rn(v.ul[2], __fmul_rn(a, v.du[2])), __fmul_rn(b, v.dv[2]))};
  Ray r;
  r.o = mk(0.f, 0.f, 0.f);
  r.d = normalize(pl);
  if (!kSimple && v.cam_type == BN_CAM_THIN_LENS && v.aperture > 0.f) {
    // ThinLensCamera.GenerateRay (ThinLens.fs:26-35)
    float dx, dy;
    concentric_disk(ulx, uly, &dx, &dy);
    const V3 o = {__fadd_rn(0.f, __fmul_rn(v.aperture, dx)), __fadd_rn(0.f, __fmul_rn(v.aperture, dy)), __fadd_rn(0.f, 0.f)};
    const V3 focus = point_at(r, v.focus_distance);
    r.d = normalize(sub(focus, o));
    r.o = o;
  }
  // CameraBase.GeneratePrimaryRay: to world, renormalise, push forward
  Ray w;
  w.o = xf_point16(v.c2w, r.o);
  const V3 dw = xf_point16(v.c2w, r.d);
  w.d = normalize(sub(dw, mk(v.c2w[12], v.c2w[13], v.c2w[14])));
  w.o = point_at(w, v.push_forward);
  return w;
}

// ------------------------------------------------------------------ BSDFs (local frame)
struct BsdfEval {
  V3 f;      // "bsdf" = f * |cos theta_i|
  float pdf;
};
struct BsdfSample {
  V3 f;
  float pdf;
  V3 wi;
};

// Extensions/Material/PBR.fs:108-131
__device__ __forceinline__ float pbr_lambda(float alpha, V3 w) {
  const float sin2 = fmaf(w.x, w.x, __fmul_rn(w.y, w.y));
  if (sin2 == 0.f) return 0.f;
  const float tan2 = __fdiv_rn(sin2, __fmul_rn(w.z, w.z));
  const float a2t2 = __fmul_rn(__fmul_rn(alpha, alpha), tan2);
  return __fdiv_rn(__fadd_rn(-1.f, __fsqrt_rn(__fadd_rn(1.f, a2t2))), 2.f);
}
// GGX D (PBR.fs:115-118).  The reference's k = 1 + (a^2 - 1) cos^2 cancels for sharp lobes
// (relative error ~ eps / a^2 in FP32); k = sin^2 + a^2 cos^2 is the same quantity without the
// cancellation, which keeps D within 1e-5 of an FP64 evaluation.
__device__ __forceinline__ float pbr_d(float alpha, V3 wh) {
  const float a2 = __fmul_rn(alpha, alpha);
  const float k = fmaf(a2, __fmul_rn(wh.z, wh.z), fmaf(wh.x, wh.x, __fmul_rn(wh.y, wh.y)));
  return __fdiv_rn(a2, __fmul_rn(kPi, __fmul_rn(k, k)));
}
__device__ __forceinline__ BsdfEval pbr_eval(V3 base, float alpha, float metallic, V3 wo, V3 wi) {
  const V3 wh = normalize(add(wo, wi));
  const float d = pbr_d(alpha, wh);
  const float g = __fdiv_rn(1.f, __fadd_rn(__fadd_rn(1.f, pbr_lambda(alpha, wo)), pbr_lambda(alpha, wi)));
  const float spec = __fdiv_rn(__fmul_rn(d, g), __fmul_rn(4.f, fabsf(wo.z)));
  const float cos_oh = dot(wo, wh);
  const float c = __fsub_rn(1.f, cos_oh);
  const float c2 = __fmul_rn(c, c);
  const float c5 = __fmul_rn(__fmul_rn(c2, c2), c);
  const V3 fc = add(base, scale(c5, sub(mk(1.f, 1.f, 1.f), base)));  // conductor Schlick, F0 = base
  const V3 metal = scale(spec, fc);
  const float fd = __fadd_rn(0.04f, __fmul_rn(__fmul_rn(__fmul_rn(__fsub_rn(1.f, 0.04f), c2), c2), c));
  const V3 diffuse = divs(scale(fabsf(wi.z), base), kPi);
  const float om = __fsub_rn(1.f, fd), omm = __fsub_rn(1.f, metallic);
  const V3 inner = {fmaf(diffuse.x, om, __fmul_rn(spec, fd)), fmaf(diffuse.y, om, __fmul_rn(spec, fd)),
                    fmaf(diffuse.z, om, __fmul_rn(spec, fd))};
  BsdfEval e;
  e.f = {fmaf(inner.x, omm, __fmul_rn(metal.x, metallic)), fmaf(inner.y, omm, __fmul_rn(metal.y, metallic)),
         fmaf(inner.z, omm, __fmul_rn(metal.z, metallic))};
  const float ps = __fdiv_rn(__fmul_rn(d, fabsf(wh.z)), __fmul_rn(4.f, cos_oh));
  const float pd = __fdiv_rn(fabsf(wi.z), kPi);
  const float tmix = __fmul_rn(0.5f, omm);
  e.pdf = fmaf(ps, __fsub_rn(1.f, tmix), __fmul_rn(pd, tmix));
  return e;
}

template <bool kSimple = false>
__device__ __forceinline__ BsdfEval bsdf_eval(const DevMaterial& m, V3 wo, V3 wi) {
  BsdfEval e{{0.f, 0.f, 0.f}, 0.f};
  if (kSimple || m.type == kMatLambertian) {
    // Lambertian.Eval (Lambertian.fs:11-16)
    if (__fmul_rn(wi.z, wo.z) < 0.f || fminf(fabsf(wi.z), fabsf(wo.z)) < 1e-6f) return e;
    const float pdf = __fdiv_rn(fabsf(wi.z), kPi);
    e.f = scale(pdf, mk(m.base[0], m.base[1], m.base[2]));
    e.pdf = pdf;
  } else if (m.type == kMatPBR) {
    e = pbr_eval(mk(m.base[0], m.base[1], m.base[2]), m.alpha, m.metallic, wo, wi);
  }
  // Mirror.Eval / Dielectric.Eval: zero (Mirror.fs:11-12, Dielectric.fs:13-14)
  return e;
}

__device__ __forceinline__ V3 cosine_dir(float u0, float u1) {
  const float cos_t = __fsqrt_rn(u0), sin_t = __fsqrt_rn(__fsub_rn(1.f, u0));
  float sp, cp;
  sincosf(__fmul_rn(2.f * kPi, u1), &sp, &cp);
  return {__fmul_rn(sin_t, cp), __fmul_rn(sin_t, sp), cos_t};
}

template <bool kSimple = false>
__device__ __forceinline__ BsdfSample bsdf_sample(const DevMaterial& m, V3 wo, float u_lobe, float u0, float u1) {
  BsdfSample s;
  const V3 base = mk(m.base[0], m.base[1], m.base[2]);
  if (kSimple || m.type == kMatLambertian) {
    // Lambertian.Sample (Lambertian.fs:18-26): cosine lobe mirrored to wo's side
    V3 wi = cosine_dir(u0, u1);
    const float pdf = __fdiv_rn(wi.z, kPi);
    s.f = scale(pdf, base);
    s.pdf = pdf;
    s.wi = wo.z > 0.f ? wi : neg(wi);
  } else if (m.type == kMatMirror) {
    // MirrorMaterial.Sample (Mirror.fs:13-14): delta, pdf 1
    s.f = base;
    s.pdf = 1.f;
    s.wi = mk(-wo.x, -wo.y, wo.z);
  } else if (m.type == kMatDielectric) {
    // DielectricMaterial.Sample (Dielectric.fs:15-31): Schlick, TIR -> reflection
    const float eta = wo.z > 0.f ? __frcp_rn(m.ior) : m.ior;
    const float cos2t = __fsub_rn(1.f, __fmul_rn(__fmul_rn(eta, eta), fmaf(-wo.z, wo.z, 1.f)));
    if (cos2t <= 0.f) {
      s.f = base; s.pdf = 1.f; s.wi = mk(-wo.x, -wo.y, wo.z);
    } else {
      const float a = __fsub_rn(eta, 1.f), b = __fadd_rn(eta, 1.f);
      const float r0 = __fdiv_rn(__fmul_rn(a, a), __fmul_rn(b, b));
      const float c = __fsub_rn(1.f, fabsf(wo.z));
      const float c2 = __fmul_rn(c, c);
      const float r = __fadd_rn(r0, __fmul_rn(__fmul_rn(__fmul_rn(__fsub_rn(1.f, r0), c2), c2), c));
      if (u_lobe < r) {
        s.f = scale(r, base); s.pdf = r; s.wi = mk(-wo.x, -wo.y, wo.z);
      } else {
        const float cos_t = __fsqrt_rn(cos2t);
        const float t = __fsub_rn(1.f, r);
        s.f = scale(t, base); s.pdf = t;
        s.wi = mk(__fmul_rn(-wo.x, eta), __fmul_rn(-wo.y, eta), -copysignf(cos_t, wo.z));
      }
    }
  } else {
    // PBRMaterial.Sample (PBR.fs:145-159): GGX half-vector or cosine lobe, then Eval
    V3 wi;
    if (u_lobe < __fsub_rn(1.f, __fmul_rn(0.5f, __fsub_rn(1.f, m.metallic)))) {
      const float th = atanf(__fmul_rn(m.alpha, __fsqrt_rn(__fdiv_rn(u0, __fsub_rn(1.f, u0)))));
      const float ph = __fmul_rn(2.f * kPi, u1);
      float st, ct, sp, cp;
      sincosf(th, &st, &ct);
      sincosf(ph, &sp, &cp);
      const V3 wh = {__fmul_rn(st, cp), __fmul_rn(st, sp), ct};
      wi = sub(scale(__fmul_rn(2.f, dot(wo, wh)), wh), wo);
    } else {
      wi = cosine_dir(u0, u1);
    }
    const BsdfEval e = pbr_eval(base, m.alpha, m.metallic, wo, wi);
    s.f = e.f; s.pdf = e.pdf; s.wi = wi;
  }
  return s;
}

// ------------------------------------------------------------------ lights
// DiffuseLight.Eval (Base/Light.fs:49-53) with wo_z = WorldToLocal(wo).z
__device__ __forceinline__ V3 light_le(const DevLight& l, float wo_z) {
  if (fabsf(wo_z) > 1e-6f && (wo_z > 0.f || l.two_sided)) return mk(l.emission[0], l.emission[1], l.emission[2]);
  return mk(0.f, 0.f, 0.f);
}

// world-space vertices of triangle tri of instance I (Triangle.Transform, Mesh.fs:101-105)
__device__ __forceinline__ void world_tri(const DevScene& s, const DevInstance* I, int tri, V3* p0, V3* p1, V3* p2) {
  float4 o2w[3];
  load_xf(I->o2w, o2w);
  const float4* tp = s.tris + 3 * (__ldg(&I->tri_base) + tri);
  *p0 = xf_point(o2w, xyz(__ldg(tp)));
  *p1 = xf_point(o2w, xyz(__ldg(tp + 1)));
  *p2 = xf_point(o2w, xyz(__ldg(tp + 2)));
}

struct SurfacePoint {
  V3 p, n;    // world position, frame normal (the reference does not renormalise it)
  float pdf;  // area-measure pdf of the surface sample
};

// Triangle.Sample (Mesh.fs:89-99): square-to-triangle map, pdf = 2 / |e0 x e1|
__device__ __forceinline__ SurfacePoint tri_sample(V3 p0, V3 p1, V3 p2, float ux, float uy) {
  float u, v;
  if (ux < uy) { u = __fmul_rn(0.5f, ux); v = fmaf(-0.5f, ux, uy); }
  else { u = fmaf(-0.5f, uy, ux); v = __fmul_rn(0.5f, uy); }
  SurfacePoint sp;
  sp.p = add(add(scale(u, p1), scale(v, p2)), scale(__fsub_rn(__fsub_rn(1.f, u), v), p0));
  const V3 n = cross(sub(p1, p0), sub(p2, p0));
  sp.pdf = __fdiv_rn(2.f, length(n));
  sp.n = scale(__fmul_rn(0.5f, sp.pdf), n);
  return sp;
}

// SphereInstance.Sample (Sphere.fs:90-113)
__device__ __forceinline__ SurfacePoint sphere_sample(const DevInstance* I, float ux, float uy) {
  float st, ct;
  sincosf(__fmul_rn(2.f * kPi, ux), &st, &ct);
  const float cp = fmaf(-2.f, uy, 1.f);
  const float spp = __fsqrt_rn(fmaf(-cp, cp, 1.f));
  const V3 n = {__fmul_rn(ct, spp), __fmul_rn(st, spp), cp};
  const float radius = __ldg(&I->bmax.w);
  const Onb f = onb_from_n(n);
  float4 o2w[3];
  load_xf(I->o2w, o2w);
  SurfacePoint s;
  s.p = xf_point(o2w, scale(radius, n));
  const V3 t2 = xf_dir(o2w, f.t), b2 = xf_dir(o2w, f.b);
  const V3 n2 = cross(t2, b2);
  const float inv_j = __fdiv_rn(1.f, length(n2));
  s.n = scale(inv_j, n2);
  s.pdf = __fdiv_rn(inv_j, __fmul_rn(__fmul_rn(4.f * kPi, radius), radius));
  return s;
}

struct LightSample {
  V3 p;      // point on the light
  V3 L;      // emitted radiance toward the shading point
  float pdf; // solid-angle pdf (includes the light choice)
  V3 wi;     // direction from the shading point to the light
  int light; // index of the sampled light
};

// LightSamplerBase.Sample: UniformLightSampler.Sample (Uniform.fs:13-29) or the alias-table
// sampler over emissive triangles
template <bool kSimple = false>
__device__ __forceinline__ LightSample sample_light(const DevScene& s, V3 p, float u_select, float ux, float uy) {
  SurfacePoint sp;
  int light;
  float sel;  // light-choice factor dividing the pdf (N for uniform, 1 for alias)
  if (!kSimple && s.light_sampler == BN_LIGHTS_ALIAS_TRIANGLES) {
    const int n = s.n_tri_lights;
    const float u = __fmul_rn(u_select, static_cast<float>(n));
    int idx = min(static_cast<int>(u), n - 1);
    const float frac = __fsub_rn(u, static_cast<float>(idx));
    if (frac >= __ldg(&s.tri_lights[idx].prob)) idx = __ldg(&s.tri_lights[idx].alias);
    const int inst = __ldg(&s.tri_lights[idx].inst), tri = __ldg(&s.tri_lights[idx].tri);
    const float pmf = __ldg(&s.tri_lights[idx].pmf);
    const DevInstance* I = s.inst + inst;
    V3 p0, p1, p2;
    world_tri(s, I, tri, &p0, &p1, &p2);
    sp = tri_sample(p0, p1, p2, ux, uy);
    sp.pdf = __fmul_rn(pmf, sp.pdf);
    light = __ldg(&I->light);
    sel = 1.f;
  } else {
    const int n = s.n_light_inst;
    float us = __fmul_rn(u_select, static_cast<float>(n));
    const int id = min(static_cast<int>(us), n - 1);
    us = __fsub_rn(us, static_cast<float>(id));
    const DevInstance* I = s.inst + __ldg(&s.light_inst[id]);
    if (!kSimple && __ldg(&I->prim_type) == kPrimSphere) {
      sp = sphere_sample(I, ux, uy);
    } else {
      // MeshInstance.Sample (Mesh.fs:289-298): the reference alias table picks int(u * n)
      const int nt = __ldg(&I->n_tris);
      const int i = min(static_cast<int>(__fmul_rn(us, static_cast<float>(nt))), nt - 1);
      const float pdf_tri = __ldg(&s.tri_pdf[__ldg(&I->tri_base) + i]);
      V3 p0, p1, p2;
      world_tri(s, I, i, &p0, &p1, &p2);
      sp = tri_sample(p0, p1, p2, ux, uy);
      sp.pdf = __fmul_rn(pdf_tri, sp.pdf);
    }
    light = __ldg(&I->light);
    sel = static_cast<float>(n);
  }
  LightSample ls;
  const V3 dp = sub(p, sp.p);
  const V3 wo = normalize(dp);
  const float cos_wo = dot(sp.n, wo);
  const float dist2 = dot(dp, dp);
  ls.p = sp.p;
  ls.L = light_le(s.lights[light], dot(wo, sp.n));
  ls.pdf = __fdiv_rn(__fmul_rn(dist2, sp.pdf), __fmul_rn(fmaxf(fabsf(cos_wo), 1e-6f), sel));
  ls.wi = neg(wo);
  ls.light = light;
  return ls;
}

// LightSamplerBase.Eval (Uniform.fs:40-49): radiance and solid-angle pdf of an emitter hit
// seen from `origin`
template <bool kSimple = false>
__device__ __forceinline__ void eval_light(const DevScene& s, V3 origin, const Interaction& it, V3* L, float* pdf) {
  const DevInstance* I = s.inst + it.inst;
  const V3 dp = sub(origin, it.p);
  const V3 wo = normalize(dp);
  const float cos_wo = dot(it.f.n, wo);
  float pdf_surface, sel;
  if (!kSimple && s.light_sampler == BN_LIGHTS_ALIAS_TRIANGLES) {
    const int e = __ldg(&I->light_entry_base) + it.tri;
    V3 p0, p1, p2;
    world_tri(s, I, it.tri, &p0, &p1, &p2);
    const float area_pdf = __fdiv_rn(2.f, length(cross(sub(p1, p0), sub(p2, p0))));
    pdf_surface = __fmul_rn(__ldg(&s.tri_lights[e].pmf), area_pdf);
    sel = 1.f;
  } else {
    if (!kSimple && __ldg(&I->prim_type) == kPrimSphere) {
      // SphereInstance.EvalPDF (Sphere.fs:115-126)
      float4 w2o[3];
      load_xf(I->w2o, w2o);
      const V3 t2 = xf_dir(w2o, it.f.t), b2 = xf_dir(w2o, it.f.b);
      const float r = __ldg(&I->bmax.w);
      pdf_surface = __fdiv_rn(length(cross(t2, b2)), __fmul_rn(__fmul_rn(4.f * kPi, r), r));
    } else {
      // MeshInstance.EvalPDF (Mesh.fs:300-304) with the tag that LocalGeometry.Transform reset
      // to 0: the pdf of triangle 0 over the area of triangle 0
      V3 p0, p1, p2;
      world_tri(s, I, 0, &p0, &p1, &p2);
      const float area = __fmul_rn(0.5f, length(cross(sub(p1, p0), sub(p2, p0))));
      pdf_surface = __fdiv_rn(__ldg(&s.tri_pdf[__ldg(&I->tri_base)]), area);
    }
    sel = static_cast<float>(s.n_light_inst);
  }
  const float dist2 = dot(dp, dp);
  *L = light_le(s.lights[__ldg(&I->light)], dot(wo, it.f.n));
  *pdf = __fdiv_rn(__fmul_rn(dist2, pdf_surface), __fmul_rn(fmaxf(fabsf(cos_wo), 1e-6f), sel));
}

// material of a hit: per-triangle slot if the mesh has one, else the instance's (-1 = none)
__device__ __forceinline__ int hit_material(const DevScene& s, const Interaction& it) {
  const DevInstance* I = s.inst + it.inst;
  const int m = __ldg(&I->material);
  if (m < 0 || __ldg(&I->prim_type) == kPrimSphere) return m;
  const int slot = __float_as_int(__ldg(&s.tris[3 * (__ldg(&I->tri_base) + it.tri)].w));
  return slot >= 0 ? slot : m;
}

// 0.5 * (n + Vector3.One), the Normal integrator's colour
__device__ __forceinline__ V3 normal_color(V3 n) {
  return {__fmul_rn(0.5f, __fadd_rn(n.x, 1.f)), __fmul_rn(0.5f, __fadd_rn(n.y, 1.f)), __fmul_rn(0.5f, __fadd_rn(n.z, 1.f))};
}

struct PathCounters {
  unsigned long long rays;
  TraceCounters tc;
};

// A light sample adds fma(a, b, L) per channel when its shadow ray is unoccluded (a = beta * f,
// b = L_e / pdf).  Where every a*b is exactly zero (a factor 0 and the other finite) and L holds
// no -0, that leaves L's bits as they are, so the shadow ray need not be traced: light samples
// below the shading point's horizon (f = 0) and the back of one-sided lights (L_e = 0).
__device__ __forceinline__ bool shadow_contributes(V3 a, V3 b, V3 L) {
  auto zero = [](float x, float y, float l) {
    const bool prod0 = (x == 0.f && isfinite(y)) || (y == 0.f && isfinite(x));
    return prod0 && !(l == 0.f && signbit(l));
  };
  return !(zero(a.x, b.x, L.x) && zero(a.y, b.y, L.y) && zero(a.z, b.z, L.z));
}

// The state of one path between bounces (PathTracingIntegrator.Li's loop variables).
struct PathState {
  Ray ray;
  V3 L, beta;
  float pdf_bsdf;
  int depth;
};

__device__ __forceinline__ void path_begin(PathState& ps, const Ray& ray) {
  ps.ray = ray;
  ps.L = mk(0.f, 0.f, 0.f);
  ps.beta = mk(1.f, 1.f, 1.f);
  ps.pdf_bsdf = 0.f;
  ps.depth = 0;
}

// One iteration of PathTracingIntegrator.Li's bounce loop (Extensions/Integrator/PathTracing.fs:
// 14-81) and, with kFixed7, of PSSMLTIntegrator.Li (PSSMLT.fs:172-245), which draws 7 samples per
// bounce in a fixed order; returns true once the path has ended (ps.L holds its radiance).
// Draw order per bounce: u_select, u_light.xy (NEE), u_lobe, u_bsdf.xy, then u_rr if depth >=
// rr_depth (PathTracing) / always (PSSMLT).  Reciprocal estimates are exact reciprocals here.
// kOutline: one out-of-line walk for both queries (see trace_walk_outline).
// kCull: evaluate the light sample first and trace its shadow ray only if it can contribute
// (shadow_contributes); the result is the same, the plain megakernel keeps the reference's order.
template <bool kWT, bool kFixed7, int kWalk, class Smp, bool kOutline = false, bool kSimple = false,
          bool kCull = false>
__device__ __forceinline__ bool li_bounce(const DevScene& s, PathState& ps, Smp& smp, int max_depth, int rr_depth,
                                          PathCounters* pc) {
  constexpr bool kCount = kWalk == kWalkCount;
  if (ps.depth >= max_depth) return true;
  Ray& ray = ps.ray;
  HitRec h;
  if (kCount) pc->rays++;
  if (!trace_closest<kWT, kWalk, kOutline>(s, ray, CUDART_INF_F, &h, &pc->tc)) return true;
  const Interaction it = make_interaction<kSimple>(s, ray, h);
  const DevInstance* I = s.inst + it.inst;
  if (__ldg(&I->light) >= 0) {
    V3 le;
    float pdf_l;
    eval_light<kSimple>(s, ray.o, it, &le, &pdf_l);
    const float mis = ps.depth == 0 ? 1.f : __fmul_rn(ps.pdf_bsdf, __frcp_rn(__fadd_rn(pdf_l, ps.pdf_bsdf)));
    ps.L = fma3(ps.beta, scale(mis, le), ps.L);
  }
  float u_sel, ulx, uly, u_lobe, ubx, uby, u_rr = 0.f;
  const int mat = hit_material(s, it);
  if (kFixed7) {
    float u7[7];
    smp.template next_n<7>(u7);
    u_sel = u7[0]; ulx = u7[1]; uly = u7[2];
    u_lobe = u7[3]; ubx = u7[4]; uby = u7[5]; u_rr = u7[6];
  }
  if (mat < 0) return true;
  if (!kFixed7) { u_sel = smp.next(); ulx = smp.next(); uly = smp.next(); }
  const DevMaterial m = s.mats[mat];
  const V3 wo_w = neg(ray.d);
  const LightSample ls = sample_light<kSimple>(s, it.p, u_sel, ulx, uly);
  const float dist = length(sub(ls.p, it.p));
  if (ls.pdf != 0.f) {
    Ray sh;
    sh.o = it.p;
    sh.d = ls.wi;
    if (kCull) {
      const BsdfEval be = bsdf_eval<kSimple>(m, to_local(it.f, wo_w), to_local(it.f, ls.wi));
      const V3 a = mul(ps.beta, be.f), b = scale(__frcp_rn(__fadd_rn(be.pdf, ls.pdf)), ls.L);
      if (shadow_contributes(a, b, ps.L)) {
        if (kCount) pc->rays++;
        if (!trace_any<kWT, kWalk, kOutline>(s, sh, __fsub_rn(dist, 1e-3f), &pc->tc)) ps.L = fma3(a, b, ps.L);
      }
    } else {
      if (kCount) pc->rays++;
      if (!trace_any<kWT, kWalk, kOutline>(s, sh, __fsub_rn(dist, 1e-3f), &pc->tc)) {
        const BsdfEval be = bsdf_eval<kSimple>(m, to_local(it.f, wo_w), to_local(it.f, ls.wi));
        ps.L = fma3(mul(ps.beta, be.f), scale(__frcp_rn(__fadd_rn(be.pdf, ls.pdf)), ls.L), ps.L);
      }
    }
  }
  if (!kFixed7) { u_lobe = smp.next(); ubx = smp.next(); uby = smp.next(); }
  const BsdfSample bs = bsdf_sample<kSimple>(m, to_local(it.f, wo_w), u_lobe, ubx, uby);
  if (bs.pdf == 0.f) return true;
  ps.pdf_bsdf = bs.pdf;
  ray.o = it.p;
  ray.d = to_world(it.f, bs.wi);
  ps.beta = scale(__frcp_rn(bs.pdf), mul(ps.beta, bs.f));
  if (ps.depth >= rr_depth) {
    const float q = fminf(1.f, fmaxf(ps.beta.x, fmaxf(ps.beta.y, ps.beta.z)));
    if (!kFixed7) u_rr = smp.next();
    if (u_rr < q) ps.beta = scale(__frcp_rn(q), ps.beta);
    else return true;
  }
  ps.depth++;
  return false;
}

// the whole path: PathTracingIntegrator.Li / PSSMLTIntegrator.Li
template <bool kWT, bool kFixed7, int kWalk, class Smp, bool kOutline = false, bool kSimple = false,
          bool kCull = false>
__device__ __forceinline__ V3 li_path(const DevScene& s, Ray ray, Smp& smp, int max_depth, int rr_depth, PathCounters* pc) {
  PathState ps;
  path_begin(ps, ray);
  while (!li_bounce<kWT, kFixed7, kWalk, Smp, kOutline, kSimple, kCull>(s, ps, smp, max_depth, rr_depth, pc)) {
  }
  return ps.L;
}

// NormalIntegrator.Li (Extensions/Integrator/Normal.fs:10-17): 0.5 (n + 1) of the shading normal
template <bool kWT, int kWalk, bool kOutline = false>
__device__ __forceinline__ V3 li_normal(const DevScene& s, Ray ray, PathCounters* pc) {
  HitRec h;
  if (kWalk == kWalkCount) pc->rays++;
  if (!trace_closest<kWT, kWalk, kOutline>(s, ray, CUDART_INF_F, &h, &pc->tc)) return mk(0.f, 0.f, 0.f);
  const Interaction it = make_interaction(s, ray, h);
  return normal_color(it.f.n);
}

// DirectIntegrator.Li (Extensions/Integrator/Direct.fs:10-40): emission seen directly (weight 1),
// one light sample weighted 1/pdf_light, and one BSDF sample that scores the light it hits with
// f / pdf_light (the reference divides by the light's pdf, not the BSDF's, and checks neither
// pdf for zero).  Draw order: u_select, u_light.xy, u_lobe, u_bsdf.xy.
template <bool kWT, int kWalk, class Smp, bool kOutline = false>
__device__ __forceinline__ V3 li_direct(const DevScene& s, Ray ray, Smp& smp, PathCounters* pc) {
  constexpr bool kCount = kWalk == kWalkCount;
  V3 L = mk(0.f, 0.f, 0.f);
  HitRec h;
  if (kCount) pc->rays++;
  if (!trace_closest<kWT, kWalk, kOutline>(s, ray, CUDART_INF_F, &h, &pc->tc)) return L;
  const Interaction it = make_interaction(s, ray, h);
  const V3 wo_w = neg(ray.d);
  const int light = __ldg(&s.inst[it.inst].light);
  if (light >= 0) L = add(L, light_le(s.lights[light], dot(wo_w, it.f.n)));  // EvalEmit(-d)
  const int mat = hit_material(s, it);
  if (mat < 0) return L;
  const float u_sel = smp.next(), ulx = smp.next(), uly = smp.next();
  const DevMaterial m = s.mats[mat];
  const LightSample ls = sample_light(s, it.p, u_sel, ulx, uly);
  const float dist = length(sub(ls.p, it.p));
  Ray sh;
  sh.o = it.p;
  sh.d = ls.wi;
  if (kCount) pc->rays++;
  if (!trace_any<kWT, kWalk, kOutline>(s, sh, __fsub_rn(dist, 1e-3f), &pc->tc)) {
    const BsdfEval be = bsdf_eval(m, to_local(it.f, wo_w), to_local(it.f, ls.wi));
    L = fma3(be.f, scale(__frcp_rn(ls.pdf), ls.L), L);
  }
  const float u_lobe = smp.next(), ubx = smp.next(), uby = smp.next();
  const BsdfSample bs = bsdf_sample(m, to_local(it.f, wo_w), u_lobe, ubx, uby);
  Ray r2;
  r2.o = it.p;
  r2.d = to_world(it.f, bs.wi);
  HitRec h2;
  if (kCount) pc->rays++;
  if (trace_closest<kWT, kWalk, kOutline>(s, r2, CUDART_INF_F, &h2, &pc->tc)) {
    const Interaction it2 = make_interaction(s, r2, h2);
    if (__ldg(&s.inst[it2.inst].light) >= 0) {
      V3 le;
      float pdf_l;
      eval_light(s, r2.o, it2, &le, &pdf_l);
      L = fma3(bs.f, scale(__frcp_rn(pdf_l), le), L);
    }
  }
  return L;
}

}  // namespace bn
