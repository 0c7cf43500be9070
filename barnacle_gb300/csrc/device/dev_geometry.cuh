// Ray geometry on the device: vector math in the reference's operation order, the slab test,
// the triangle and sphere tests, and the two-level (TLAS -> instance -> BLAS) traversal.
//
// Every float operation of the reference path is written with __fadd_rn/__fmul_rn/... so
// nvcc cannot contract it into an FMA; an FMA appears only where the reference itself calls
// FusedMultiplyAdd (Ray.PointAt, Triangle.Sample, the BSDFs).  With IEEE division, reciprocal
// and square root (the nvcc defaults) this reproduces the CPU restatement's bits.
#pragma once
#include <cuda_runtime.h>
#include <math_constants.h>

#include "dev_types.cuh"
#include "../../../include/barnacle_gpu.h"

namespace bn {

// ------------------------------------------------------------------ exact vector math
struct V3 {
  float x, y, z;
};
__device__ __forceinline__ V3 mk(float x, float y, float z) { return V3{x, y, z}; }
__device__ __forceinline__ V3 add(V3 a, V3 b) { return {__fadd_rn(a.x, b.x), __fadd_rn(a.y, b.y), __fadd_rn(a.z, b.z)}; }
__device__ __forceinline__ V3 sub(V3 a, V3 b) { return {__fsub_rn(a.x, b.x), __fsub_rn(a.y, b.y), __fsub_rn(a.z, b.z)}; }
__device__ __forceinline__ V3 mul(V3 a, V3 b) { return {__fmul_rn(a.x, b.x), __fmul_rn(a.y, b.y), __fmul_rn(a.z, b.z)}; }
__device__ __forceinline__ V3 scale(float s, V3 a) { return {__fmul_rn(s, a.x), __fmul_rn(s, a.y), __fmul_rn(s, a.z)}; }
__device__ __forceinline__ V3 divs(V3 a, float s) { return {__fdiv_rn(a.x, s), __fdiv_rn(a.y, s), __fdiv_rn(a.z, s)}; }
__device__ __forceinline__ V3 neg(V3 a) { return {-a.x, -a.y, -a.z}; }
__device__ __forceinline__ float dot(V3 a, V3 b) {
  return __fadd_rn(__fadd_rn(__fmul_rn(a.x, b.x), __fmul_rn(a.y, b.y)), __fmul_rn(a.z, b.z));
}
__device__ __forceinline__ V3 cross(V3 a, V3 b) {
  return {__fsub_rn(__fmul_rn(a.y, b.z), __fmul_rn(a.z, b.y)), __fsub_rn(__fmul_rn(a.z, b.x), __fmul_rn(a.x, b.z)),
          __fsub_rn(__fmul_rn(a.x, b.y), __fmul_rn(a.y, b.x))};
}
__device__ __forceinline__ float length(V3 a) { return __fsqrt_rn(dot(a, a)); }
__device__ __forceinline__ V3 normalize(V3 a) { return divs(a, length(a)); }
// Vector3.FusedMultiplyAdd(a, b, c)
__device__ __forceinline__ V3 fma3(V3 a, V3 b, V3 c) { return {fmaf(a.x, b.x, c.x), fmaf(a.y, b.y, c.y), fmaf(a.z, b.z, c.z)}; }
__device__ __forceinline__ float comp(V3 a, int i) { return i == 0 ? a.x : (i == 1 ? a.y : a.z); }
// Vector3.MinNative / MaxNative: x86 minps / maxps, the second operand when unordered or equal
__device__ __forceinline__ V3 min_native(V3 a, V3 b) {
  return {a.x < b.x ? a.x : b.x, a.y < b.y ? a.y : b.y, a.z < b.z ? a.z : b.z};
}
__device__ __forceinline__ V3 max_native(V3 a, V3 b) {
  return {a.x > b.x ? a.x : b.x, a.y > b.y ? a.y : b.y, a.z > b.z ? a.z : b.z};
}
__device__ __forceinline__ V3 xyz(float4 v) { return {v.x, v.y, v.z}; }

// Vector3.Transform(v, M) with the matrix stored as three columns (M1r, M2r, M3r, M4r)
__device__ __forceinline__ float xf_row(float4 c, V3 v) {
  return __fadd_rn(__fadd_rn(__fadd_rn(__fmul_rn(v.x, c.x), __fmul_rn(v.y, c.y)), __fmul_rn(v.z, c.z)), c.w);
}
__device__ __forceinline__ V3 xf_point(const float4 m[3], V3 v) { return {xf_row(m[0], v), xf_row(m[1], v), xf_row(m[2], v)}; }
// Transform(v) - Translation: the reference's direction transform (Ray.fs:19-22)
__device__ __forceinline__ V3 xf_dir(const float4 m[3], V3 v) {
  return {__fsub_rn(xf_row(m[0], v), m[0].w), __fsub_rn(xf_row(m[1], v), m[1].w), __fsub_rn(xf_row(m[2], v), m[2].w)};
}
// same on a Matrix4x4 in memory order (cameras)
__device__ __forceinline__ V3 xf_point16(const float* m, V3 v) {
  return {__fadd_rn(__fadd_rn(__fadd_rn(__fmul_rn(v.x, m[0]), __fmul_rn(v.y, m[4])), __fmul_rn(v.z, m[8])), m[12]),
          __fadd_rn(__fadd_rn(__fadd_rn(__fmul_rn(v.x, m[1]), __fmul_rn(v.y, m[5])), __fmul_rn(v.z, m[9])), m[13]),
          __fadd_rn(__fadd_rn(__fadd_rn(__fmul_rn(v.x, m[2]), __fmul_rn(v.y, m[6])), __fmul_rn(v.z, m[10])), m[14])};
}

struct Ray {
  V3 o, d;
};
// Ray.PointAt: Vector3.FusedMultiplyAdd(Vector3(t), d, o) (Ray.fs:16-17)
__device__ __forceinline__ V3 point_at(const Ray& r, float t) {
  return {fmaf(t, r.d.x, r.o.x), fmaf(t, r.d.y, r.o.y), fmaf(t, r.d.z, r.o.z)};
}

// OrthonormalBasis (Base/Primitive.fs:9-40)
struct Onb {
  V3 n, t, b;
};
__device__ __forceinline__ Onb onb_from_n(V3 n) {
  const V3 axis = fabsf(n.x) > 0.1f ? mk(0.f, 1.f, 0.f) : mk(1.f, 0.f, 0.f);
  const V3 t = normalize(cross(n, axis));
  return {n, t, cross(n, t)};
}
__device__ __forceinline__ V3 to_world(const Onb& f, V3 v) {
  // v.X * t + v.Y * b + v.Z * n, summed left to right
  return add(add(scale(v.x, f.t), scale(v.y, f.b)), scale(v.z, f.n));
}
__device__ __forceinline__ V3 to_local(const Onb& f, V3 v) { return {dot(v, f.t), dot(v, f.b), dot(v, f.n)}; }
// OrthonormalBasis.Transform (Primitive.fs:34-38)
__device__ __forceinline__ Onb onb_xf(const Onb& f, const float4 m[3]) {
  const V3 t = normalize(xf_dir(m, f.t));
  const V3 b = normalize(xf_dir(m, f.b));
  return {cross(t, b), t, b};
}

// ------------------------------------------------------------------ slab test (Ray.fs:29-39)
// invDir = 1/d; t0' = MinNative(t0, t1) and t1' = MaxNative(t0, t1) (x86 minps/maxps: the second
// operand when unordered), then Math.Max/Min, which propagate NaN.  A NaN in t1 on any axis
// makes both t0' and t1' NaN there and the box is missed; every other case is an ordinary
// max/min.  tMin starts at 1e-3.
__device__ __forceinline__ bool box_hit(V3 bmin, V3 bmax, const Ray& r, V3 inv, float tmax_in) {
  const float t0x = __fmul_rn(__fsub_rn(bmin.x, r.o.x), inv.x), t1x = __fmul_rn(__fsub_rn(bmax.x, r.o.x), inv.x);
  const float t0y = __fmul_rn(__fsub_rn(bmin.y, r.o.y), inv.y), t1y = __fmul_rn(__fsub_rn(bmax.y, r.o.y), inv.y);
  const float t0z = __fmul_rn(__fsub_rn(bmin.z, r.o.z), inv.z), t1z = __fmul_rn(__fsub_rn(bmax.z, r.o.z), inv.z);
  // fminf/fmaxf decide exactly as MinNative/MaxNative would: they differ only for a NaN t1,
  // which the NaN check below rejects, and zero signs cannot change the comparison
  const float tmin = fmaxf(1e-3f, fmaxf(fminf(t0x, t1x), fmaxf(fminf(t0y, t1y), fminf(t0z, t1z))));
  const float tmax = fminf(tmax_in, fminf(fmaxf(t0x, t1x), fminf(fmaxf(t0y, t1y), fmaxf(t0z, t1z))));
  const bool nan = (t1x != t1x) | (t1y != t1y) | (t1z != t1z);
  return (tmin <= tmax) & !nan;
}
__device__ __forceinline__ V3 inv_dir(V3 d) { return {__frcp_rn(d.x), __frcp_rn(d.y), __frcp_rn(d.z)}; }

// ------------------------------------------------------------------ triangles
// Moller-Trumbore exactly as Triangle.Intersect (Extensions/Primitive/Mesh.fs:50-82):
// eps = Single.Epsilon for both the determinant and t; two-sided; (u, v) = (b1, b2).
__device__ __forceinline__ bool tri_mt(V3 p0, V3 p1, V3 p2, const Ray& r, float tmax, float* t_out, float* u_out, float* v_out) {
  const float eps = 1.40129846e-45f;
  const V3 e0 = sub(p1, p0), e1 = sub(p2, p0);
  const V3 rce1 = cross(r.d, e1);
  const float det = dot(e0, rce1);
  if (fabsf(det) < eps) return false;
  const float inv = __frcp_rn(det);
  const V3 s = sub(r.o, p0);
  const float u = __fmul_rn(inv, dot(s, rce1));
  if (u < 0.f || u > 1.f) return false;
  const V3 sce0 = cross(s, e0);
  const float v = __fmul_rn(inv, dot(r.d, sce0));
  if (v < 0.f || __fadd_rn(u, v) > 1.f) return false;
  const float t = __fmul_rn(inv, dot(e1, sce0));
  if (!(t > eps && t < tmax)) return false;
  *t_out = t; *u_out = u; *v_out = v;
  return true;
}

// Watertight ray/triangle test (Woop, Benthin, Wald, "Watertight Ray/Triangle Intersection",
// JCGT 2013): permute so the dominant direction axis is z, shear the vertices into ray space,
// take the 2-D edge functions with a double-precision fallback on exact zeros, and accept the
// hit when all edge functions share a sign.  Same t/(u, v) conventions as tri_mt.
struct WtRay {
  int k;  // the permutation: kx | ky << 2 | kz << 4 (one register across the walk)
  float sx, sy, sz;
  __device__ __forceinline__ int kx() const { return k & 3; }
  __device__ __forceinline__ int ky() const { return (k >> 2) & 3; }
  __device__ __forceinline__ int kz() const { return k >> 4; }
};
__device__ __forceinline__ WtRay wt_setup(V3 d) {
  const float ax = fabsf(d.x), ay = fabsf(d.y), az = fabsf(d.z);
  int kz = (ax > ay) ? (ax > az ? 0 : 2) : (ay > az ? 1 : 2);
  int kx = kz == 2 ? 0 : kz + 1;
  int ky = kx == 2 ? 0 : kx + 1;
  if (comp(d, kz) < 0.f) { const int tmp = kx; kx = ky; ky = tmp; }
  WtRay w;
  w.k = kx | (ky << 2) | (kz << 4);
  const float dz = comp(d, kz);
  w.sx = __fdiv_rn(comp(d, kx), dz);
  w.sy = __fdiv_rn(comp(d, ky), dz);
  w.sz = __frcp_rn(dz);
  return w;
}
__device__ __forceinline__ bool tri_wt(V3 p0, V3 p1, V3 p2, const Ray& r, const WtRay& w, float tmax, float* t_out, float* u_out,
                                       float* v_out) {
  const V3 A = sub(p0, r.o), B = sub(p1, r.o), C = sub(p2, r.o);
  const int kx = w.kx(), ky = w.ky(), kz = w.kz();
  const float az = comp(A, kz), bz = comp(B, kz), cz = comp(C, kz);
  const float ax = __fsub_rn(comp(A, kx), __fmul_rn(w.sx, az)), ay = __fsub_rn(comp(A, ky), __fmul_rn(w.sy, az));
  const float bx = __fsub_rn(comp(B, kx), __fmul_rn(w.sx, bz)), by = __fsub_rn(comp(B, ky), __fmul_rn(w.sy, bz));
  const float cx = __fsub_rn(comp(C, kx), __fmul_rn(w.sx, cz)), cy = __fsub_rn(comp(C, ky), __fmul_rn(w.sy, cz));
  float U = __fsub_rn(__fmul_rn(cx, by), __fmul_rn(cy, bx));
  float V = __fsub_rn(__fmul_rn(ax, cy), __fmul_rn(ay, cx));
  float W = __fsub_rn(__fmul_rn(bx, ay), __fmul_rn(by, ax));
  if (U == 0.f || V == 0.f || W == 0.f) {
    // exact products in double: the difference of two float products is exact before rounding
    U = __double2float_rn(__dsub_rn(__dmul_rn(cx, by), __dmul_rn(cy, bx)));
    V = __double2float_rn(__dsub_rn(__dmul_rn(ax, cy), __dmul_rn(ay, cx)));
    W = __double2float_rn(__dsub_rn(__dmul_rn(bx, ay), __dmul_rn(by, ax)));
  }
  if ((U < 0.f || V < 0.f || W < 0.f) && (U > 0.f || V > 0.f || W > 0.f)) return false;
  const float det = __fadd_rn(__fadd_rn(U, V), W);
  if (det == 0.f) return false;
  const float T = __fadd_rn(__fadd_rn(__fmul_rn(U, __fmul_rn(w.sz, az)), __fmul_rn(V, __fmul_rn(w.sz, bz))),
                            __fmul_rn(W, __fmul_rn(w.sz, cz)));
  const float inv = __frcp_rn(det);
  const float t = __fmul_rn(T, inv);
  if (!(t > 1.40129846e-45f && t < tmax)) return false;
  *t_out = t; *u_out = __fmul_rn(V, inv); *v_out = __fmul_rn(W, inv);
  return true;
}

// ------------------------------------------------------------------ spheres (Sphere.fs:35-77)
// Returns 0 = miss, 1 = the near root t0 (normal flipped toward the ray), 2 = the far root t1.
__device__ __forceinline__ int sphere_hit(float radius, const Ray& r, float tmax, float* t_out) {
  const float eps = 1e-3f;
  const V3 f = r.o;
  const float a = dot(r.d, r.d);
  const float b = -dot(f, r.d);
  const float r2 = __fmul_rn(radius, radius);
  const float c = __fsub_rn(dot(f, f), r2);
  const V3 fb = add(f, scale(__fdiv_rn(b, a), r.d));
  const float disc = __fsub_rn(r2, dot(fb, fb));
  if (disc < 0.f) return 0;
  const float q = __fadd_rn(b, copysignf(__fsqrt_rn(__fmul_rn(a, disc)), b));
  const float t0 = __fdiv_rn(c, q);
  if (t0 > eps && t0 < tmax) { *t_out = t0; return 1; }
  const float t1 = __fdiv_rn(q, a);
  if (t1 > eps && t1 < tmax) { *t_out = t1; return 2; }
  return 0;
}

// ------------------------------------------------------------------ node access
struct NodeRec {
  V3 bmin, bmax;
  int link;     // right child (interior) or first item (leaf)
  int leaf, axis, count;
};
__device__ __forceinline__ NodeRec load_node(const float4* __restrict__ nodes, int i) {
  const float4 a = __ldg(nodes + 2 * i);
  const float4 b = __ldg(nodes + 2 * i + 1);
  NodeRec n;
  n.bmin = mk(a.x, a.y, a.z);
  n.bmax = mk(a.w, b.x, b.y);
  n.link = __float_as_int(b.z);
  const unsigned packed = static_cast<unsigned>(__float_as_int(b.w));
  n.leaf = packed & 0xffu;
  n.axis = static_cast<int>((packed >> 8) & 0xffu);
  n.count = static_cast<int>(static_cast<signed char>((packed >> 16) & 0xffu));
  return n;
}
__device__ __forceinline__ void load_xf(const float4* __restrict__ src, float4 m[3]) {
  m[0] = __ldg(src); m[1] = __ldg(src + 1); m[2] = __ldg(src + 2);
}

// traversal statistics (algorithmic-bytes accounting), off unless requested
struct TraceCounters {
  unsigned long long nodes, tris, insts;
};

struct HitRec {
  float t, u, v;
  int inst;      // TLAS order, -1 = miss
  int tri;       // BLAS-permuted triangle index within the mesh; sphere: 0
  int sphere_root;  // 1 near root, 2 far root (spheres only)
};

__device__ __forceinline__ void flag_error(const DevScene& s, unsigned bit) {
  if (s.error_word) atomicOr(s.error_word, bit);
}

}  // namespace bn

#include "dev_traverse.cuh"

namespace bn {

// ------------------------------------------------------------------ surface interaction
// The shading frame of a hit: LocalGeometry in object space, then LocalGeometry.Transform with
// ObjectToWorld (Primitive.fs:57-58).  The reference drops the triangle tag there; the tag is
// kept separately here (tri) and used only where the chosen light sampler needs it.
struct Interaction {
  V3 p;       // world position
  Onb f;      // world shading frame
  float u, v; // uv
  int inst;
  int tri;
};

template <bool kSimple = false>  // triangle meshes only
__device__ __forceinline__ Interaction make_interaction(const DevScene& s, const Ray& ray, const HitRec& h) {
  const DevInstance* I = s.inst + h.inst;
  float4 w2o[3], o2w[3];
  load_xf(I->w2o, w2o);
  load_xf(I->o2w, o2w);
  Ray oray;
  oray.o = xf_point(w2o, ray.o);
  oray.d = xf_dir(w2o, ray.d);
  Interaction it;
  it.inst = h.inst;
  it.tri = h.tri;
  V3 p_obj;
  Onb f_obj;
  if (!kSimple && __ldg(&I->prim_type) == kPrimSphere) {
    p_obj = point_at(oray, h.t);
    V3 n = normalize(p_obj);
    it.u = __fadd_rn(__fdiv_rn(atan2f(n.z, n.x), __fmul_rn(2.f, CUDART_PI_F)), 0.5f);
    it.v = __fdiv_rn(acosf(n.y), CUDART_PI_F);
    if (h.sphere_root == 1 && dot(n, oray.d) > 0.f) n = neg(n);
    f_obj = onb_from_n(n);
  } else {
    const float4* tp = s.tris + 3 * (__ldg(&I->tri_base) + h.tri);
    const V3 p0 = xyz(__ldg(tp)), p1 = xyz(__ldg(tp + 1)), p2 = xyz(__ldg(tp + 2));
    const V3 e0 = sub(p1, p0), e1 = sub(p2, p0);
    f_obj = onb_from_n(normalize(cross(e0, e1)));
    p_obj = point_at(oray, h.t);
    it.u = h.u;
    it.v = h.v;
  }
  it.p = xf_point(o2w, p_obj);
  it.f = onb_xf(f_obj, o2w);
  return it;
}

}  // namespace bn
