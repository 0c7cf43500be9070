// ORACLE — test infrastructure only.  A CPU restatement of the Barnacle render path, used by
// tests/, the smoke check and bench.py's CPU baseline as the checker; never by the product.
//
// It follows the F# reference function by function (file:line cited at each), with the
// reference's operation order and with these recorded choices:
//   * MathF.ReciprocalEstimate is an exact 1/x.
//   * Vector3.Transform sums ((x*M11 + y*M21) + z*M31) + M41; Dot sums (x + y) + z.
//   * MinNative/MaxNative are x86 minps/maxps; Math.Max/Min propagate NaN.
//   * no FMA contraction (-ffp-contract=off); FusedMultiplyAdd where the reference calls it.
// The reference itself (F#, .NET 9) cannot be built here, so parity against it is unpinned;
// the oracle is pinned against known-answer vectors computed from the reference's formulas.
#include <algorithm>
#include <atomic>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <limits>
#include <memory>
#include <thread>
#include <vector>

#include "../../include/barnacle_gpu.h"
#include "oracle.h"
#include "oracle_math.hpp"

namespace orc {

constexpr float PI = 3.14159265f;  // MathF.PI
const float kInf = std::numeric_limits<float>::infinity();

// ---------------------------------------------------------------- Util/Hash.fs:6-32
uint32_t XXHash32Two(uint32_t x, uint32_t y) {
  const uint32_t p2 = 2246822519u, p3 = 3266489917u, p4 = 668265263u, p5 = 374761393u;
  uint32_t h = y + p5 + x * p3;
  h = p4 * ((h << 17) | (h >> 15));
  h = p2 * (h ^ (h >> 15));
  h = p3 * (h ^ (h >> 13));
  return h ^ (h >> 16);
}
uint32_t XXHash32Three(uint32_t x, uint32_t y, uint32_t z) {
  const uint32_t p2 = 2246822519u, p3 = 3266489917u, p4 = 668265263u, p5 = 374761393u;
  uint32_t h = z + p5 + x * p3;
  h = p4 * ((h << 17) | (h >> 15));
  h = h + y * p3;
  h = p4 * ((h << 17) | (h >> 15));
  h = p2 * (h ^ (h >> 15));
  h = p3 * (h ^ (h >> 13));
  return h ^ (h >> 16);
}
float LCG(uint32_t& seed) {
  seed = 0x00269ec3u + seed * 0x000343fdu;
  const uint32_t bits = (seed >> 9) | 0x3f800000u;
  float f;
  std::memcpy(&f, &bits, 4);
  return f - 1.f;
}

// Base/Sampler.fs:7-16
struct Sampler {
  uint32_t state;
  static Sampler Two(uint32_t x, uint32_t y) { return {XXHash32Two(x, y)}; }
  static Sampler Three(uint32_t x, uint32_t y, uint32_t z) { return {XXHash32Three(x, y, z)}; }
  float Next1D() { return LCG(state); }
};

// ---------------------------------------------------------------- Util/BVH.fs:9-50
struct AABB {
  Vector3 pMin, pMax;
  Vector3 Centroid() const { return 0.5f * (pMin + pMax); }
  Vector3 Diagonal() const { return pMax - pMin; }
  float SurfaceArea() const {
    const Vector3 d = Diagonal();
    return 2.f * ((d.X * d.Y + d.Y * d.Z) + d.Z * d.X);
  }
  int SplitAxis() const {
    const Vector3 d = Diagonal();
    if (d.X >= d.Y && d.X >= d.Z) return 0;
    return d.Y >= d.Z ? 1 : 2;
  }
  static AABB Default() { return {Vector3(kInf), Vector3(-kInf)}; }
  static AABB Union(const AABB& a, const AABB& b) {
    return {Vector3::MinNative(a.pMin, b.pMin), Vector3::MaxNative(a.pMax, b.pMax)};
  }
  static AABB Union(const AABB& a, const Vector3& b) { return {Vector3::MinNative(a.pMin, b), Vector3::MaxNative(a.pMax, b)}; }
  static AABB Transform(const AABB& a, const Matrix4x4& m) {
    Vector3 lo(kInf), hi(-kInf);
    for (int i = 0; i < 8; ++i) {
      const Vector3 p((i & 1) == 0 ? a.pMin.X : a.pMax.X, (i & 2) == 0 ? a.pMin.Y : a.pMax.Y,
                      (i & 4) == 0 ? a.pMin.Z : a.pMax.Z);
      const Vector3 q = orc::Transform(p, m);
      lo = Vector3::MinNative(lo, q);
      hi = Vector3::MaxNative(hi, q);
    }
    return {lo, hi};
  }
};

struct Counters {
  uint64_t rays = 0, nodes = 0, tris = 0, insts = 0;
};

// ---------------------------------------------------------------- Base/Ray.fs
struct Ray {
  Vector3 Origin, Direction;
  Vector3 PointAt(float t) const { return Vector3::FusedMultiplyAdd(Vector3(t), Direction, Origin); }
  static Ray Transform(const Ray& r, const Matrix4x4& m) {
    return {orc::Transform(r.Origin, m), orc::Transform(r.Direction, m) - m.Translation()};
  }
};
// AxisAlignedBoundingBox.Intersect (Ray.fs:29-39)
bool BoxIntersect(const AABB& b, const Ray& r, float t) {
  const Vector3 invDir = Vector3(1.f) / r.Direction;
  float tMin = 1e-3f, tMax = t;
  const Vector3 t0 = (b.pMin - r.Origin) * invDir;
  const Vector3 t1 = (b.pMax - r.Origin) * invDir;
  const Vector3 a = Vector3::MinNative(t0, t1);
  const Vector3 c = Vector3::MaxNative(t0, t1);
  tMin = MathMax(tMin, MathMax(a.X, MathMax(a.Y, a.Z)));
  tMax = MathMin(tMax, MathMin(c.X, MathMin(c.Y, c.Z)));
  return tMin <= tMax;
}

// ---------------------------------------------------------------- Util/BVH.fs:99-247
struct BuildItem {
  AABB bounds;
  int index;
};
struct Tree {
  bool leaf;
  AABB bounds;
  int offset, count;  // leaf
  int axis;           // interior
  std::unique_ptr<Tree> left, right;
};

std::unique_ptr<Tree> TreeBuild(std::vector<BuildItem>& instances, int first, int last, int depth) {
  const int n = last - first;
  std::vector<BuildItem> sub(instances.begin() + first, instances.begin() + last);  // Slice(...).ToArray()
  AABB bounds = AABB::Default();
  for (int i = 0; i < n; ++i) bounds = AABB::Union(bounds, sub[i].bounds);
  auto t = std::make_unique<Tree>();
  t->bounds = bounds;
  if (n <= 4 || depth >= 64) {
    t->leaf = true; t->offset = first; t->count = n;
    return t;
  }
  AABB cb = AABB::Default();
  for (int i = 0; i < n; ++i) cb = AABB::Union(cb, sub[i].bounds.Centroid());
  const int axis = cb.SplitAxis();
  const float extent = cb.Diagonal()[axis];
  t->leaf = false;
  t->axis = axis;
  if (extent == 0.f) {
    const int mid = first + n / 2;
    t->left = TreeBuild(instances, first, mid, depth + 1);
    t->right = TreeBuild(instances, mid, last, depth + 1);
    return t;
  }
  AABB binB[12];
  int binC[12];
  for (int i = 0; i < 12; ++i) { binB[i] = AABB::Default(); binC[i] = 0; }
  auto findBin = [&](const BuildItem& it) {
    // int(...) converts as .NET 9 does: truncation, saturated, NaN -> 0 (infinite boxes give NaN)
    const float f = (12.f * (it.bounds.Centroid()[axis] - cb.pMin[axis])) / extent;
    const int b = f != f ? 0 : (f >= 2147483647.f ? 2147483647 : static_cast<int>(f));
    return std::min(11, b);
  };
  for (int i = first; i < last; ++i) {
    const BuildItem& it = sub[i - first];
    const int b = findBin(it);
    binB[b] = AABB::Union(binB[b], it.bounds);
    binC[b] = binC[b] + 1;
  }
  float costs[11];
  for (float& c : costs) c = 0.f;
  AABB lB = AABB::Default(), rB = AABB::Default();
  int lC = 0, rC = 0;
  for (int i = 0; i < 11; ++i) {
    lB = AABB::Union(lB, binB[i]);
    lC = lC + binC[i];
    costs[i] = costs[i] + static_cast<float>(lC) * lB.SurfaceArea();
    rB = AABB::Union(rB, binB[11 - i]);
    rC = rC + binC[11 - i];
    costs[10 - i] = costs[10 - i] + static_cast<float>(rC) * rB.SurfaceArea();
  }
  float minCost = kInf;
  int best = 0;
  for (int i = 0; i < 11; ++i) {
    const float cost = costs[i] + static_cast<float>(n) * cb.SurfaceArea();
    if (cost < minCost) { minCost = cost; best = i; }
  }
  int left = first, right = last - 1;
  for (int i = 0; i < n; ++i) {
    const BuildItem it = sub[i];
    if (findBin(it) > best) { instances[right] = it; right = right - 1; }
    else { instances[left] = it; left = left + 1; }
  }
  t->left = TreeBuild(instances, first, left, depth + 1);
  t->right = TreeBuild(instances, right + 1, last, depth + 1);
  return t;
}

int Flatten(const Tree& t, std::vector<bn_bvh_node>& nodes) {
  const int index = static_cast<int>(nodes.size());
  bn_bvh_node n{};
  n.bounds_min[0] = t.bounds.pMin.X; n.bounds_min[1] = t.bounds.pMin.Y; n.bounds_min[2] = t.bounds.pMin.Z;
  n.bounds_max[0] = t.bounds.pMax.X; n.bounds_max[1] = t.bounds.pMax.Y; n.bounds_max[2] = t.bounds.pMax.Z;
  if (t.leaf) {
    n.right_or_offset = t.offset;
    n.is_leaf = 1;
    n.count = static_cast<int8_t>(t.count);
    nodes.push_back(n);
  } else {
    nodes.push_back(bn_bvh_node{});
    Flatten(*t.left, nodes);
    n.right_or_offset = Flatten(*t.right, nodes);
    n.is_leaf = 0;
    n.split_axis = static_cast<int8_t>(t.axis);
    nodes[index] = n;
  }
  return index;
}

// BVHNode.Build: returns nodes and the permutation (perm[k] = original index at k)
std::vector<bn_bvh_node> BVHBuild(const std::vector<AABB>& boxes, std::vector<int>* perm) {
  std::vector<BuildItem> items(boxes.size());
  for (size_t i = 0; i < boxes.size(); ++i) items[i] = {boxes[i], static_cast<int>(i)};
  auto tree = TreeBuild(items, 0, static_cast<int>(items.size()), 0);
  std::vector<bn_bvh_node> nodes;
  Flatten(*tree, nodes);
  perm->resize(items.size());
  for (size_t i = 0; i < items.size(); ++i) (*perm)[i] = items[i].index;
  return nodes;
}

AABB NodeBounds(const bn_bvh_node& n) {
  return {Vector3(n.bounds_min[0], n.bounds_min[1], n.bounds_min[2]), Vector3(n.bounds_max[0], n.bounds_max[1], n.bounds_max[2])};
}

// ---------------------------------------------------------------- Base/Primitive.fs:9-60
struct ONB {
  Vector3 n, t, b;
  static ONB FromN(const Vector3& n) {
    const Vector3 axis = std::fabs(n.X) > 0.1f ? Vector3(0, 1, 0) : Vector3(1, 0, 0);
    const Vector3 t = Vector3::Normalize(Vector3::Cross(n, axis));
    return {n, t, Vector3::Cross(n, t)};
  }
  Vector3 LocalToWorld(const Vector3& v) const { return (v.X * t + v.Y * b) + v.Z * n; }
  Vector3 WorldToLocal(const Vector3& v) const { return {Vector3::Dot(v, t), Vector3::Dot(v, b), Vector3::Dot(v, n)}; }
  static ONB Transform(const ONB& f, const Matrix4x4& m) {
    const Vector3 t2 = Vector3::Normalize(orc::Transform(f.t, m) - m.Translation());
    const Vector3 b2 = Vector3::Normalize(orc::Transform(f.b, m) - m.Translation());
    return {Vector3::Cross(t2, b2), t2, b2};
  }
};
struct LocalGeometry {
  Vector3 p;
  ONB onb;
  float u = 0, v = 0;
  int tag = 0;
  static LocalGeometry Transform(const LocalGeometry& g, const Matrix4x4& m) {
    LocalGeometry r;
    r.p = orc::Transform(g.p, m);
    r.onb = ONB::Transform(g.onb, m);
    r.u = g.u; r.v = g.v;
    r.tag = 0;  // the 3-argument constructor resets the tag (Primitive.fs:57-58, :49)
    return r;
  }
};

// ---------------------------------------------------------------- Extensions/Primitive/Mesh.fs
struct Triangle {
  Vector3 P0, P1, P2;
  AABB Bounds() const {
    return {Vector3::MinNative(Vector3::MinNative(P0, P1), P2), Vector3::MaxNative(Vector3::MaxNative(P0, P1), P2)};
  }
  // Mesh.fs:24-82, Moller-Trumbore with eps = Single.Epsilon
  bool Intersect(const Ray& ray, float* t, float* u_out, float* v_out) const {
    const float eps = std::numeric_limits<float>::denorm_min();
    const Vector3 e0 = P1 - P0, e1 = P2 - P0;
    const Vector3 rce1 = Vector3::Cross(ray.Direction, e1);
    const float det = Vector3::Dot(e0, rce1);
    if (std::fabs(det) < eps) return false;
    const float invDet = 1.f / det;
    const Vector3 s = ray.Origin - P0;
    const float u = invDet * Vector3::Dot(s, rce1);
    if (u < 0.f || u > 1.f) return false;
    const Vector3 sce0 = Vector3::Cross(s, e0);
    const float v = invDet * Vector3::Dot(ray.Direction, sce0);
    if (v < 0.f || u + v > 1.f) return false;
    const float tt = invDet * Vector3::Dot(e1, sce0);
    if (!(tt > eps && tt < *t)) return false;
    *t = tt; *u_out = u; *v_out = v;
    return true;
  }
  // watertight test (Woop, Benthin, Wald 2013): the same formulation as the device kernel
  bool IntersectWatertight(const Ray& ray, float* t, float* u_out, float* v_out) const {
    const Vector3 d = ray.Direction;
    const float ax = std::fabs(d.X), ay = std::fabs(d.Y), az = std::fabs(d.Z);
    int kz = (ax > ay) ? (ax > az ? 0 : 2) : (ay > az ? 1 : 2);
    int kx = kz == 2 ? 0 : kz + 1;
    int ky = kx == 2 ? 0 : kx + 1;
    if (d[kz] < 0.f) std::swap(kx, ky);
    const float Sx = d[kx] / d[kz], Sy = d[ky] / d[kz], Sz = 1.f / d[kz];
    const Vector3 A = P0 - ray.Origin, B = P1 - ray.Origin, C = P2 - ray.Origin;
    const float Az = A[kz], Bz = B[kz], Cz = C[kz];
    const float Ax = A[kx] - Sx * Az, Ay = A[ky] - Sy * Az;
    const float Bx = B[kx] - Sx * Bz, By = B[ky] - Sy * Bz;
    const float Cx = C[kx] - Sx * Cz, Cy = C[ky] - Sy * Cz;
    float U = Cx * By - Cy * Bx, V = Ax * Cy - Ay * Cx, W = Bx * Ay - By * Ax;
    if (U == 0.f || V == 0.f || W == 0.f) {
      U = static_cast<float>(static_cast<double>(Cx) * By - static_cast<double>(Cy) * Bx);
      V = static_cast<float>(static_cast<double>(Ax) * Cy - static_cast<double>(Ay) * Cx);
      W = static_cast<float>(static_cast<double>(Bx) * Ay - static_cast<double>(By) * Ax);
    }
    if ((U < 0.f || V < 0.f || W < 0.f) && (U > 0.f || V > 0.f || W > 0.f)) return false;
    const float det = (U + V) + W;
    if (det == 0.f) return false;
    const float T = (U * (Sz * Az) + V * (Sz * Bz)) + W * (Sz * Cz);
    const float inv = 1.f / det;
    const float tt = T * inv;
    if (!(tt > std::numeric_limits<float>::denorm_min() && tt < *t)) return false;
    *t = tt; *u_out = V * inv; *v_out = W * inv;
    return true;
  }
  float SurfaceArea() const { return 0.5f * Vector3::Cross(P1 - P0, P2 - P0).Length(); }
  // Mesh.fs:89-99
  void Sample(float ux, float uy, LocalGeometry* g, float* pdf) const {
    float u, v;
    if (ux < uy) { u = 0.5f * ux; v = std::fma(-0.5f, ux, uy); }
    else { u = std::fma(-0.5f, uy, ux); v = 0.5f * uy; }
    const Vector3 p = (u * P1 + v * P2) + ((1.f - u) - v) * P0;
    const Vector3 n = Vector3::Cross(P1 - P0, P2 - P0);
    *pdf = 2.f / n.Length();
    g->p = p;
    g->onb = ONB::FromN((0.5f * *pdf) * n);
    g->u = u; g->v = v;
    g->tag = 0;
  }
  static Triangle Transform(const Triangle& t, const Matrix4x4& m) {
    return {orc::Transform(t.P0, m), orc::Transform(t.P1, m), orc::Transform(t.P2, m)};
  }
};

// Util/AliasTable.fs:14-62 (the construction as written: prob = w / sum)
struct RefAliasEntry {
  int alias;
  float prob, pdf;
};
std::vector<RefAliasEntry> RefAliasTable(const std::vector<float>& w) {
  const size_t n = w.size();
  float sum = 0.f;
  for (float x : w) sum = sum + x;
  std::vector<RefAliasEntry> table(n);
  if (sum == 0.f) {
    for (size_t i = 0; i < n; ++i) table[i] = {static_cast<int>(i), 1.f, 1.f / static_cast<float>(n)};
    return table;
  }
  for (size_t i = 0; i < n; ++i) table[i] = {static_cast<int>(i), w[i] / sum, w[i] / sum};
  std::vector<int> under, over;
  for (size_t i = 0; i < n; ++i) (table[i].prob > 1.f ? over : under).push_back(static_cast<int>(i));
  while (!under.empty() && !over.empty()) {
    const int o = over.back(); over.pop_back();
    const int u = under.back(); under.pop_back();
    table[o].prob = table[o].prob + table[u].prob - 1.f;
    table[u].alias = o;
    (table[o].prob > 1.f ? over : under).push_back(o);
  }
  for (int o : over) { table[o].alias = o; table[o].prob = 1.f; }
  for (int u : under) { table[u].alias = u; table[u].prob = 1.f; }
  return table;
}
// AliasTable.Sample
int RefAliasSample(const std::vector<RefAliasEntry>& t, float u, float* pdf) {
  u = u * static_cast<float>(t.size());
  int idx = static_cast<int>(u);
  if (idx >= static_cast<int>(t.size())) idx = static_cast<int>(t.size()) - 1;  // out-of-range read guard
  const RefAliasEntry e = t[idx];
  u = u - static_cast<float>(idx);
  if (u < e.prob) { *pdf = e.pdf; return idx; }
  *pdf = t[e.alias].pdf;
  return e.alias;
}

struct Mesh {
  std::vector<Vector3> vertices;
  std::vector<int> tri_index;     // 3 per triangle, in BLAS-permuted order
  std::vector<int> tri_orig;      // original triangle index per permuted slot
  std::vector<int> tri_material;  // per permuted slot, -1 = none
  std::vector<bn_bvh_node> nodes;
  std::vector<RefAliasEntry> alias;
  int n_tris() const { return static_cast<int>(tri_orig.size()); }
  Triangle Tri(int i) const {
    return {vertices[tri_index[3 * i]], vertices[tri_index[3 * i + 1]], vertices[tri_index[3 * i + 2]]};
  }
  // MeshPrimitive constructor order: indices -> BVHNodes (permutes) -> AliasTable (Mesh.fs:123-186)
  void Init(const bn_mesh_desc& d) {
    vertices.resize(d.n_vertices);
    for (int i = 0; i < d.n_vertices; ++i) vertices[i] = {d.vertices[3 * i], d.vertices[3 * i + 1], d.vertices[3 * i + 2]};
    std::vector<AABB> boxes(d.n_triangles);
    for (int t = 0; t < d.n_triangles; ++t) {
      const Triangle tr{vertices[d.indices[3 * t]], vertices[d.indices[3 * t + 1]], vertices[d.indices[3 * t + 2]]};
      boxes[t] = tr.Bounds();
    }
    std::vector<int> perm;
    nodes = BVHBuild(boxes, &perm);
    tri_orig = perm;
    tri_index.resize(3 * perm.size());
    tri_material.assign(perm.size(), -1);
    for (size_t k = 0; k < perm.size(); ++k) {
      for (int c = 0; c < 3; ++c) tri_index[3 * k + c] = d.indices[3 * perm[k] + c];
      if (d.tri_material) tri_material[k] = d.tri_material[perm[k]];
    }
    std::vector<float> w(perm.size());
    for (size_t k = 0; k < perm.size(); ++k) w[k] = Tri(static_cast<int>(k)).SurfaceArea();
    alias = RefAliasTable(w);
  }
  // MeshPrimitive.Intersect(ray, geom, t): closest hit (Mesh.fs:217-242)
  bool IntersectClosest(const Ray& ray, float* t, int* tag, float* u, float* v, bool wt, Counters* c) const {
    int stack[128];
    int top = 0;
    stack[top++] = 0;
    bool hit = false;
    while (top != 0) {
      const int i = stack[--top];
      const bn_bvh_node& node = nodes[i];
      c->nodes++;
      if (!BoxIntersect(NodeBounds(node), ray, *t)) continue;
      if (node.is_leaf) {
        for (int k = node.right_or_offset; k < node.right_or_offset + node.count; ++k) {
          const Triangle tr = Tri(k);
          c->tris++;
          // the triangle AABB pre-test (Mesh.fs:231) precedes either triangle test
          bool h = BoxIntersect(tr.Bounds(), ray, *t);
          if (h) h = wt ? tr.IntersectWatertight(ray, t, u, v) : tr.Intersect(ray, t, u, v);
          if (h) { *tag = k; hit = true; }
        }
      } else if (ray.Direction[node.split_axis] > 0.f) {
        stack[top++] = node.right_or_offset; stack[top++] = i + 1;
      } else {
        stack[top++] = i + 1; stack[top++] = node.right_or_offset;
      }
    }
    return hit;
  }
  // MeshPrimitive.Intersect(ray, t): any hit (Mesh.fs:188-215).  The reference starts with
  // stackTop = 1, which re-traverses the root from the zeroed slot 0 after a miss; the result
  // is the same, so the second pass is not repeated here.
  bool IntersectAny(const Ray& ray, float t, bool wt, Counters* c) const {
    int stack[128];
    int top = 0;
    stack[top++] = 0;
    while (top != 0) {
      const int i = stack[--top];
      const bn_bvh_node& node = nodes[i];
      c->nodes++;
      if (!BoxIntersect(NodeBounds(node), ray, t)) continue;
      if (node.is_leaf) {
        for (int k = node.right_or_offset; k < node.right_or_offset + node.count; ++k) {
          const Triangle tr = Tri(k);
          c->tris++;
          float tt = t, u, v;
          bool h = BoxIntersect(tr.Bounds(), ray, t);
          if (h) h = wt ? tr.IntersectWatertight(ray, &tt, &u, &v) : tr.Intersect(ray, &tt, &u, &v);
          if (h) return true;
        }
      } else if (ray.Direction[node.split_axis] > 0.f) {
        stack[top++] = node.right_or_offset; stack[top++] = i + 1;
      } else {
        stack[top++] = i + 1; stack[top++] = node.right_or_offset;
      }
    }
    return false;
  }
};

// ---------------------------------------------------------------- Sphere.fs:13-77
// 0 = miss, 1 = near root, 2 = far root
int SphereIntersect(float radius, const Ray& ray, float* t) {
  const float eps = 1e-3f;
  const Vector3 f = ray.Origin;
  const float a = ray.Direction.LengthSquared();
  const float b = -Vector3::Dot(f, ray.Direction);
  const float r2 = radius * radius;
  const float c = f.LengthSquared() - r2;
  const float d = r2 - (f + (b / a) * ray.Direction).LengthSquared();
  if (d < 0.f) return 0;
  const float q = b + std::copysign(std::sqrt(a * d), b);
  const float t0 = c / q;
  if (t0 > eps && t0 < *t) { *t = t0; return 1; }
  const float t1 = q / a;
  if (t1 > eps && t1 < *t) { *t = t1; return 2; }
  return 0;
}

// ---------------------------------------------------------------- materials (local frame)
template <class T>
struct BSDFEvalT {
  Vec3<T> bsdf;
  T pdf;
};
template <class T>
struct BSDFSampleT {
  BSDFEvalT<T> eval;
  Vec3<T> wi;
};

template <class T>
inline T fmaT(T a, T b, T c) { return std::fma(a, b, c); }

template <class T>
struct Material {
  int type;
  Vec3<T> base;
  T ior, alpha, metallic;
  static Material From(const bn_material_desc& m) {
    Material r;
    r.type = m.type;
    r.base = {static_cast<T>(m.base_color[0]), static_cast<T>(m.base_color[1]), static_cast<T>(m.base_color[2])};
    r.ior = m.ior;
    const float a = m.roughness * m.roughness;  // MathF.Max(roughness * roughness, 1e-3f)
    r.alpha = static_cast<T>(a > 1e-3f ? a : 1e-3f);
    r.metallic = static_cast<T>(std::min(std::max(m.metallic, 0.f), 1.f));
    return r;
  }
  static T Pi() { return static_cast<T>(PI); }
  // PBR.fs:108-131
  T Lambda(const Vec3<T>& w) const {
    const T sin2 = fmaT(w.X, w.X, w.Y * w.Y);
    if (sin2 == 0) return 0;
    const T tan2 = sin2 / (w.Z * w.Z);
    const T a2t2 = alpha * alpha * tan2;
    return (T(-1) + std::sqrt(T(1) + a2t2)) / T(2);
  }
  T D(const Vec3<T>& wh) const {
    const T c = std::fabs(wh.Z);
    const T k = T(1) + fmaT(alpha, alpha, T(-1)) * c * c;
    return alpha * alpha / (Pi() * (k * k));
  }
  T G(const Vec3<T>& wo, const Vec3<T>& wi) const { return T(1) / (T(1) + Lambda(wo) + Lambda(wi)); }
  BSDFEvalT<T> PBREval(const Vec3<T>& wo, const Vec3<T>& wi) const {
    const Vec3<T> wh = Vec3<T>::Normalize(wo + wi);
    const T d = D(wh);
    const T g = G(wo, wi);
    const T spec = d * g / (T(4) * std::fabs(wo.Z));
    const T cosOH = Vec3<T>::Dot(wo, wh);
    const T c = T(1) - cosOH;
    const T c2 = c * c;
    const Vec3<T> fc = base + (Vec3<T>(T(1)) - base) * (c2 * c2 * c);
    const Vec3<T> metal = spec * fc;
    const T fd = T(0.04f) + (T(1) - T(0.04f)) * c2 * c2 * c;
    const Vec3<T> diffuse = base * std::fabs(wi.Z) / Pi();
    const T om = T(1) - fd, omm = T(1) - metallic;
    const Vec3<T> inner = Vec3<T>::FusedMultiplyAdd(diffuse, Vec3<T>(om), Vec3<T>(spec) * fd);
    BSDFEvalT<T> e;
    e.bsdf = Vec3<T>::FusedMultiplyAdd(inner, Vec3<T>(omm), metal * metallic);
    const T tmix = T(0.5f) * omm;
    e.pdf = fmaT(d * std::fabs(wh.Z) / (T(4) * cosOH), T(1) - tmix, std::fabs(wi.Z) / Pi() * tmix);
    return e;
  }
  BSDFEvalT<T> Eval(const Vec3<T>& wo, const Vec3<T>& wi) const {
    BSDFEvalT<T> e{Vec3<T>(T(0)), T(0)};
    if (type == BN_MAT_LAMBERTIAN) {
      // Lambertian.fs:11-16
      if (wi.Z * wo.Z < 0 || std::min(std::fabs(wi.Z), std::fabs(wo.Z)) < T(1e-6f)) return e;
      const T pdf = std::fabs(wi.Z) / Pi();
      e.bsdf = base * pdf;
      e.pdf = pdf;
    } else if (type == BN_MAT_PBR) {
      e = PBREval(wo, wi);
    }
    return e;
  }
  static Vec3<T> Cosine(T u0, T u1) {
    const T cosT = std::sqrt(u0), sinT = std::sqrt(T(1) - u0);
    const T phi = T(2) * Pi() * u1;
    return {sinT * std::cos(phi), sinT * std::sin(phi), cosT};
  }
  BSDFSampleT<T> Sample(const Vec3<T>& wo, T uLobe, T u0, T u1) const {
    BSDFSampleT<T> s;
    if (type == BN_MAT_LAMBERTIAN) {
      // Lambertian.fs:18-26
      const Vec3<T> wi = Cosine(u0, u1);
      const T pdf = wi.Z / Pi();
      s.eval = {base * pdf, pdf};
      s.wi = wo.Z > 0 ? wi : -wi;
    } else if (type == BN_MAT_MIRROR) {
      // Mirror.fs:13-14
      s.eval = {base, T(1)};
      s.wi = {-wo.X, -wo.Y, wo.Z};
    } else if (type == BN_MAT_DIELECTRIC) {
      // Dielectric.fs:15-31
      const T eta = wo.Z > 0 ? T(1) / ior : ior;
      const T cos2 = T(1) - eta * eta * fmaT(-wo.Z, wo.Z, T(1));
      if (cos2 <= 0) {
        s.eval = {base, T(1)};
        s.wi = {-wo.X, -wo.Y, wo.Z};
      } else {
        const T a = eta - T(1), b = eta + T(1);
        const T r0 = a * a / (b * b);
        const T c = T(1) - std::fabs(wo.Z);
        const T c2 = c * c;
        const T r = r0 + (T(1) - r0) * c2 * c2 * c;
        if (uLobe < r) {
          s.eval = {r * base, r};
          s.wi = {-wo.X, -wo.Y, wo.Z};
        } else {
          const T cosT = std::sqrt(cos2);
          s.eval = {(T(1) - r) * base, T(1) - r};
          s.wi = {-wo.X * eta, -wo.Y * eta, -std::copysign(cosT, wo.Z)};
        }
      }
    } else {
      // PBR.fs:145-159
      Vec3<T> wi;
      if (uLobe < T(1) - T(0.5f) * (T(1) - metallic)) {
        const T th = std::atan(alpha * std::sqrt(u0 / (T(1) - u0)));
        const T ph = T(2) * Pi() * u1;
        const Vec3<T> wh{std::sin(th) * std::cos(ph), std::sin(th) * std::sin(ph), std::cos(th)};
        wi = (T(2) * Vec3<T>::Dot(wo, wh)) * wh - wo;
      } else {
        wi = Cosine(u0, u1);
      }
      s.eval = PBREval(wo, wi);
      s.wi = wi;
    }
    return s;
  }
};
using MaterialF = Material<float>;

// Base/Light.fs:49-53
struct DiffuseLight {
  Vector3 emission;
  bool twoSided;
  Vector3 Eval(const Vector3& wo) const {
    if (std::fabs(wo.Z) > 1e-6f && (wo.Z > 0.f || twoSided)) return emission;
    return Vector3(0.f);
  }
};

// ---------------------------------------------------------------- instances + aggregate
struct Scene;
struct Instance {
  int prim_type;  // 0 mesh, 1 sphere
  const Mesh* mesh = nullptr;
  int mesh_id = -1;
  float radius = 0;
  int material = -1, light = -1;
  Matrix4x4 o2w, w2o;
  AABB bounds;
  int light_entry_base = -1;
};

struct Interaction {
  LocalGeometry geom;
  int inst = -1;
  int tri = -1;  // the closest-hit tag before LocalGeometry.Transform reset it
};

struct TriLightEntry {
  float prob;
  int alias;
  float pmf;
  int inst, tri;
};

struct Scene {
  std::vector<Mesh> meshes;
  std::vector<Instance> inst;  // TLAS order
  std::vector<int> order;      // TLAS order -> descriptor index
  std::vector<bn_bvh_node> tlas;
  std::vector<MaterialF> mats;
  std::vector<bn_material_desc> mat_desc;
  std::vector<DiffuseLight> lights;
  std::vector<int> light_inst;
  int light_sampler = 0;
  std::vector<TriLightEntry> tri_lights;

  // PrimitiveInstance.Intersect(ray, interaction, t) (Primitive.fs:118-129)
  bool InstClosest(int k, const Ray& ray, float* t, Interaction* it, bool wt, Counters* c) const {
    const Instance& I = inst[k];
    c->insts++;
    if (!BoxIntersect(I.bounds, ray, *t)) return false;
    const Ray oray = Ray::Transform(ray, I.w2o);
    LocalGeometry g;
    if (I.prim_type == 1) {
      const int root = SphereIntersect(I.radius, oray, t);
      if (!root) return false;
      const Vector3 p = oray.PointAt(*t);
      Vector3 n = Vector3::Normalize(p);
      g.u = std::atan2(n.Z, n.X) / (2.f * PI) + 0.5f;
      g.v = std::acos(n.Y) / PI;
      if (root == 1 && Vector3::Dot(n, oray.Direction) > 0.f) n = -n;
      g.p = p;
      g.onb = ONB::FromN(n);
      it->tri = 0;
    } else {
      int tag;
      float u, v;
      if (!I.mesh->IntersectClosest(oray, t, &tag, &u, &v, wt, c)) return false;
      const Triangle tr = I.mesh->Tri(tag);
      g.p = oray.PointAt(*t);
      g.onb = ONB::FromN(Vector3::Normalize(Vector3::Cross(tr.P1 - tr.P0, tr.P2 - tr.P0)));
      g.u = u; g.v = v;
      g.tag = tag;
      it->tri = tag;
    }
    it->geom = LocalGeometry::Transform(g, I.o2w);
    it->inst = k;
    return true;
  }
  bool InstAny(int k, const Ray& ray, float t, bool wt, Counters* c) const {
    const Instance& I = inst[k];
    c->insts++;
    if (!BoxIntersect(I.bounds, ray, t)) return false;
    const Ray oray = Ray::Transform(ray, I.w2o);
    if (I.prim_type == 1) {
      float tt = t;
      return SphereIntersect(I.radius, oray, &tt) != 0;
    }
    return I.mesh->IntersectAny(oray, t, wt, c);
  }
  // BVHAggregate.Intersect(ray, interaction, t) (Aggregate/BVH.fs:37-58)
  bool Closest(const Ray& ray, float* t, Interaction* it, bool wt, Counters* c) const {
    int stack[65 + 64];
    int top = 0;
    stack[top++] = 0;
    bool hit = false;
    c->rays++;
    while (top != 0) {
      const int i = stack[--top];
      const bn_bvh_node& node = tlas[i];
      c->nodes++;
      if (!BoxIntersect(NodeBounds(node), ray, *t)) continue;
      if (node.is_leaf) {
        for (int k = node.right_or_offset; k < node.right_or_offset + node.count; ++k)
          hit = InstClosest(k, ray, t, it, wt, c) || hit;
      } else if (ray.Direction[node.split_axis] > 0.f) {
        stack[top++] = node.right_or_offset; stack[top++] = i + 1;
      } else {
        stack[top++] = i + 1; stack[top++] = node.right_or_offset;
      }
    }
    return hit;
  }
  // BVHAggregate.Intersect(ray, t) (Aggregate/BVH.fs:11-35)
  bool Any(const Ray& ray, float t, bool wt, Counters* c) const {
    int stack[128];
    int top = 0;
    stack[top++] = 0;
    bool hit = false;
    c->rays++;
    while (!hit && top != 0) {
      const int i = stack[--top];
      const bn_bvh_node& node = tlas[i];
      c->nodes++;
      if (!BoxIntersect(NodeBounds(node), ray, t)) continue;
      if (node.is_leaf) {
        int k = node.right_or_offset;
        while (!hit && k < node.right_or_offset + node.count) { hit = InstAny(k, ray, t, wt, c); ++k; }
      } else if (ray.Direction[node.split_axis] > 0.f) {
        stack[top++] = node.right_or_offset; stack[top++] = i + 1;
      } else {
        stack[top++] = i + 1; stack[top++] = node.right_or_offset;
      }
    }
    return hit;
  }

  int HitMaterial(const Interaction& it) const {
    const Instance& I = inst[it.inst];
    if (I.material < 0 || I.prim_type == 1) return I.material;
    const int slot = I.mesh->tri_material[it.tri];
    return slot >= 0 ? slot : I.material;
  }

  // surface sample of an emitter: world point, frame normal, area pdf
  struct SurfacePoint {
    Vector3 p, n;
    float pdf;
  };
  // MeshInstance.Sample (Mesh.fs:289-298) / SphereInstance.Sample (Sphere.fs:90-113)
  SurfacePoint InstSample(const Instance& I, float uSelect, float ux, float uy) const {
    SurfacePoint sp;
    if (I.prim_type == 1) {
      const float a = 2.f * PI * ux;
      const float sinT = std::sin(a), cosT = std::cos(a);
      const float cosP = std::fma(-2.f, uy, 1.f);
      const float sinP = std::sqrt(std::fma(-cosP, cosP, 1.f));
      const Vector3 n(cosT * sinP, sinT * sinP, cosP);
      const ONB f = ONB::FromN(n);
      const Vector3 p2 = Transform(n * I.radius, I.o2w);
      const Vector3 t2 = Transform(f.t, I.o2w) - I.o2w.Translation();
      const Vector3 b2 = Transform(f.b, I.o2w) - I.o2w.Translation();
      const Vector3 n2 = Vector3::Cross(t2, b2);
      const float invJ = 1.f / n2.Length();
      sp.p = p2;
      sp.n = invJ * n2;
      sp.pdf = invJ / (4.f * PI * I.radius * I.radius);
      return sp;
    }
    float pdfTri;
    const int i = RefAliasSample(I.mesh->alias, uSelect, &pdfTri);
    const Triangle tr = Triangle::Transform(I.mesh->Tri(i), I.o2w);
    LocalGeometry g;
    float pdfArea;
    tr.Sample(ux, uy, &g, &pdfArea);
    sp.p = g.p;
    sp.n = g.onb.n;
    sp.pdf = pdfTri * pdfArea;
    return sp;
  }

  struct LightSample {
    Vector3 p, L;
    float pdf;
    Vector3 wi;
    int light;
  };
  // UniformLightSampler.Sample (Uniform.fs:13-29) or the alias-table sampler over triangles
  LightSample SampleLight(const Vector3& p, float uSelect, float ux, float uy) const {
    SurfacePoint sp;
    int light;
    float sel;
    if (light_sampler == BN_LIGHTS_ALIAS_TRIANGLES) {
      const int n = static_cast<int>(tri_lights.size());
      const float u = uSelect * static_cast<float>(n);
      int idx = std::min(static_cast<int>(u), n - 1);
      const float frac = u - static_cast<float>(idx);
      if (frac >= tri_lights[idx].prob) idx = tri_lights[idx].alias;
      const TriLightEntry& e = tri_lights[idx];
      const Instance& I = inst[e.inst];
      const Triangle tr = Triangle::Transform(I.mesh->Tri(e.tri), I.o2w);
      LocalGeometry g;
      float pdfArea;
      tr.Sample(ux, uy, &g, &pdfArea);
      sp.p = g.p;
      sp.n = g.onb.n;
      sp.pdf = e.pmf * pdfArea;
      light = I.light;
      sel = 1.f;
    } else {
      const int N = static_cast<int>(light_inst.size());
      float us = uSelect * static_cast<float>(N);
      const int id = std::min(static_cast<int>(us), N - 1);
      us = us - static_cast<float>(id);
      const Instance& I = inst[light_inst[id]];
      sp = InstSample(I, us, ux, uy);
      light = I.light;
      sel = static_cast<float>(N);
    }
    LightSample ls;
    const Vector3 wo = Vector3::Normalize(p - sp.p);
    const float cosWo = Vector3::Dot(sp.n, wo);
    const float dist2 = (p - sp.p).LengthSquared();
    const ONB f = ONB::FromN(sp.n);
    ls.p = sp.p;
    ls.L = lights[light].Eval(f.WorldToLocal(wo));
    ls.pdf = dist2 * sp.pdf / (std::max(std::fabs(cosWo), 1e-6f) * sel);
    ls.wi = -wo;
    ls.light = light;
    return ls;
  }
  // LightSamplerBase.Eval (Uniform.fs:40-49)
  void EvalLight(const Vector3& p, const Interaction& it, Vector3* L, float* pdf) const {
    const Instance& I = inst[it.inst];
    const Vector3 wo = Vector3::Normalize(p - it.geom.p);
    const float cosWo = Vector3::Dot(it.geom.onb.n, wo);
    float pdfSurface, sel;
    if (light_sampler == BN_LIGHTS_ALIAS_TRIANGLES) {
      const Triangle tr = Triangle::Transform(I.mesh->Tri(it.tri), I.o2w);
      const float areaPdf = 2.f / Vector3::Cross(tr.P1 - tr.P0, tr.P2 - tr.P0).Length();
      pdfSurface = tri_lights[I.light_entry_base + it.tri].pmf * areaPdf;
      sel = 1.f;
    } else {
      if (I.prim_type == 1) {
        const Vector3 t2 = Transform(it.geom.onb.t, I.w2o) - I.w2o.Translation();
        const Vector3 b2 = Transform(it.geom.onb.b, I.w2o) - I.w2o.Translation();
        pdfSurface = Vector3::Cross(t2, b2).Length() / (4.f * PI * I.radius * I.radius);
      } else {
        const int i = it.geom.tag;  // always 0 after LocalGeometry.Transform
        const Triangle tr = Triangle::Transform(I.mesh->Tri(i), I.o2w);
        pdfSurface = I.mesh->alias[i].pdf / tr.SurfaceArea();
      }
      sel = static_cast<float>(light_inst.size());
    }
    const float dist2 = (p - it.geom.p).LengthSquared();
    *L = lights[I.light].Eval(it.geom.onb.WorldToLocal(wo));
    *pdf = dist2 * pdfSurface / (std::max(std::fabs(cosWo), 1e-6f) * sel);
  }
};

// Vose alias table, the same construction as the library's upload (double-precision build)
void BuildVose(const std::vector<double>& w, std::vector<TriLightEntry>* t) {
  const size_t n = w.size();
  double sum = 0.0;
  for (double x : w) sum += x;
  std::vector<double> scaled(n);
  std::vector<size_t> small, large;
  for (size_t i = 0; i < n; ++i) {
    (*t)[i].alias = static_cast<int>(i);
    (*t)[i].prob = 1.f;
    (*t)[i].pmf = static_cast<float>(sum > 0 ? w[i] / sum : 1.0 / n);
    scaled[i] = sum > 0 ? w[i] * n / sum : 1.0;
    (scaled[i] < 1.0 ? small : large).push_back(i);
  }
  while (!small.empty() && !large.empty()) {
    const size_t s = small.back(), l = large.back();
    small.pop_back();
    (*t)[s].prob = static_cast<float>(scaled[s]);
    (*t)[s].alias = static_cast<int>(l);
    scaled[l] = (scaled[l] + scaled[s]) - 1.0;
    if (scaled[l] < 1.0) {
      large.pop_back();
      small.push_back(l);
    }
  }
}

// ---------------------------------------------------------------- cameras
struct Camera {
  int type;
  float aperture, focus, pushForward;
  Matrix4x4 c2w;
  Vector3 ul, du, dv;
  int W, H;
  static Camera From(const bn_view& v) {
    Camera c;
    c.type = v.camera.type;
    c.aperture = v.camera.aperture;
    c.focus = v.camera.focus_distance;
    c.pushForward = v.camera.push_forward;
    std::memcpy(c.c2w.m, v.camera.camera_to_world, sizeof(c.c2w.m));
    c.W = v.width;
    c.H = v.height;
    // PinholeCamera.GenerateRay (Pinhole.fs:16-22)
    const float vh = 2.f * std::tan(v.camera.fov_y_degrees * PI / 360.f);
    const float vw = vh * v.camera.aspect_ratio;
    const Vector3 U = vw * Vector3(1, 0, 0), V = vh * Vector3(0, 1, 0);
    c.du = U / static_cast<float>(v.width);
    c.dv = V / static_cast<float>(v.height);
    c.ul = Vector3(-0.f, -0.f, -1.f) - 0.5f * (U + V);
    return c;
  }
  // ThinLensCamera.SampleDiskConcentric (ThinLens.fs:12-24)
  static void Disk(float ux, float uy, float* dx, float* dy) {
    const float x = ux * 2.f - 1.f, y = uy * 2.f - 1.f;
    if (x == 0.f || y == 0.f) { *dx = 0.f; *dy = 0.f; return; }
    float r, th;
    if (std::fabs(x) > std::fabs(y)) { r = x; th = PI / 4.f * (y / x); }
    else { r = y; th = PI / 2.f - PI / 4.f * (x / y); }
    *dx = r * std::cos(th);
    *dy = r * std::sin(th);
  }
  // CameraBase.GeneratePrimaryRay (Camera.fs:12-20)
  Ray Generate(int x, int y, float upx, float upy, float ulx, float uly) const {
    const Vector3 pl = (ul + (static_cast<float>(x) + upx) * du) + (static_cast<float>(y) + upy) * dv;
    Ray r{Vector3(0.f), Vector3::Normalize(pl)};
    if (type == BN_CAM_THIN_LENS && aperture > 0.f) {
      float dx, dy;
      Disk(ulx, uly, &dx, &dy);
      const Vector3 o = r.Origin + Vector3(aperture * dx, aperture * dy, 0.f);
      r.Direction = Vector3::Normalize(r.PointAt(focus) - o);
      r.Origin = o;
    }
    Ray w;
    w.Origin = Transform(r.Origin, c2w);
    w.Direction = Vector3::Normalize(Transform(r.Direction, c2w) - c2w.Translation());
    w.Origin = w.PointAt(pushForward);
    return w;
  }
};

// ---------------------------------------------------------------- integrators
struct IndepSampler {
  Sampler s;
  float next() { return s.Next1D(); }
};

// PathTracingIntegrator.Li (PathTracing.fs:14-81); kFixed7: PSSMLTIntegrator.Li (PSSMLT.fs:172-245)
template <bool kFixed7, class Smp>
Vector3 Li(const Scene& sc, Ray ray, Smp& smp, int maxDepth, int rrDepth, bool wt, Counters* c) {
  Vector3 L(0.f), beta(1.f);
  float pdfBsdf = 0.f;
  int depth = 0;
  while (depth < maxDepth) {
    float t = kInf;
    Interaction it;
    if (!sc.Closest(ray, &t, &it, wt, c)) break;
    const Instance& I = sc.inst[it.inst];
    if (I.light >= 0) {
      Vector3 le;
      float pdfL;
      sc.EvalLight(ray.Origin, it, &le, &pdfL);
      const float mis = depth == 0 ? 1.f : pdfBsdf * (1.f / (pdfL + pdfBsdf));
      L = Vector3::FusedMultiplyAdd(beta, le * mis, L);
    }
    float uSel = 0, ulx = 0, uly = 0, uLobe = 0, ubx = 0, uby = 0, uRR = 0;
    if (kFixed7) {
      uSel = smp.next(); ulx = smp.next(); uly = smp.next();
      uLobe = smp.next(); ubx = smp.next(); uby = smp.next(); uRR = smp.next();
    }
    const int mat = sc.HitMaterial(it);
    if (mat < 0) break;
    if (!kFixed7) { uSel = smp.next(); ulx = smp.next(); uly = smp.next(); }
    const MaterialF& m = sc.mats[mat];
    const Vector3 wo = -ray.Direction;
    const Scene::LightSample ls = sc.SampleLight(it.geom.p, uSel, ulx, uly);
    const float dist = (ls.p - it.geom.p).Length();
    if (ls.pdf != 0.f) {
      const Ray sh{it.geom.p, ls.wi};
      if (!sc.Any(sh, dist - 1e-3f, wt, c)) {
        const BSDFEvalT<float> be = m.Eval(it.geom.onb.WorldToLocal(wo), it.geom.onb.WorldToLocal(ls.wi));
        L = Vector3::FusedMultiplyAdd(beta * be.bsdf, ls.L * (1.f / (be.pdf + ls.pdf)), L);
      }
    }
    if (!kFixed7) { uLobe = smp.next(); ubx = smp.next(); uby = smp.next(); }
    const BSDFSampleT<float> bs = m.Sample(it.geom.onb.WorldToLocal(wo), uLobe, ubx, uby);
    if (bs.eval.pdf == 0.f) break;
    pdfBsdf = bs.eval.pdf;
    ray = {it.geom.p, it.geom.onb.LocalToWorld(bs.wi)};
    beta = beta * bs.eval.bsdf * (1.f / bs.eval.pdf);
    if (depth >= rrDepth) {
      const float q = MathMin(1.f, MathMax(beta.X, MathMax(beta.Y, beta.Z)));
      if (!kFixed7) uRR = smp.next();
      if (uRR < q) beta = beta * (1.f / q);
      else break;
    }
    depth++;
  }
  return L;
}

// NormalIntegrator.Li (Extensions/Integrator/Normal.fs:10-17)
Vector3 LiNormal(const Scene& sc, const Ray& ray, bool wt, Counters* c) {
  float t = kInf;
  Interaction it;
  if (!sc.Closest(ray, &t, &it, wt, c)) return Vector3(0.f);
  return 0.5f * (it.geom.onb.n + Vector3(1.f));
}

// DirectIntegrator.Li (Extensions/Integrator/Direct.fs:10-40).  Neither pdf is checked for zero,
// and the BSDF-sampled hit is weighted by the light's pdf, as in the reference.
template <class Smp>
Vector3 LiDirect(const Scene& sc, const Ray& ray, Smp& smp, bool wt, Counters* c) {
  float t = kInf;
  Interaction it;
  Vector3 L(0.f);
  if (!sc.Closest(ray, &t, &it, wt, c)) return L;
  const Instance& I = sc.inst[it.inst];
  if (I.light >= 0) L = L + sc.lights[I.light].Eval(it.geom.onb.WorldToLocal(-ray.Direction));
  const int mat = sc.HitMaterial(it);
  if (mat < 0) return L;
  const float uSel = smp.next(), ulx = smp.next(), uly = smp.next();
  const Scene::LightSample ls = sc.SampleLight(it.geom.p, uSel, ulx, uly);
  const Ray sh{it.geom.p, ls.wi};
  const float dist = (ls.p - it.geom.p).Length();
  const MaterialF& m = sc.mats[mat];
  const Vector3 wo = -ray.Direction;
  if (!sc.Any(sh, dist - 1e-3f, wt, c)) {
    const BSDFEvalT<float> be = m.Eval(it.geom.onb.WorldToLocal(wo), it.geom.onb.WorldToLocal(ls.wi));
    L = Vector3::FusedMultiplyAdd(be.bsdf, ls.L * (1.f / ls.pdf), L);
  }
  const float uLobe = smp.next(), ubx = smp.next(), uby = smp.next();
  const BSDFSampleT<float> bs = m.Sample(it.geom.onb.WorldToLocal(wo), uLobe, ubx, uby);
  const Ray r2{it.geom.p, it.geom.onb.LocalToWorld(bs.wi)};
  float t2 = kInf;
  Interaction it2;
  if (sc.Closest(r2, &t2, &it2, wt, c) && sc.inst[it2.inst].light >= 0) {
    Vector3 le;
    float pdfL;
    sc.EvalLight(r2.Origin, it2, &le, &pdfL);
    L = Vector3::FusedMultiplyAdd(bs.eval.bsdf, le * (1.f / pdfL), L);
  }
  return L;
}

// ---------------------------------------------------------------- PSSMLT (PSSMLT.fs)
// Giles' single-precision erfinv as the reference evaluates it (PSSMLT.fs:69-94)
float ErfInv(float x) {
  x = std::min(std::max(x, -0.99999f), 0.99999f);
  float w = -std::log(std::fma(x, -x, 1.f));
  float p;
  if (w < 5.f) {
    w = w - 2.5f;
    p = 2.81022636e-08f;
    p = std::fma(p, w, 3.43273939e-07f);
    p = std::fma(p, w, -3.5233877e-06f);
    p = std::fma(p, w, -4.39150654e-06f);
    p = std::fma(p, w, 0.00021858087f);
    p = std::fma(p, w, -0.00125372503f);
    p = std::fma(p, w, -0.00417768164f);
    p = std::fma(p, w, 0.246640727f);
    return std::fma(p, w, 1.50140941f) * x;
  }
  w = std::sqrt(w) - 3.f;
  p = -0.000200214257f;
  p = std::fma(p, w, 0.000100950558f);
  p = std::fma(p, w, 0.00134934322f);
  p = std::fma(p, w, -0.00367342844f);
  p = std::fma(p, w, 0.00573950773f);
  p = std::fma(p, w, -0.0076224613f);
  p = std::fma(p, w, 0.00943887047f);
  p = std::fma(p, w, 1.00167406f);
  return std::fma(p, w, 2.83297682f) * x;
}

struct PrimarySample {
  float Value = 0, ValueBackUp = 0;
  int LastModification = 0, ModificationBackUp = 0;
};

// MLTSampler (PSSMLT.fs:36-150)
struct MLTSampler {
  Sampler Inner;
  float LargeStepProb;
  bool kelemen;
  float sigma, epsMin, epsMax;
  PrimarySample* Xs;
  bool LargeStep = false;
  int LastLargeStepIteration = 0, CurrentIteration = 0, SampleIndex = 0, InitializedSampleCount = 0;

  void StartIteration() {
    LargeStep = CurrentIteration == 0 || Inner.Next1D() < LargeStepProb;
    CurrentIteration = CurrentIteration + 1;
    SampleIndex = 0;
  }
  float EnsureReady(int index) {
    PrimarySample& x = Xs[index];
    if (InitializedSampleCount <= index) {
      x = PrimarySample{};
      InitializedSampleCount = index + 1;
    }
    if (x.LastModification < LastLargeStepIteration) {
      x.Value = Inner.Next1D();
      x.LastModification = LastLargeStepIteration;
    }
    x.ValueBackUp = x.Value;
    x.ModificationBackUp = x.LastModification;
    float v;
    if (LargeStep) {
      v = Inner.Next1D();
    } else if (!kelemen) {
      const float normal = std::sqrt(2.f) * ErfInv(std::fma(2.f, Inner.Next1D(), -1.f));
      const float eff = sigma * std::sqrt(static_cast<float>(CurrentIteration - x.LastModification));
      v = std::fma(normal, eff, x.Value);
    } else {
      v = x.Value;
      const float a = std::log(epsMax / epsMin);
      for (int k = x.LastModification; k <= CurrentIteration - 1; ++k) {
        const float u1 = Inner.Next1D() - 0.5f;
        const float u2 = u1 < 0.f ? 1.f + 2.f * u1 : 2.f * u1;
        v = v + std::copysign(epsMax * std::exp(-a * u2), u1);
      }
    }
    x.Value = v - std::floor(v);
    x.LastModification = CurrentIteration;
    return x.Value;
  }
  float next() { return EnsureReady(SampleIndex++); }
  void Reject() {
    for (int i = 0; i < InitializedSampleCount; ++i) {
      Xs[i].Value = Xs[i].ValueBackUp;
      Xs[i].LastModification = Xs[i].ModificationBackUp;
    }
    CurrentIteration = CurrentIteration - 1;
  }
  void Accept() {
    if (LargeStep) LastLargeStepIteration = CurrentIteration;
  }
};

float Luminance(const Vector3& L) { return Vector3::Dot(L, Vector3(0.2126f, 0.7152f, 0.0722f)); }

template <class Smp>
Ray MltCamera(const Camera& cam, Smp& smp, int* px, int* py) {
  const float ux = smp.next() * static_cast<float>(cam.W);
  const float uy = smp.next() * static_cast<float>(cam.H);
  const int x = std::min(cam.W - 1, static_cast<int>(ux)), y = std::min(cam.H - 1, static_cast<int>(uy));
  const float fx = ux - static_cast<float>(x), fy = uy - static_cast<float>(y);
  const float lx = smp.next(), ly = smp.next();
  *px = x;
  *py = y;
  return cam.Generate(x, y, fx, fy, lx, ly);
}

std::unique_ptr<Scene> BuildScene(const bn_scene_desc* d) {
  auto sc = std::make_unique<Scene>();
  sc->meshes.resize(d->n_meshes);
  for (int i = 0; i < d->n_meshes; ++i) sc->meshes[i].Init(d->meshes[i]);
  std::vector<Instance> raw(d->n_instances);
  std::vector<AABB> boxes(d->n_instances);
  for (int i = 0; i < d->n_instances; ++i) {
    const bn_instance_desc& in = d->instances[i];
    const bn_primitive_desc& p = d->primitives[in.primitive];
    Instance& I = raw[i];
    I.prim_type = p.type == BN_PRIM_SPHERE ? 1 : 0;
    I.radius = p.radius;
    I.mesh = p.type == BN_PRIM_MESH ? &sc->meshes[p.mesh] : nullptr;
    I.mesh_id = p.type == BN_PRIM_MESH ? p.mesh : -1;
    I.material = in.material;
    I.light = in.light;
    std::memcpy(I.o2w.m, in.object_to_world, sizeof(I.o2w.m));
    std::memcpy(I.w2o.m, in.world_to_object, sizeof(I.w2o.m));
    // PrimitiveInstance.UpdateTransform (Primitive.fs:131-138)
    const AABB local = I.prim_type == 1 ? AABB{Vector3(-p.radius), Vector3(p.radius)} : NodeBounds(I.mesh->nodes[0]);
    I.bounds = AABB::Transform(local, I.o2w);
    boxes[i] = I.bounds;
  }
  sc->tlas = BVHBuild(boxes, &sc->order);
  sc->inst.resize(raw.size());
  for (size_t k = 0; k < raw.size(); ++k) sc->inst[k] = raw[sc->order[k]];
  for (int i = 0; i < d->n_materials; ++i) {
    sc->mats.push_back(MaterialF::From(d->materials[i]));
    sc->mat_desc.push_back(d->materials[i]);
  }
  for (int i = 0; i < d->n_lights; ++i)
    sc->lights.push_back({Vector3(d->lights[i].emission[0], d->lights[i].emission[1], d->lights[i].emission[2]),
                          d->lights[i].two_sided != 0});
  for (size_t k = 0; k < sc->inst.size(); ++k)
    if (sc->inst[k].light >= 0) sc->light_inst.push_back(static_cast<int>(k));
  sc->light_sampler = d->light_sampler;
  if (d->light_sampler == BN_LIGHTS_ALIAS_TRIANGLES) {
    std::vector<double> w;
    for (int k : sc->light_inst) {
      Instance& I = sc->inst[k];
      const DiffuseLight& L = sc->lights[I.light];
      const double lum = 0.2126 * L.emission.X + 0.7152 * L.emission.Y + 0.0722 * L.emission.Z;
      I.light_entry_base = static_cast<int>(sc->tri_lights.size());
      for (int j = 0; j < I.mesh->n_tris(); ++j) {
        const Triangle tr = Triangle::Transform(I.mesh->Tri(j), I.o2w);
        sc->tri_lights.push_back({1.f, 0, 0.f, k, j});
        w.push_back(static_cast<double>(tr.SurfaceArea()) * std::max(lum, 0.0));
      }
    }
    BuildVose(w, &sc->tri_lights);
  }
  return sc;
}

}  // namespace orc

// ==================================================================== C API
using namespace orc;

struct or_scene {
  std::unique_ptr<Scene> s;
};

extern "C" {

int or_scene_create(const bn_scene_desc* d, or_scene** out) {
  if (!d || !out) return 1;
  auto* o = new or_scene();
  o->s = BuildScene(d);
  *out = o;
  return 0;
}
void or_scene_free(or_scene* s) { delete s; }

int or_scene_tlas(const or_scene* s, bn_bvh_node* nodes, int32_t* n_nodes, int32_t* order) {
  std::memcpy(nodes, s->s->tlas.data(), s->s->tlas.size() * sizeof(bn_bvh_node));
  *n_nodes = static_cast<int32_t>(s->s->tlas.size());
  for (size_t k = 0; k < s->s->order.size(); ++k) order[k] = s->s->order[k];
  return 0;
}
int or_scene_blas(const or_scene* s, int32_t mesh, bn_bvh_node* nodes, int32_t* n_nodes, int32_t* perm) {
  const Mesh& m = s->s->meshes[mesh];
  std::memcpy(nodes, m.nodes.data(), m.nodes.size() * sizeof(bn_bvh_node));
  *n_nodes = static_cast<int32_t>(m.nodes.size());
  for (size_t k = 0; k < m.tri_orig.size(); ++k) perm[k] = m.tri_orig[k];
  return 0;
}

int or_bvh_build(const float* bounds, int32_t n, bn_bvh_node* nodes, int32_t* n_nodes, int32_t* perm) {
  std::vector<AABB> boxes(n);
  for (int i = 0; i < n; ++i)
    boxes[i] = {Vector3(bounds[6 * i], bounds[6 * i + 1], bounds[6 * i + 2]),
                Vector3(bounds[6 * i + 3], bounds[6 * i + 4], bounds[6 * i + 5])};
  std::vector<int> p;
  auto v = BVHBuild(boxes, &p);
  std::memcpy(nodes, v.data(), v.size() * sizeof(bn_bvh_node));
  *n_nodes = static_cast<int32_t>(v.size());
  for (int i = 0; i < n; ++i) perm[i] = p[i];
  return 0;
}

int or_trace(const or_scene* os, const bn_ray* rays, int64_t n, uint32_t flags, bn_hit* hits, uint64_t* counts) {
  const Scene& sc = *os->s;
  Counters c;
  const bool wt = flags & BN_TRACE_WATERTIGHT;
  for (int64_t i = 0; i < n; ++i) {
    const bn_ray& r = rays[i];
    const Ray ray{Vector3(r.origin[0], r.origin[1], r.origin[2]), Vector3(r.direction[0], r.direction[1], r.direction[2])};
    bn_hit h{};
    if (flags & BN_TRACE_ANY) {
      h.instance = sc.Any(ray, r.t_max, wt, &c) ? 0 : -1;
      h.t = r.t_max;
      h.primitive = -1;
    } else {
      float t = r.t_max;
      Interaction it;
      if (sc.Closest(ray, &t, &it, wt, &c)) {
        h.t = t; h.u = it.geom.u; h.v = it.geom.v;
        h.instance = it.inst; h.primitive = it.tri;
        h.normal[0] = it.geom.onb.n.X; h.normal[1] = it.geom.onb.n.Y; h.normal[2] = it.geom.onb.n.Z;
        h.position[0] = it.geom.p.X; h.position[1] = it.geom.p.Y; h.position[2] = it.geom.p.Z;
      } else {
        h.t = r.t_max;
        h.instance = -1;
        h.primitive = -1;
      }
    }
    hits[i] = h;
  }
  if (counts) { counts[0] = c.rays; counts[1] = c.nodes; counts[2] = c.tris; counts[3] = c.insts; }
  return 0;
}

// Film.PostProcess (Base/Film.fs:21-30) and the Rgba32(Vector3) packing of Film.Save (:55-66):
// ImageSharp 3.1.6 (a NuGet dependency, not vendored) packs each component as
// (byte)clamp(v * 255 + 0.5, 0, 255), and .NET converts a NaN to 0.  Vector3.Clamp is
// Min(Max(x, 0), 1), whose Math semantics keep a NaN.
int or_tonemap(const float* rgb, int64_t n, int32_t tone_mapping, uint8_t* rgba) {
  auto clamp01 = [](float x) { return x != x ? x : MathMin(MathMax(x, 0.f), 1.f); };
  auto pack = [](float v) -> uint8_t {
    const float w = v * 255.f + 0.5f;
    if (w != w) return 0;
    return static_cast<uint8_t>(static_cast<int>(std::min(std::max(w, 0.f), 255.f)));
  };
  for (int64_t i = 0; i < n; ++i) {
    Vector3 x(rgb[3 * i], rgb[3 * i + 1], rgb[3 * i + 2]);
    if (tone_mapping == BN_TONE_ACES) {
      x = x * (2.51f * x + Vector3(0.03f)) / (x * (2.43f * x + Vector3(0.59f)) + Vector3(0.14f));
    } else if (tone_mapping == BN_TONE_GAMMA) {
      const float gamma = 1.f / 2.2f;
      x = Vector3(std::pow(x.X, gamma), std::pow(x.Y, gamma), std::pow(x.Z, gamma));
    } else if (tone_mapping != BN_TONE_IDENTITY) {
      return 1;
    }
    rgba[4 * i] = pack(clamp01(x.X));
    rgba[4 * i + 1] = pack(clamp01(x.Y));
    rgba[4 * i + 2] = pack(clamp01(x.Z));
    rgba[4 * i + 3] = 255;
  }
  return 0;
}

int or_sampler_stream(const uint32_t* seeds, int64_t n, int32_t draws, float* out) {
  for (int64_t i = 0; i < n; ++i) {
    Sampler s = Sampler::Three(seeds[3 * i], seeds[3 * i + 1], seeds[3 * i + 2]);
    for (int k = 0; k < draws; ++k) out[i * draws + k] = s.Next1D();
  }
  return 0;
}
uint32_t or_xxhash32_two(uint32_t x, uint32_t y) { return XXHash32Two(x, y); }
uint32_t or_xxhash32_three(uint32_t x, uint32_t y, uint32_t z) { return XXHash32Three(x, y, z); }

// BSDF eval/sample for one material description: double != 0 -> FP64 evaluation
int or_bsdf(const bn_material_desc* md, const bn_bsdf_query* q, int64_t n, int sample, int use_double, double* out7) {
  for (int64_t i = 0; i < n; ++i) {
    const bn_bsdf_query& a = q[i];
    double* o = out7 + 7 * i;
    if (use_double) {
      const Material<double> m = Material<double>::From(md[a.material]);
      const Vec3<double> wo(a.wo[0], a.wo[1], a.wo[2]);
      if (sample) {
        const auto s = m.Sample(wo, a.u_lobe, a.u_bsdf[0], a.u_bsdf[1]);
        o[0] = s.eval.bsdf.X; o[1] = s.eval.bsdf.Y; o[2] = s.eval.bsdf.Z; o[3] = s.eval.pdf;
        o[4] = s.wi.X; o[5] = s.wi.Y; o[6] = s.wi.Z;
      } else {
        const auto e = m.Eval(wo, Vec3<double>(a.wi[0], a.wi[1], a.wi[2]));
        o[0] = e.bsdf.X; o[1] = e.bsdf.Y; o[2] = e.bsdf.Z; o[3] = e.pdf;
        o[4] = a.wi[0]; o[5] = a.wi[1]; o[6] = a.wi[2];
      }
    } else {
      const MaterialF m = MaterialF::From(md[a.material]);
      const Vector3 wo(a.wo[0], a.wo[1], a.wo[2]);
      if (sample) {
        const auto s = m.Sample(wo, a.u_lobe, a.u_bsdf[0], a.u_bsdf[1]);
        o[0] = s.eval.bsdf.X; o[1] = s.eval.bsdf.Y; o[2] = s.eval.bsdf.Z; o[3] = s.eval.pdf;
        o[4] = s.wi.X; o[5] = s.wi.Y; o[6] = s.wi.Z;
      } else {
        const auto e = m.Eval(wo, Vector3(a.wi[0], a.wi[1], a.wi[2]));
        o[0] = e.bsdf.X; o[1] = e.bsdf.Y; o[2] = e.bsdf.Z; o[3] = e.pdf;
        o[4] = a.wi[0]; o[5] = a.wi[1]; o[6] = a.wi[2];
      }
    }
  }
  return 0;
}

// ProgressiveIntegrator.Render / RenderTile (Base/Integrator.fs:22-55) with PathTracingIntegrator
// (or the Normal / Direct integrator, by d->integrator):
// 16x16 tiles over `threads` workers; only tiles intersecting the crop [x0,x1) x [y0,y1) render.
// out: W*H*3 floats in Film.Pixels order (row-flipped); pixels outside the crop are left as is.
int or_render_pt(const or_scene* os, const bn_render_desc* d, const bn_view* view, int32_t x0, int32_t y0, int32_t x1,
                 int32_t y1, int32_t threads, float* out, uint64_t* counts) {
  const Scene& sc = *os->s;
  const Camera cam = Camera::From(*view);
  const int W = view->width, H = view->height;
  const int tile = 16;
  const int tx0 = x0 / tile, ty0 = y0 / tile, tx1 = (x1 + tile - 1) / tile, ty1 = (y1 + tile - 1) / tile;
  const int ntx = tx1 - tx0, nty = ty1 - ty0;
  std::atomic<int> next{0};
  const bool wt = d->flags & BN_RENDER_WATERTIGHT;
  std::vector<Counters> per(std::max(threads, 1));
  auto worker = [&](int w) {
    Counters& c = per[w];
    for (;;) {
      const int id = next.fetch_add(1);
      if (id >= ntx * nty) break;
      const int tx = tx0 + id % ntx, ty = ty0 + id / ntx;
      const float invSpp = 1.f / static_cast<float>(d->spp);
      for (int y = std::max(ty * tile, y0); y < std::min((ty + 1) * tile, std::min(y1, H)); ++y)
        for (int x = std::max(tx * tile, x0); x < std::min((tx + 1) * tile, std::min(x1, W)); ++x) {
          Vector3 acc(0.f);
          for (int s = 0; s < d->spp; ++s) {
            IndepSampler smp{Sampler::Three(static_cast<uint32_t>(x), static_cast<uint32_t>(y),
                                             static_cast<uint32_t>(d->frame_id * d->spp + s))};
            const float upx = smp.next(), upy = smp.next();
            const float ulx = smp.next(), uly = smp.next();
            const Ray ray = cam.Generate(x, y, upx, upy, ulx, uly);
            Vector3 L;
            if (d->integrator == BN_INTEGRATOR_NORMAL) L = LiNormal(sc, ray, wt, &c);
            else if (d->integrator == BN_INTEGRATOR_DIRECT) L = LiDirect(sc, ray, smp, wt, &c);
            else L = Li<false>(sc, ray, smp, d->max_depth, d->rr_depth, wt, &c);
            acc = Vector3::FusedMultiplyAdd(Vector3(invSpp), L, acc);
          }
          const size_t idx = static_cast<size_t>(H - y - 1) * W + x;
          out[3 * idx] = acc.X; out[3 * idx + 1] = acc.Y; out[3 * idx + 2] = acc.Z;
        }
    }
  };
  std::vector<std::thread> pool;
  for (int w = 0; w < std::max(threads, 1); ++w) pool.emplace_back(worker, w);
  for (auto& t : pool) t.join();
  if (counts) {
    Counters tot;
    for (const auto& c : per) { tot.rays += c.rays; tot.nodes += c.nodes; tot.tris += c.tris; tot.insts += c.insts; }
    counts[0] = tot.rays; counts[1] = tot.nodes; counts[2] = tot.tris; counts[3] = tot.insts;
  }
  return 0;
}

// Differentiable-material forward (no reference counterpart): PathTracingIntegrator.Li where
// material slots 0..emissive_base-1 are PBR materials built from `params` (values) and
// `sparams` (sampling decisions: direction, pdf, MIS, RR), and light l's emission is scaled by
// params[6 * (emissive_base + l) + 5].  With sparams == params this is the plain estimator.
int or_render_slots(const or_scene* os, const bn_render_desc* d, const bn_view* view, int32_t n_slots,
                    int32_t emissive_base, const float* params, const float* sparams, int32_t threads, float* out) {
  const Scene& sc = *os->s;
  const Camera cam = Camera::From(*view);
  const int W = view->width, H = view->height;
  auto slot_mat = [&](const float* prm, int s) {
    bn_material_desc md{};
    md.type = BN_MAT_PBR;
    md.base_color[0] = prm[6 * s]; md.base_color[1] = prm[6 * s + 1]; md.base_color[2] = prm[6 * s + 2];
    md.roughness = prm[6 * s + 3];
    md.metallic = prm[6 * s + 4];
    md.ior = 1.5f;
    return MaterialF::From(md);
  };
  auto scale_of = [&](int light) {
    const int s = emissive_base + light;
    return (light >= 0 && s < n_slots) ? params[6 * s + 5] : 1.f;
  };
  std::atomic<int> next{0};
  auto worker = [&]() {
    Counters c;
    for (;;) {
      const int row = next.fetch_add(1);
      if (row >= H) break;
      const int y = row;
      for (int x = 0; x < W; ++x) {
        Vector3 acc(0.f);
        const float invSpp = 1.f / static_cast<float>(d->spp);
        for (int si = 0; si < d->spp; ++si) {
          IndepSampler smp{Sampler::Three(static_cast<uint32_t>(x), static_cast<uint32_t>(y),
                                           static_cast<uint32_t>(d->frame_id * d->spp + si))};
          const float upx = smp.next(), upy = smp.next(), ulx = smp.next(), uly = smp.next();
          Ray ray = cam.Generate(x, y, upx, upy, ulx, uly);
          Vector3 L(0.f), beta(1.f), beta_s(1.f);
          float pdfB = 0.f;
          int depth = 0;
          while (depth < d->max_depth) {
            float t = kInf;
            Interaction it;
            if (!sc.Closest(ray, &t, &it, false, &c)) break;
            const Instance& I = sc.inst[it.inst];
            if (I.light >= 0) {
              Vector3 le;
              float pdfL;
              sc.EvalLight(ray.Origin, it, &le, &pdfL);
              const float mis = depth == 0 ? 1.f : pdfB * (1.f / (pdfL + pdfB));
              L = Vector3::FusedMultiplyAdd(beta, (scale_of(I.light) * le) * mis, L);
            }
            const int mat = sc.HitMaterial(it);
            if (mat < 0) break;
            const float uSel = smp.next(), ulx2 = smp.next(), uly2 = smp.next();
            const bool slotted = mat < emissive_base && mat < n_slots;
            const MaterialF ms = slotted ? slot_mat(sparams, mat) : sc.mats[mat];
            const MaterialF mv = slotted ? slot_mat(params, mat) : ms;
            const Vector3 wo = it.geom.onb.WorldToLocal(-ray.Direction);
            const Scene::LightSample ls = sc.SampleLight(it.geom.p, uSel, ulx2, uly2);
            const float dist = (ls.p - it.geom.p).Length();
            if (ls.pdf != 0.f && !sc.Any(Ray{it.geom.p, ls.wi}, dist - 1e-3f, false, &c)) {
              const Vector3 wi = it.geom.onb.WorldToLocal(ls.wi);
              const BSDFEvalT<float> bes = ms.Eval(wo, wi);
              const BSDFEvalT<float> bev = slotted ? mv.Eval(wo, wi) : bes;
              const Vector3 leV = scale_of(ls.light) * ls.L;
              L = Vector3::FusedMultiplyAdd(beta * bev.bsdf, leV * (1.f / (bes.pdf + ls.pdf)), L);
            }
            const float uLobe = smp.next(), ubx = smp.next(), uby = smp.next();
            const BSDFSampleT<float> bs = ms.Sample(wo, uLobe, ubx, uby);
            if (bs.eval.pdf == 0.f) break;
            const Vector3 fv = slotted ? mv.Eval(wo, bs.wi).bsdf : bs.eval.bsdf;
            pdfB = bs.eval.pdf;
            ray = {it.geom.p, it.geom.onb.LocalToWorld(bs.wi)};
            beta = beta * fv * (1.f / bs.eval.pdf);
            beta_s = beta_s * bs.eval.bsdf * (1.f / bs.eval.pdf);
            if (depth >= d->rr_depth) {
              const float q = MathMin(1.f, MathMax(beta_s.X, MathMax(beta_s.Y, beta_s.Z)));
              if (smp.next() < q) { beta = beta * (1.f / q); beta_s = beta_s * (1.f / q); }
              else break;
            }
            depth++;
          }
          acc = Vector3::FusedMultiplyAdd(Vector3(invSpp), L, acc);
        }
        const size_t idx = static_cast<size_t>(H - y - 1) * W + x;
        out[3 * idx] = acc.X; out[3 * idx + 1] = acc.Y; out[3 * idx + 2] = acc.Z;
      }
    }
  };
  std::vector<std::thread> pool;
  for (int w = 0; w < std::max(threads, 1); ++w) pool.emplace_back(worker);
  for (auto& t : pool) t.join();
  return 0;
}

// PSSMLTIntegrator.Render (PSSMLT.fs:379-414).  Chains run on `threads` workers with their own
// film copies, summed at the end (the reference's shared non-atomic film is racy).
// out: W*H*3 floats; stats: [b, accepted, proposed].  bootstrap_out (optional): n_bootstrap y.
int or_render_pssmlt(const or_scene* os, const bn_render_desc* d, const bn_view* view, int32_t threads, float* out,
                     double* stats, float* bootstrap_out) {
  const Scene& sc = *os->s;
  const Camera cam = Camera::From(*view);
  const int W = view->width, H = view->height;
  const bool wt = d->flags & BN_RENDER_WATERTIGHT;
  const int dims = 4 + 7 * d->max_depth;
  const int nb = d->n_bootstrap, nc = d->n_chains;
  const int T = std::max(threads, 1);
  std::vector<float> weights(nb);
  {
    std::atomic<int> next{0};
    auto boot = [&]() {
      Counters c;
      std::vector<PrimarySample> xs(dims);
      for (;;) {
        const int id = next.fetch_add(1);
        if (id >= nb) break;
        MLTSampler m{Sampler::Two(static_cast<uint32_t>(d->frame_id), static_cast<uint32_t>(id)), d->large_step_prob,
                     d->mutation == BN_MUTATION_KELEMEN, d->sigma, d->eps_min, d->eps_max, xs.data()};
        m.StartIteration();
        int px, py;
        const Ray ray = MltCamera(cam, m, &px, &py);
        const Vector3 L = Li<true>(sc, ray, m, d->max_depth, d->rr_depth, wt, &c) * (1.f / 1.f);
        weights[id] = Luminance(L);
      }
    };
    std::vector<std::thread> pool;
    for (int w = 0; w < T; ++w) pool.emplace_back(boot);
    for (auto& t : pool) t.join();
  }
  if (bootstrap_out) std::memcpy(bootstrap_out, weights.data(), weights.size() * sizeof(float));
  float sum = 0.f;
  for (float x : weights) sum = sum + x;
  const float B = sum / static_cast<float>(nb);
  stats[0] = B;
  const long long mpc = (static_cast<long long>(d->spp) * W * H + nc - 1) / nc;
  stats[2] = static_cast<double>(mpc) * nc;
  std::fill(out, out + 3LL * W * H, 0.f);
  if (B == 0.f) { stats[1] = 0; return 0; }
  // the AliasTable as built samples uniformly; with BN_RENDER_FIXED_ALIAS, proportionally to y
  std::vector<TriLightEntry> table;
  if (d->flags & BN_RENDER_FIXED_ALIAS) {
    std::vector<double> w(nb);
    for (int i = 0; i < nb; ++i) w[i] = weights[i] > 0.f ? weights[i] : 0.f;
    table.resize(nb);
    BuildVose(w, &table);
  }
  const float invEff = 1.f / ((static_cast<float>(mpc) * static_cast<float>(nc)) / static_cast<float>(W * H));
  const float invB = 1.f / B;
  std::atomic<int> next{0};
  std::atomic<long long> accepted{0};
  std::vector<std::vector<float>> films(T, std::vector<float>(3LL * W * H, 0.f));
  auto chains = [&](int wi) {
    Counters c;
    std::vector<PrimarySample> xs(dims);
    std::vector<float>& film = films[wi];
    auto splat = [&](int x, int y, const Vector3& v) {
      const size_t i = static_cast<size_t>(H - y - 1) * W + x;
      film[3 * i] += v.X; film[3 * i + 1] += v.Y; film[3 * i + 2] += v.Z;
    };
    long long acc_local = 0;
    for (;;) {
      const int chain = next.fetch_add(1);
      if (chain >= nc) break;
      Sampler cs = Sampler::Two(static_cast<uint32_t>(d->frame_id), static_cast<uint32_t>(chain));
      float u = cs.Next1D() * static_cast<float>(nb);
      int bid = std::min(static_cast<int>(u), nb - 1);
      if (!table.empty() && u - static_cast<float>(bid) >= table[bid].prob) bid = table[bid].alias;
      MLTSampler m{Sampler::Two(static_cast<uint32_t>(d->frame_id), static_cast<uint32_t>(bid)), d->large_step_prob,
                   d->mutation == BN_MUTATION_KELEMEN, d->sigma, d->eps_min, d->eps_max, xs.data()};
      m.StartIteration();
      int px, py;
      Ray ray = MltCamera(cam, m, &px, &py);
      Vector3 L = Li<true>(sc, ray, m, d->max_depth, d->rr_depth, wt, &c) * (1.f / 1.f);
      float y = Luminance(L);
      m.Accept();
      m.Inner = Sampler::Three(static_cast<uint32_t>(chain), static_cast<uint32_t>(bid), static_cast<uint32_t>(d->frame_id));
      Vector3 radiance(0.f);
      for (long long it = 0; it < mpc; ++it) {
        m.StartIteration();
        int nx, ny;
        ray = MltCamera(cam, m, &nx, &ny);
        const Vector3 Ln = Li<true>(sc, ray, m, d->max_depth, d->rr_depth, wt, &c) * (1.f / 1.f);
        const float yn = Luminance(Ln);
        const float accept = MathMin(1.f, yn / y);
        const float wOld = (1.f - accept) / std::fma(y, invB, d->large_step_prob);
        radiance = radiance + wOld * L;
        const float wNew = (accept + (m.LargeStep ? 1.f : 0.f)) / std::fma(yn, invB, d->large_step_prob);
        if (cs.Next1D() < accept) {
          ++acc_local;
          splat(px, py, radiance * invEff);
          radiance = wNew * Ln;
          px = nx; py = ny;
          L = Ln;
          y = yn;
          m.Accept();
        } else {
          if (accept > 0.f) splat(nx, ny, (wNew * invEff) * Ln);
          m.Reject();
        }
      }
      splat(px, py, radiance * invEff);
    }
    accepted += acc_local;
  };
  std::vector<std::thread> pool;
  for (int w = 0; w < T; ++w) pool.emplace_back(chains, w);
  for (auto& t : pool) t.join();
  for (int w = 0; w < T; ++w)
    for (size_t i = 0; i < films[w].size(); ++i) out[i] += films[w][i];
  stats[1] = static_cast<double>(accepted.load());
  return 0;
}

}  // extern "C"
