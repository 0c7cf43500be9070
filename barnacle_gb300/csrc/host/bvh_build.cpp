// Reference-compatible binned SAH builder.
//
// Produces exactly the node array and item permutation of BVHNode.Build (Util/BVH.fs:239-247):
//   * 12 bins, leaves of <= 4 items, depth cut at 64            (Util/BVH.fs:99-107)
//   * split axis = longest centroid-bounds axis; median split when its extent is 0 (:147-156)
//   * bin = min(11, int(12 * (c - cmin) / extent))                                  (:163-169)
//     with .NET 9's saturating conversion (NaN -> 0), which infinite boxes reach
//   * cost[i] = SAH(bins 0..i) + SAH(bins i+1..11) + n * SA(centroid bounds)        (:179-203)
//   * unstable partition: items in bins > best fill from the end, the rest from the front,
//     both read from a copy of the subrange                                          (:205-217)
//   * nodes in preorder, left child at i+1, right child index stored                 (:224-237)
// Instead of building a tree of F# objects and flattening it, the nodes are emitted in preorder
// while the recursion runs (the order is the same), and one scratch array replaces the per-node
// subarray copies.  Float operations follow the reference order; compile with -ffp-contract=off.
#include <cstdint>
#include <limits>
#include <vector>

#include "bvh_build.hpp"

namespace bnh {
namespace {

constexpr int kBins = 12;
constexpr int kMaxLeaf = 4;
constexpr int kMaxDepth = 64;

struct Box {
  V3 lo, hi;
};
static inline Box box_empty() {
  const float inf = std::numeric_limits<float>::infinity();
  return {{inf, inf, inf}, {-inf, -inf, -inf}};
}
static inline Box box_union(const Box& a, const Box& b) {
  return {min_native(a.lo, b.lo), max_native(a.hi, b.hi)};
}
static inline Box box_union(const Box& a, V3 p) { return {min_native(a.lo, p), max_native(a.hi, p)}; }
static inline V3 centroid(const Box& b) { return 0.5f * (b.lo + b.hi); }
static inline float surface_area(const Box& b) {
  V3 d = b.hi - b.lo;
  return 2.f * ((d.x * d.y + d.y * d.z) + d.z * d.x);
}
// float -> int32 as .NET 9 converts: truncation, saturated at the int range, NaN -> 0
static inline int saturating_int(float f) {
  if (f != f) return 0;
  if (f >= 2147483647.f) return 2147483647;
  if (f <= -2147483648.f) return -2147483647 - 1;
  return static_cast<int>(f);
}
static inline int split_axis(const Box& b) {
  V3 d = b.hi - b.lo;
  if (d.x >= d.y && d.x >= d.z) return 0;
  return d.y >= d.z ? 1 : 2;
}

struct Item {
  Box box;
  int32_t index;
};

struct Builder {
  std::vector<Item>& items;
  std::vector<Item> scratch;
  std::vector<bn_bvh_node>& nodes;
  bool count_overflow = false;

  int emit_leaf(const Box& b, int first, int count) {
    bn_bvh_node n{};
    n.bounds_min[0] = b.lo.x; n.bounds_min[1] = b.lo.y; n.bounds_min[2] = b.lo.z;
    n.bounds_max[0] = b.hi.x; n.bounds_max[1] = b.hi.y; n.bounds_max[2] = b.hi.z;
    n.right_or_offset = first;
    n.is_leaf = 1;
    n.count = static_cast<int8_t>(count);
    if (count > 127) count_overflow = true;
    nodes.push_back(n);
    return static_cast<int>(nodes.size()) - 1;
  }

  int build(int first, int last, int depth) {
    const int count = last - first;
    Box bounds = box_empty();
    for (int i = first; i < last; ++i) bounds = box_union(bounds, items[i].box);
    if (count <= kMaxLeaf || depth >= kMaxDepth) return emit_leaf(bounds, first, count);

    Box cb = box_empty();
    for (int i = first; i < last; ++i) cb = box_union(cb, centroid(items[i].box));
    const int axis = split_axis(cb);
    const float extent = comp(cb.hi - cb.lo, axis);

    const int self = static_cast<int>(nodes.size());
    nodes.push_back(bn_bvh_node{});
    int right_child;
    if (extent == 0.f) {
      const int mid = first + count / 2;
      build(first, mid, depth + 1);
      right_child = build(mid, last, depth + 1);
    } else {
      const float cmin = comp(cb.lo, axis);
      auto bin_of = [&](const Box& b) {
        // .NET's saturating float -> int conversion: a NaN (inf - inf with infinite boxes) is 0
        int k = saturating_int((static_cast<float>(kBins) * (comp(centroid(b), axis) - cmin)) / extent);
        return k < kBins - 1 ? k : kBins - 1;
      };
      Box bin_box[kBins];
      int bin_cnt[kBins];
      for (int k = 0; k < kBins; ++k) { bin_box[k] = box_empty(); bin_cnt[k] = 0; }
      // the subrange copy that the partition reads from (Util/BVH.fs:130)
      scratch.assign(items.begin() + first, items.begin() + last);
      for (int i = 0; i < count; ++i) {
        const int k = bin_of(scratch[i].box);
        bin_box[k] = box_union(bin_box[k], scratch[i].box);
        bin_cnt[k] += 1;
      }
      float costs[kBins - 1];
      for (int i = 0; i < kBins - 1; ++i) costs[i] = 0.f;
      Box lb = box_empty(), rb = box_empty();
      int lc = 0, rc = 0;
      const int nc = kBins - 1;
      for (int i = 0; i < nc; ++i) {
        lb = box_union(lb, bin_box[i]);
        lc += bin_cnt[i];
        costs[i] = costs[i] + static_cast<float>(lc) * surface_area(lb);
        rb = box_union(rb, bin_box[nc - i]);
        rc += bin_cnt[nc - i];
        costs[nc - 1 - i] = costs[nc - 1 - i] + static_cast<float>(rc) * surface_area(rb);
      }
      float min_cost = std::numeric_limits<float>::infinity();
      int best = 0;
      const float base = static_cast<float>(count) * surface_area(cb);
      for (int i = 0; i < nc; ++i) {
        const float c = costs[i] + base;
        if (c < min_cost) { min_cost = c; best = i; }
      }
      int left = first, right = last - 1;
      for (int i = 0; i < count; ++i) {
        const Item it = scratch[i];
        if (bin_of(it.box) > best) items[right--] = it;
        else items[left++] = it;
      }
      const int split_left = left, split_right = right + 1;
      build(first, split_left, depth + 1);
      right_child = build(split_right, last, depth + 1);
    }
    bn_bvh_node n{};
    n.bounds_min[0] = bounds.lo.x; n.bounds_min[1] = bounds.lo.y; n.bounds_min[2] = bounds.lo.z;
    n.bounds_max[0] = bounds.hi.x; n.bounds_max[1] = bounds.hi.y; n.bounds_max[2] = bounds.hi.z;
    n.right_or_offset = right_child;
    n.is_leaf = 0;
    n.split_axis = static_cast<int8_t>(axis);
    nodes[self] = n;
    return self;
  }
};

}  // namespace

bool bvh_build(const float* bounds, int32_t n, std::vector<bn_bvh_node>* nodes, std::vector<int32_t>* perm) {
  nodes->clear();
  perm->assign(n, 0);
  if (n <= 0) {
    // BVHNode.Build on an empty span yields one empty leaf (Tree.Build with count 0).
    std::vector<Item> none;
    Builder b{none, {}, *nodes};
    b.emit_leaf(box_empty(), 0, 0);
    return true;
  }
  std::vector<Item> items(n);
  for (int32_t i = 0; i < n; ++i) {
    const float* p = bounds + 6 * static_cast<size_t>(i);
    items[i].box = {{p[0], p[1], p[2]}, {p[3], p[4], p[5]}};
    items[i].index = i;
  }
  nodes->reserve(2 * static_cast<size_t>(n));
  Builder b{items, {}, *nodes};
  b.scratch.reserve(n);
  b.build(0, n, 0);
  for (int32_t i = 0; i < n; ++i) (*perm)[i] = items[i].index;
  // a leaf count is stored in an int8 (Util/BVH.fs:70); refuse trees it cannot hold
  return !b.count_overflow;
}

}  // namespace bnh
