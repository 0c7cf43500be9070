// GPU BVH builder, host side: the per-node decisions of BVHNode.Build (Util/BVH.fs:99-247) for
// the large node ranges, made level by level from the device reductions of k_bvh.cu, then one
// device thread per small range, then the preorder assembly.  The result equals the host
// builder's (csrc/host/bvh_build.cpp) node for node and in the item permutation.
//
// Per level: chunk lists (256 items of one range) go up; the bounds/centroid reduction, the 12
// SAH bins and the per-chunk left counts come back; the host takes the reference's decisions
// (leaf at depth 64, median split when the centroid extent is 0, else the cheapest of the 11
// bin splits with the reference's float arithmetic) and the stable partition runs on the device.
// Ranges of at most `small` items are finished by k_bvh_small.  Boxes with a NaN coordinate,
// where the fold's order decides the bounds, are built by the host builder instead.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <functional>
#include <string>
#include <vector>

#include "../device/bvh_gpu.hpp"
#include "../host/bvh_build.hpp"
#include "context.hpp"

namespace {

unsigned f2o(float f) {
  unsigned u;
  std::memcpy(&u, &f, 4);
  return (u & 0x80000000u) ? ~u : (u | 0x80000000u);
}
float o2f(unsigned o) {
  const unsigned u = (o & 0x80000000u) ? (o & 0x7fffffffu) : ~o;
  float f;
  std::memcpy(&f, &u, 4);
  return f;
}

struct HBox {
  bnh::V3 lo, hi;
};
HBox hbox_empty() {
  const float inf = std::numeric_limits<float>::infinity();
  return {{inf, inf, inf}, {-inf, -inf, -inf}};
}
HBox hunion(const HBox& a, const HBox& b) { return {bnh::min_native(a.lo, b.lo), bnh::max_native(a.hi, b.hi)}; }
float harea(const HBox& b) {
  const bnh::V3 d = b.hi - b.lo;
  return 2.f * ((d.x * d.y + d.y * d.z) + d.z * d.x);
}

struct TopNode {
  bn_bvh_node node{};
  int left = 0, right = 0;  // >= 0: top node; < 0: -(1 + small range)
};
struct Range {
  int first, last, depth, parent, side;
};

template <class T>
cudaError_t put(DevBuf& b, const std::vector<T>& v, cudaStream_t st) {
  cudaError_t e = b.reserve(std::max<size_t>(v.size() * sizeof(T), 16));
  if (e == cudaSuccess && !v.empty()) e = cudaMemcpyAsync(b.ptr, v.data(), v.size() * sizeof(T), cudaMemcpyHostToDevice, st);
  return e;
}
template <class T>
cudaError_t get(std::vector<T>* v, const DevBuf& b, size_t n, cudaStream_t st) {
  v->resize(n);
  cudaError_t e = n ? cudaMemcpyAsync(v->data(), b.ptr, n * sizeof(T), cudaMemcpyDeviceToHost, st) : cudaSuccess;
  if (e == cudaSuccess) e = cudaStreamSynchronize(st);
  return e;
}

}  // namespace

namespace bnc {

// nodes / perm as bnh::bvh_build; returns BN_OK, BN_ERR_UNSUPPORTED (a leaf over 127 items) or a
// CUDA error, with the message in ctx->err
int gpu_bvh_build(bn_context* ctx, const float* bounds, int32_t n, std::vector<bn_bvh_node>* nodes,
                  std::vector<int32_t>* perm, int small) {
  for (int64_t i = 0; i < 6LL * n; ++i)
    if (std::isnan(bounds[i])) {
      if (!bnh::bvh_build(bounds, n, nodes, perm)) return ctx->fail(BN_ERR_UNSUPPORTED, "BVH leaf larger than 127 items");
      return BN_OK;
    }
  if (n <= 0) {
    bnh::bvh_build(bounds, n, nodes, perm);
    return BN_OK;
  }
  small = std::max(small, 4);
  cudaStream_t st = ctx->stream;
  DevBuf items, out, chunks_d, acc, bounds_d, sah_d, bins_d, left_d, base_d, smalls_d, snodes, scounts, flag;
  struct Guard {
    std::vector<DevBuf*> b;
    ~Guard() {
      for (DevBuf* x : b) x->release();
    }
  } guard{{&items, &out, &chunks_d, &acc, &bounds_d, &sah_d, &bins_d, &left_d, &base_d, &smalls_d, &snodes,
           &scounts, &flag}};
  cudaError_t e;
  {
    std::vector<bn::BvhItem> h(n);
    for (int i = 0; i < n; ++i) {
      const float* b = bounds + 6 * static_cast<size_t>(i);
      float idx;
      std::memcpy(&idx, &i, 4);
      h[i].a = make_float4(b[0], b[1], b[2], idx);
      h[i].b = make_float4(b[3], b[4], b[5], 0.f);
    }
    if ((e = put(items, h, st)) != cudaSuccess) return ctx->cuda_fail(e, "BVH items");
    if ((e = out.reserve(h.size() * sizeof(bn::BvhItem))) != cudaSuccess) return ctx->cuda_fail(e, "BVH items");
  }
  std::vector<TopNode> top;
  std::vector<bn::BvhSmall> smalls;
  int root = 0;
  auto link = [&](int parent, int side, int ref) {
    if (parent < 0) root = ref;
    else if (side) top[parent].right = ref;
    else top[parent].left = ref;
  };
  std::vector<Range> level;
  auto add_range = [&](const Range& r) {
    if (r.last - r.first > small) {
      level.push_back(r);
    } else {
      link(r.parent, r.side, -1 - static_cast<int>(smalls.size()));
      smalls.push_back({r.first, r.last, r.depth, 0});
    }
  };
  add_range({0, n, 0, -1, 0});
  while (!level.empty()) {
    const std::vector<Range> cur = std::move(level);
    level.clear();
    std::vector<bn::BvhChunk> ch;
    for (size_t s = 0; s < cur.size(); ++s)
      for (int b = cur[s].first; b < cur[s].last; b += 256)
        ch.push_back({static_cast<int>(s), b, std::min(b + 256, cur[s].last), 0});
    const int ns = static_cast<int>(cur.size()), nch = static_cast<int>(ch.size());
    if ((e = put(chunks_d, ch, st)) != cudaSuccess || (e = acc.reserve(ns * sizeof(bn::BvhSegAcc))) != cudaSuccess ||
        (e = bounds_d.reserve(ns * 12 * sizeof(float))) != cudaSuccess ||
        (e = bn::bvh_launch_init_acc(acc.as<bn::BvhSegAcc>(), ns, st)) != cudaSuccess ||
        (e = bn::bvh_launch_reduce(items.as<bn::BvhItem>(), chunks_d.as<bn::BvhChunk>(), nch, acc.as<bn::BvhSegAcc>(),
                                   st)) != cudaSuccess ||
        (e = bn::bvh_launch_finalize(items.as<bn::BvhItem>(), acc.as<bn::BvhSegAcc>(), ns, bounds_d.as<float>(), st)) !=
            cudaSuccess)
      return ctx->cuda_fail(e, "BVH bounds");
    std::vector<float> b12;
    if ((e = get(&b12, bounds_d, static_cast<size_t>(ns) * 12, st)) != cudaSuccess) return ctx->cuda_fail(e, "BVH bounds");
    std::vector<bn::BvhSah> sah;
    std::vector<int> sah_top, sah_range;
    for (int s = 0; s < ns; ++s) {
      const Range& r = cur[s];
      const float* b = &b12[12 * static_cast<size_t>(s)];
      const int t = static_cast<int>(top.size());
      top.push_back({});
      link(r.parent, r.side, t);
      bn_bvh_node& nd = top[t].node;
      for (int k = 0; k < 3; ++k) {
        nd.bounds_min[k] = b[k];
        nd.bounds_max[k] = b[3 + k];
      }
      const int count = r.last - r.first;
      if (r.depth >= 64) {
        if (count > 127) return ctx->fail(BN_ERR_UNSUPPORTED, "BVH leaf larger than 127 items");
        nd.right_or_offset = r.first;
        nd.is_leaf = 1;
        nd.count = static_cast<int8_t>(count);
        continue;
      }
      const bnh::V3 clo = {b[6], b[7], b[8]}, chi = {b[9], b[10], b[11]};
      const bnh::V3 d = chi - clo;
      const int axis = (d.x >= d.y && d.x >= d.z) ? 0 : (d.y >= d.z ? 1 : 2);
      const float extent = bnh::comp(d, axis);
      nd.split_axis = static_cast<int8_t>(axis);
      if (extent == 0.f) {
        const int mid = r.first + count / 2;
        add_range({r.first, mid, r.depth + 1, t, 0});
        add_range({mid, r.last, r.depth + 1, t, 1});
        continue;
      }
      sah.push_back({r.first, r.last, axis, -1, bnh::comp(clo, axis), extent, 0, 0});
      sah_top.push_back(t);
      sah_range.push_back(s);
    }
    if (sah.empty()) continue;
    // bins of the SAH ranges
    const int nh = static_cast<int>(sah.size());
    std::vector<bn::BvhChunk> hc;
    for (int h = 0; h < nh; ++h)
      for (int b = sah[h].first; b < sah[h].last; b += 256) hc.push_back({h, b, std::min(b + 256, sah[h].last), 0});
    const int nhc = static_cast<int>(hc.size());
    if ((e = put(sah_d, sah, st)) != cudaSuccess || (e = put(chunks_d, hc, st)) != cudaSuccess ||
        (e = bins_d.reserve(static_cast<size_t>(nh) * bn::kBvhBins * sizeof(bn::BvhBin))) != cudaSuccess ||
        (e = bn::bvh_launch_init_bins(bins_d.as<bn::BvhBin>(), nh * bn::kBvhBins, st)) != cudaSuccess ||
        (e = bn::bvh_launch_bins(items.as<bn::BvhItem>(), chunks_d.as<bn::BvhChunk>(), nhc, sah_d.as<bn::BvhSah>(),
                                 bins_d.as<bn::BvhBin>(), st)) != cudaSuccess)
      return ctx->cuda_fail(e, "BVH bins");
    std::vector<bn::BvhBin> bins;
    if ((e = get(&bins, bins_d, static_cast<size_t>(nh) * bn::kBvhBins, st)) != cudaSuccess)
      return ctx->cuda_fail(e, "BVH bins");
    std::vector<int> n_left(nh);
    for (int h = 0; h < nh; ++h) {
      // the reference's costs (Util/BVH.fs:179-203) from the bin boxes and counts
      HBox bb[bn::kBvhBins];
      int cnt[bn::kBvhBins];
      for (int k = 0; k < bn::kBvhBins; ++k) {
        const bn::BvhBin& x = bins[static_cast<size_t>(h) * bn::kBvhBins + k];
        bb[k] = {{o2f(x.lo[0]), o2f(x.lo[1]), o2f(x.lo[2])}, {o2f(x.hi[0]), o2f(x.hi[1]), o2f(x.hi[2])}};
        cnt[k] = x.cnt;
      }
      constexpr int nc = bn::kBvhBins - 1;
      float costs[nc];
      for (int i = 0; i < nc; ++i) costs[i] = 0.f;
      HBox lb = hbox_empty(), rb = hbox_empty();
      int lc = 0, rc = 0;
      for (int i = 0; i < nc; ++i) {
        lb = hunion(lb, bb[i]);
        lc += cnt[i];
        costs[i] = costs[i] + static_cast<float>(lc) * harea(lb);
        rb = hunion(rb, bb[nc - i]);
        rc += cnt[nc - i];
        costs[nc - 1 - i] = costs[nc - 1 - i] + static_cast<float>(rc) * harea(rb);
      }
      const float* b = &b12[12 * static_cast<size_t>(sah_range[h])];
      const HBox cb = {{b[6], b[7], b[8]}, {b[9], b[10], b[11]}};
      const float base = static_cast<float>(sah[h].last - sah[h].first) * harea(cb);
      float min_cost = std::numeric_limits<float>::infinity();
      int best = 0;
      for (int i = 0; i < nc; ++i) {
        const float c = costs[i] + base;
        if (c < min_cost) {
          min_cost = c;
          best = i;
        }
      }
      sah[h].best = best;
      int l = 0;
      for (int k = 0; k <= best; ++k) l += cnt[k];
      n_left[h] = l;
    }
    // stable partition: per-chunk left counts, their prefix within each range, then the scatter
    if ((e = put(sah_d, sah, st)) != cudaSuccess || (e = left_d.reserve(nhc * sizeof(int))) != cudaSuccess ||
        (e = bn::bvh_launch_count_left(items.as<bn::BvhItem>(), chunks_d.as<bn::BvhChunk>(), nhc,
                                       sah_d.as<bn::BvhSah>(), left_d.as<int>(), st)) != cudaSuccess)
      return ctx->cuda_fail(e, "BVH partition");
    std::vector<int> cl;
    if ((e = get(&cl, left_d, nhc, st)) != cudaSuccess) return ctx->cuda_fail(e, "BVH partition");
    std::vector<int> cbase(nhc);
    for (int c = 0, run = 0; c < nhc; ++c) {
      if (c == 0 || hc[c].seg != hc[c - 1].seg) run = 0;
      cbase[c] = run;
      run += cl[c];
    }
    if ((e = put(base_d, cbase, st)) != cudaSuccess ||
        (e = bn::bvh_launch_partition(items.as<bn::BvhItem>(), out.as<bn::BvhItem>(), chunks_d.as<bn::BvhChunk>(), nhc,
                                      sah_d.as<bn::BvhSah>(), base_d.as<int>(), st)) != cudaSuccess ||
        (e = bn::bvh_launch_copy(items.as<bn::BvhItem>(), out.as<bn::BvhItem>(), chunks_d.as<bn::BvhChunk>(), nhc, st)) !=
            cudaSuccess)
      return ctx->cuda_fail(e, "BVH partition");
    for (int h = 0; h < nh; ++h) {
      const Range& r = cur[sah_range[h]];
      const int split = r.first + n_left[h];
      add_range({r.first, split, r.depth + 1, sah_top[h], 0});
      add_range({split, r.last, r.depth + 1, sah_top[h], 1});
    }
  }
  // small ranges, one thread each
  long long total = 0;
  for (auto& s : smalls) {
    s.node_base = static_cast<int>(total);
    total += 2LL * (s.last - s.first) + 1;
  }
  if (total > (1LL << 31) - 1) return ctx->fail(BN_ERR_UNSUPPORTED, "BVH too large");
  const int nsm = static_cast<int>(smalls.size());
  int overflow = 0;
  if ((e = put(smalls_d, smalls, st)) != cudaSuccess ||
      (e = snodes.reserve(std::max<size_t>(total, 1) * sizeof(bn_bvh_node))) != cudaSuccess ||
      (e = scounts.reserve(std::max(nsm, 1) * sizeof(int))) != cudaSuccess ||
      (e = flag.reserve(sizeof(int))) != cudaSuccess ||
      (e = cudaMemsetAsync(flag.ptr, 0, sizeof(int), st)) != cudaSuccess ||
      (e = bn::bvh_launch_small(items.as<bn::BvhItem>(), out.as<bn::BvhItem>(), smalls_d.as<bn::BvhSmall>(), nsm,
                                snodes.as<bn_bvh_node>(), scounts.as<int>(), flag.as<int>(), st)) != cudaSuccess ||
      (e = cudaMemcpyAsync(&overflow, flag.ptr, sizeof(int), cudaMemcpyDeviceToHost, st)) != cudaSuccess)
    return ctx->cuda_fail(e, "BVH small ranges");
  std::vector<int> counts;
  std::vector<bn_bvh_node> sn;
  std::vector<bn::BvhItem> fin;
  if ((e = get(&counts, scounts, nsm, st)) != cudaSuccess || (e = get(&sn, snodes, total, st)) != cudaSuccess ||
      (e = get(&fin, items, n, st)) != cudaSuccess)
    return ctx->cuda_fail(e, "BVH download");
  if (overflow) return ctx->fail(BN_ERR_UNSUPPORTED, "BVH leaf larger than 127 items");
  // preorder assembly: a top node, its left subtree, its right subtree
  nodes->clear();
  nodes->reserve(top.size() + static_cast<size_t>(total));
  std::function<int(int)> emit = [&](int ref) -> int {
    const int at = static_cast<int>(nodes->size());
    if (ref < 0) {
      const bn::BvhSmall& s = smalls[-1 - ref];
      for (int k = 0; k < counts[-1 - ref]; ++k) {
        bn_bvh_node x = sn[static_cast<size_t>(s.node_base) + k];
        if (!x.is_leaf) x.right_or_offset += at;
        nodes->push_back(x);
      }
      return at;
    }
    nodes->push_back(top[ref].node);
    if (!top[ref].node.is_leaf) {
      emit(top[ref].left);
      const int r = emit(top[ref].right);
      (*nodes)[at].right_or_offset = r;
    }
    return at;
  };
  emit(root);
  perm->resize(n);
  for (int i = 0; i < n; ++i) std::memcpy(&(*perm)[i], &fin[i].a.w, 4);
  return BN_OK;
}

}  // namespace bnc

extern "C" int bn_bvh_build_device(bn_context* ctx, const float* bounds, int32_t n, bn_bvh_node* nodes,
                                   int32_t* n_nodes, int32_t* perm) {
  if (!ctx) return BN_ERR_INVALID_ARG;
  if ((!bounds && n > 0) || !nodes || !n_nodes || (!perm && n > 0) || n < 0)
    return ctx->fail(BN_ERR_INVALID_ARG, "bn_bvh_build_device: null pointer or negative count");
  cudaSetDevice(ctx->device);
  std::vector<bn_bvh_node> nv;
  std::vector<int32_t> pv;
  const int rc = bnc::gpu_bvh_build(ctx, bounds, n, &nv, &pv, 256);
  if (rc) return rc;
  std::copy(nv.begin(), nv.end(), nodes);
  *n_nodes = static_cast<int32_t>(nv.size());
  std::copy(pv.begin(), pv.end(), perm);
  return BN_OK;
}
