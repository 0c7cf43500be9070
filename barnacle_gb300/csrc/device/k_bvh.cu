// GPU BVH builder kernels: the binned SAH build of BVHNode.Build (Util/BVH.fs:99-247) with the
// reference's results.  Large node ranges are processed level by level (chunked reductions of
// bounds, centroid bounds and bins, then a stable partition); small ranges are finished by one
// thread each, running the reference's sequential algorithm.
//
// Exactness.  Every float operation is written with _rn intrinsics in the reference's order (no
// contraction).  Bounds are reduced as order-preserving unsigned encodings, which give the same
// value as the reference's sequential MinNative/MaxNative fold for finite boxes; the one thing an
// order-free reduction loses is the sign of a zero bound (the fold keeps the last item that
// compares equal), so the reduction also records the last item with a zero coordinate and the
// finalisation takes its sign.  Centroid and bin bounds only feed differences and comparisons,
// where the sign of a zero does not matter.  The partition keeps the reference's order: items of
// bins <= best fill the range from the front in their order, the others from the back.
#include <math_constants.h>

#include <cstdint>

#include "bvh_gpu.hpp"

namespace bn {
namespace {

__device__ __forceinline__ unsigned f2o(float f) {
  const unsigned u = __float_as_uint(f);
  return (u & 0x80000000u) ? ~u : (u | 0x80000000u);
}
__device__ __forceinline__ float o2f(unsigned o) {
  return __uint_as_float((o & 0x80000000u) ? (o & 0x7fffffffu) : ~o);
}
__device__ __forceinline__ float cen(float lo, float hi) { return __fmul_rn(0.5f, __fadd_rn(lo, hi)); }
__device__ __forceinline__ float comp4(const float4& v, int a) { return a == 0 ? v.x : (a == 1 ? v.y : v.z); }
__device__ __forceinline__ float min_native(float a, float b) { return a < b ? a : b; }
__device__ __forceinline__ float max_native(float a, float b) { return a > b ? a : b; }

// bin = min(11, int(12 * (c - cmin) / extent))  (Util/BVH.fs:163-169)
__device__ __forceinline__ int bin_of(const BvhItem& it, int axis, float cmin, float extent) {
  const float c = cen(comp4(it.a, axis), comp4(it.b, axis));
  const int k = __float2int_rz(__fdiv_rn(__fmul_rn(12.f, __fsub_rn(c, cmin)), extent));
  return k < kBvhBins - 1 ? k : kBvhBins - 1;
}

__global__ void __launch_bounds__(256) k_bvh_init_acc(BvhSegAcc* acc, int n) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  BvhSegAcc a;
  for (int k = 0; k < 3; ++k) {
    a.lo[k] = a.clo[k] = f2o(CUDART_INF_F);
    a.hi[k] = a.chi[k] = f2o(-CUDART_INF_F);
    a.zlo[k] = a.zhi[k] = -1;
  }
  acc[i] = a;
}

__global__ void __launch_bounds__(256) k_bvh_init_bins(BvhBin* bins, int n) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  BvhBin b;
  for (int k = 0; k < 3; ++k) {
    b.lo[k] = f2o(CUDART_INF_F);
    b.hi[k] = f2o(-CUDART_INF_F);
  }
  b.cnt = 0;
  b.pad = 0;
  bins[i] = b;
}

__global__ void __launch_bounds__(256) k_bvh_reduce(const BvhItem* __restrict__ items, const BvhChunk* __restrict__ chunks,
                                                    BvhSegAcc* acc) {
  __shared__ unsigned s[12];
  __shared__ int z[6];
  const BvhChunk c = chunks[blockIdx.x];
  if (threadIdx.x < 12) s[threadIdx.x] = (threadIdx.x % 6) < 3 ? f2o(CUDART_INF_F) : f2o(-CUDART_INF_F);
  if (threadIdx.x < 6) z[threadIdx.x] = -1;
  __syncthreads();
  const int i = c.begin + threadIdx.x;
  if (i < c.end) {
    const BvhItem it = items[i];
    const float lo[3] = {it.a.x, it.a.y, it.a.z}, hi[3] = {it.b.x, it.b.y, it.b.z};
    for (int k = 0; k < 3; ++k) {
      atomicMin(&s[k], f2o(lo[k]));
      atomicMax(&s[3 + k], f2o(hi[k]));
      const float cc = cen(lo[k], hi[k]);
      atomicMin(&s[6 + k], f2o(cc));
      atomicMax(&s[9 + k], f2o(cc));
      if (lo[k] == 0.f) atomicMax(&z[k], i);
      if (hi[k] == 0.f) atomicMax(&z[3 + k], i);
    }
  }
  __syncthreads();
  BvhSegAcc* a = acc + c.seg;
  const int t = threadIdx.x;
  if (t < 3) {
    atomicMin(&a->lo[t], s[t]);
  } else if (t < 6) {
    atomicMax(&a->hi[t - 3], s[t]);
  } else if (t < 9) {
    atomicMin(&a->clo[t - 6], s[t]);
  } else if (t < 12) {
    atomicMax(&a->chi[t - 9], s[t]);
  } else if (t < 15) {
    if (z[t - 12] >= 0) atomicMax(&a->zlo[t - 12], z[t - 12]);
  } else if (t < 18) {
    if (z[t - 12] >= 0) atomicMax(&a->zhi[t - 15], z[t - 12]);
  }
}

// bounds12 per range: box lo/hi with the fold's zero signs, centroid lo/hi
__global__ void __launch_bounds__(256) k_bvh_finalize(const BvhItem* __restrict__ items, const BvhSegAcc* __restrict__ acc,
                                                      int n, float* __restrict__ out) {
  const int s = blockIdx.x * blockDim.x + threadIdx.x;
  if (s >= n) return;
  const BvhSegAcc a = acc[s];
  float* o = out + 12 * s;
  for (int k = 0; k < 3; ++k) {
    float lo = o2f(a.lo[k]), hi = o2f(a.hi[k]);
    if (lo == 0.f && a.zlo[k] >= 0) lo = comp4(items[a.zlo[k]].a, k);
    if (hi == 0.f && a.zhi[k] >= 0) hi = comp4(items[a.zhi[k]].b, k);
    o[k] = lo;
    o[3 + k] = hi;
    o[6 + k] = o2f(a.clo[k]);
    o[9 + k] = o2f(a.chi[k]);
  }
}

__global__ void __launch_bounds__(256) k_bvh_bins(const BvhItem* __restrict__ items, const BvhChunk* __restrict__ chunks,
                                                  const BvhSah* __restrict__ sah, BvhBin* bins) {
  __shared__ unsigned lo[kBvhBins][3], hi[kBvhBins][3];
  __shared__ int cnt[kBvhBins];
  const BvhChunk c = chunks[blockIdx.x];
  const BvhSah h = sah[c.seg];
  const int t = threadIdx.x;
  if (t < kBvhBins * 3) {
    lo[t / 3][t % 3] = f2o(CUDART_INF_F);
    hi[t / 3][t % 3] = f2o(-CUDART_INF_F);
  }
  if (t < kBvhBins) cnt[t] = 0;
  __syncthreads();
  const int i = c.begin + t;
  if (i < c.end) {
    const BvhItem it = items[i];
    const int k = bin_of(it, h.axis, h.cmin, h.extent);
    atomicAdd(&cnt[k], 1);
    atomicMin(&lo[k][0], f2o(it.a.x));
    atomicMin(&lo[k][1], f2o(it.a.y));
    atomicMin(&lo[k][2], f2o(it.a.z));
    atomicMax(&hi[k][0], f2o(it.b.x));
    atomicMax(&hi[k][1], f2o(it.b.y));
    atomicMax(&hi[k][2], f2o(it.b.z));
  }
  __syncthreads();
  BvhBin* b = bins + kBvhBins * c.seg;
  if (t < kBvhBins * 3) {
    const int k = t / 3, a = t % 3;
    if (cnt[k]) {
      atomicMin(&b[k].lo[a], lo[k][a]);
      atomicMax(&b[k].hi[a], hi[k][a]);
    }
  } else if (t < kBvhBins * 4) {
    const int k = t - kBvhBins * 3;
    if (cnt[k]) atomicAdd(&b[k].cnt, cnt[k]);
  }
}

__global__ void __launch_bounds__(256) k_bvh_count_left(const BvhItem* __restrict__ items, const BvhChunk* __restrict__ chunks,
                                                        const BvhSah* __restrict__ sah, int* chunk_left) {
  __shared__ int n;
  const BvhChunk c = chunks[blockIdx.x];
  const BvhSah h = sah[c.seg];
  if (threadIdx.x == 0) n = 0;
  __syncthreads();
  const int i = c.begin + threadIdx.x;
  const bool left = i < c.end && bin_of(items[i], h.axis, h.cmin, h.extent) <= h.best;
  const unsigned m = __ballot_sync(0xffffffffu, left);
  if ((threadIdx.x & 31) == 0 && m) atomicAdd(&n, __popc(m));
  __syncthreads();
  if (threadIdx.x == 0) chunk_left[blockIdx.x] = n;
}

// items of bins <= best to first + (left items before them), the others to
// last - 1 - (right items before them): the reference's two-pointer fill
__global__ void __launch_bounds__(256) k_bvh_partition(const BvhItem* __restrict__ items, BvhItem* __restrict__ out,
                                                       const BvhChunk* __restrict__ chunks, const BvhSah* __restrict__ sah,
                                                       const int* __restrict__ chunk_left_base) {
  __shared__ int warp_left[8];
  const BvhChunk c = chunks[blockIdx.x];
  const BvhSah h = sah[c.seg];
  const int t = threadIdx.x, lane = t & 31, wid = t >> 5;
  const int i = c.begin + t;
  const bool valid = i < c.end;
  BvhItem it;
  bool left = false;
  if (valid) {
    it = items[i];
    left = bin_of(it, h.axis, h.cmin, h.extent) <= h.best;
  }
  const unsigned m = __ballot_sync(0xffffffffu, left);
  if (lane == 0) warp_left[wid] = __popc(m);
  __syncthreads();
  int before = __popc(m & ((1u << lane) - 1u));
  for (int w = 0; w < wid; ++w) before += warp_left[w];
  if (valid) {
    const int lrank = chunk_left_base[blockIdx.x] + before;  // left items before i in the range
    const int dst = left ? h.first + lrank : h.last - 1 - ((i - h.first) - lrank);
    out[dst] = it;
  }
}

__global__ void __launch_bounds__(256) k_bvh_copy(BvhItem* __restrict__ items, const BvhItem* __restrict__ from,
                                                  const BvhChunk* __restrict__ chunks) {
  const BvhChunk c = chunks[blockIdx.x];
  const int i = c.begin + threadIdx.x;
  if (i < c.end) items[i] = from[i];
}

// One thread per small range: the reference's recursion (Util/BVH.fs:99-237) as a loop over an
// explicit stack, nodes in preorder.  The bounds folds, bins and costs are the host builder's.
struct Frame {
  int first, last, depth, parent;
};
constexpr int kFrames = 72;  // the depth cap of 64 bounds the stack

__global__ void __launch_bounds__(128) k_bvh_small(BvhItem* __restrict__ items, BvhItem* __restrict__ scratch,
                                                   const BvhSmall* __restrict__ smalls, int n_small,
                                                   bn_bvh_node* __restrict__ nodes, int* __restrict__ node_counts,
                                                   int* overflow) {
  const int s = blockIdx.x * blockDim.x + threadIdx.x;
  if (s >= n_small) return;
  const BvhSmall sm = smalls[s];
  bn_bvh_node* out = nodes + sm.node_base;
  Frame stack[kFrames];
  int sp = 0, nn = 0;
  stack[sp++] = {sm.first, sm.last, sm.depth, -1};
  const float inf = CUDART_INF_F;
  while (sp > 0) {
    const Frame f = stack[--sp];
    const int self = nn++;
    if (f.parent >= 0) out[f.parent].right_or_offset = self;
    const int count = f.last - f.first;
    float lo[3] = {inf, inf, inf}, hi[3] = {-inf, -inf, -inf};
    for (int i = f.first; i < f.last; ++i) {
      const BvhItem it = items[i];
      lo[0] = min_native(lo[0], it.a.x); lo[1] = min_native(lo[1], it.a.y); lo[2] = min_native(lo[2], it.a.z);
      hi[0] = max_native(hi[0], it.b.x); hi[1] = max_native(hi[1], it.b.y); hi[2] = max_native(hi[2], it.b.z);
    }
    bn_bvh_node n{};
    for (int k = 0; k < 3; ++k) {
      n.bounds_min[k] = lo[k];
      n.bounds_max[k] = hi[k];
    }
    if (count <= 4 || f.depth >= 64) {
      n.right_or_offset = f.first;
      n.is_leaf = 1;
      n.count = static_cast<int8_t>(count);
      if (count > 127) atomicOr(overflow, 1);
      out[self] = n;
      continue;
    }
    float clo[3] = {inf, inf, inf}, chi[3] = {-inf, -inf, -inf};
    for (int i = f.first; i < f.last; ++i) {
      const BvhItem it = items[i];
      const float c0 = cen(it.a.x, it.b.x), c1 = cen(it.a.y, it.b.y), c2 = cen(it.a.z, it.b.z);
      clo[0] = min_native(clo[0], c0); clo[1] = min_native(clo[1], c1); clo[2] = min_native(clo[2], c2);
      chi[0] = max_native(chi[0], c0); chi[1] = max_native(chi[1], c1); chi[2] = max_native(chi[2], c2);
    }
    const float dx = __fsub_rn(chi[0], clo[0]), dy = __fsub_rn(chi[1], clo[1]), dz = __fsub_rn(chi[2], clo[2]);
    const int axis = (dx >= dy && dx >= dz) ? 0 : (dy >= dz ? 1 : 2);
    const float extent = axis == 0 ? dx : (axis == 1 ? dy : dz);
    n.is_leaf = 0;
    n.split_axis = static_cast<int8_t>(axis);
    n.right_or_offset = -1;  // set when the right child is emitted
    out[self] = n;
    if (sp + 2 > kFrames) {  // cannot happen below the depth cap; refuse rather than overrun
      atomicOr(overflow, 2);
      return;
    }
    if (extent == 0.f) {
      const int mid = f.first + count / 2;
      stack[sp++] = {mid, f.last, f.depth + 1, self};
      stack[sp++] = {f.first, mid, f.depth + 1, -1};
      continue;
    }
    const float cmin = clo[axis];
    float blo[kBvhBins][3], bhi[kBvhBins][3];
    int bcnt[kBvhBins];
    for (int k = 0; k < kBvhBins; ++k) {
      blo[k][0] = blo[k][1] = blo[k][2] = inf;
      bhi[k][0] = bhi[k][1] = bhi[k][2] = -inf;
      bcnt[k] = 0;
    }
    for (int i = f.first; i < f.last; ++i) {
      const BvhItem it = items[i];
      scratch[i] = it;  // the subrange copy the partition reads from (Util/BVH.fs:130)
      const int k = bin_of(it, axis, cmin, extent);
      blo[k][0] = min_native(blo[k][0], it.a.x); blo[k][1] = min_native(blo[k][1], it.a.y);
      blo[k][2] = min_native(blo[k][2], it.a.z);
      bhi[k][0] = max_native(bhi[k][0], it.b.x); bhi[k][1] = max_native(bhi[k][1], it.b.y);
      bhi[k][2] = max_native(bhi[k][2], it.b.z);
      bcnt[k] += 1;
    }
    auto area = [](float x0, float y0, float z0, float x1, float y1, float z1) {
      const float ex = __fsub_rn(x1, x0), ey = __fsub_rn(y1, y0), ez = __fsub_rn(z1, z0);
      return __fmul_rn(2.f, __fadd_rn(__fadd_rn(__fmul_rn(ex, ey), __fmul_rn(ey, ez)), __fmul_rn(ez, ex)));
    };
    float costs[kBvhBins - 1];
    for (int i = 0; i < kBvhBins - 1; ++i) costs[i] = 0.f;
    float l0 = inf, l1 = inf, l2 = inf, l3 = -inf, l4 = -inf, l5 = -inf;
    float r0 = inf, r1 = inf, r2 = inf, r3 = -inf, r4 = -inf, r5 = -inf;
    int lc = 0, rc = 0;
    const int nc = kBvhBins - 1;
    for (int i = 0; i < nc; ++i) {
      l0 = min_native(l0, blo[i][0]); l1 = min_native(l1, blo[i][1]); l2 = min_native(l2, blo[i][2]);
      l3 = max_native(l3, bhi[i][0]); l4 = max_native(l4, bhi[i][1]); l5 = max_native(l5, bhi[i][2]);
      lc += bcnt[i];
      costs[i] = __fadd_rn(costs[i], __fmul_rn(static_cast<float>(lc), area(l0, l1, l2, l3, l4, l5)));
      const int j = nc - i;
      r0 = min_native(r0, blo[j][0]); r1 = min_native(r1, blo[j][1]); r2 = min_native(r2, blo[j][2]);
      r3 = max_native(r3, bhi[j][0]); r4 = max_native(r4, bhi[j][1]); r5 = max_native(r5, bhi[j][2]);
      rc += bcnt[j];
      costs[nc - 1 - i] = __fadd_rn(costs[nc - 1 - i], __fmul_rn(static_cast<float>(rc), area(r0, r1, r2, r3, r4, r5)));
    }
    float min_cost = inf;
    int best = 0;
    const float base = __fmul_rn(static_cast<float>(count), area(clo[0], clo[1], clo[2], chi[0], chi[1], chi[2]));
    for (int i = 0; i < nc; ++i) {
      const float c = __fadd_rn(costs[i], base);
      if (c < min_cost) {
        min_cost = c;
        best = i;
      }
    }
    int left = f.first, right = f.last - 1;
    for (int i = f.first; i < f.last; ++i) {
      const BvhItem it = scratch[i];
      if (bin_of(it, axis, cmin, extent) > best) items[right--] = it;
      else items[left++] = it;
    }
    stack[sp++] = {left, f.last, f.depth + 1, self};
    stack[sp++] = {f.first, left, f.depth + 1, -1};
  }
  node_counts[s] = nn;
}

int blocks_for(long long n, int bs) { return static_cast<int>((n + bs - 1) / bs); }

}  // namespace

cudaError_t bvh_launch_init_acc(BvhSegAcc* acc, int n, cudaStream_t st) {
  if (n > 0) k_bvh_init_acc<<<blocks_for(n, 256), 256, 0, st>>>(acc, n);
  return cudaGetLastError();
}
cudaError_t bvh_launch_init_bins(BvhBin* bins, int n, cudaStream_t st) {
  if (n > 0) k_bvh_init_bins<<<blocks_for(n, 256), 256, 0, st>>>(bins, n);
  return cudaGetLastError();
}
cudaError_t bvh_launch_reduce(const BvhItem* items, const BvhChunk* chunks, int n_chunks, BvhSegAcc* acc,
                              cudaStream_t st) {
  if (n_chunks > 0) k_bvh_reduce<<<n_chunks, 256, 0, st>>>(items, chunks, acc);
  return cudaGetLastError();
}
cudaError_t bvh_launch_finalize(const BvhItem* items, const BvhSegAcc* acc, int n_segs, float* bounds12,
                                cudaStream_t st) {
  if (n_segs > 0) k_bvh_finalize<<<blocks_for(n_segs, 256), 256, 0, st>>>(items, acc, n_segs, bounds12);
  return cudaGetLastError();
}
cudaError_t bvh_launch_bins(const BvhItem* items, const BvhChunk* chunks, int n_chunks, const BvhSah* sah,
                            BvhBin* bins, cudaStream_t st) {
  if (n_chunks > 0) k_bvh_bins<<<n_chunks, 256, 0, st>>>(items, chunks, sah, bins);
  return cudaGetLastError();
}
cudaError_t bvh_launch_count_left(const BvhItem* items, const BvhChunk* chunks, int n_chunks, const BvhSah* sah,
                                  int* chunk_left, cudaStream_t st) {
  if (n_chunks > 0) k_bvh_count_left<<<n_chunks, 256, 0, st>>>(items, chunks, sah, chunk_left);
  return cudaGetLastError();
}
cudaError_t bvh_launch_partition(const BvhItem* items, BvhItem* out, const BvhChunk* chunks, int n_chunks,
                                 const BvhSah* sah, const int* chunk_left_base, cudaStream_t st) {
  if (n_chunks > 0) k_bvh_partition<<<n_chunks, 256, 0, st>>>(items, out, chunks, sah, chunk_left_base);
  return cudaGetLastError();
}
cudaError_t bvh_launch_copy(BvhItem* items, const BvhItem* from, const BvhChunk* chunks, int n_chunks,
                            cudaStream_t st) {
  if (n_chunks > 0) k_bvh_copy<<<n_chunks, 256, 0, st>>>(items, from, chunks);
  return cudaGetLastError();
}
cudaError_t bvh_launch_small(BvhItem* items, BvhItem* scratch, const BvhSmall* smalls, int n_small,
                             bn_bvh_node* nodes, int* node_counts, int* overflow, cudaStream_t st) {
  if (n_small > 0) k_bvh_small<<<blocks_for(n_small, 128), 128, 0, st>>>(items, scratch, smalls, n_small, nodes,
                                                                          node_counts, overflow);
  return cudaGetLastError();
}

}  // namespace bn
