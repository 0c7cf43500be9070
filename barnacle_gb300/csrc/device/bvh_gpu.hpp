// Device side of the GPU BVH builder (k_bvh.cu): the reference-compatible binned SAH build of
// BVHNode.Build (Util/BVH.fs:99-247), level by level for large node ranges and one thread per
// small range.  The host side (csrc/capi/bvh_gpu.cu) makes the per-node decisions of the large
// ranges from the reductions these kernels return.
#pragma once
#include <cuda_runtime.h>

#include "../../../include/barnacle_gpu.h"

namespace bn {

// one box to build over: (lo.xyz, item index as int bits), (hi.xyz, 0)
struct BvhItem {
  float4 a, b;
};

// up to 256 consecutive items of one node range
struct BvhChunk {
  int seg, begin, end, pad;
};

// per-range reduction: box bounds and centroid bounds as order-preserving unsigned encodings,
// and per bound component the last item index whose coordinate is +-0 (the sign a sequential
// MinNative/MaxNative fold leaves on a zero bound)
struct BvhSegAcc {
  unsigned lo[3], hi[3], clo[3], chi[3];
  int zlo[3], zhi[3];
};

// a range split by SAH this level: the split axis, the centroid range and (after the bins are
// read) the chosen bin
struct BvhSah {
  int first, last, axis, best;
  float cmin, extent;
  int pad0, pad1;
};

constexpr int kBvhBins = 12;
struct BvhBin {
  unsigned lo[3], hi[3];
  int cnt, pad;
};

// a small range finished by one thread: the sequential build writes its nodes (preorder, right
// child indices relative to the range's first node) from node_base on
struct BvhSmall {
  int first, last, depth, node_base;
};

cudaError_t bvh_launch_reduce(const BvhItem* items, const BvhChunk* chunks, int n_chunks, BvhSegAcc* acc,
                              cudaStream_t st);
cudaError_t bvh_launch_finalize(const BvhItem* items, const BvhSegAcc* acc, int n_segs, float* bounds12,
                                cudaStream_t st);
cudaError_t bvh_launch_bins(const BvhItem* items, const BvhChunk* chunks, int n_chunks, const BvhSah* sah,
                            BvhBin* bins, cudaStream_t st);
cudaError_t bvh_launch_count_left(const BvhItem* items, const BvhChunk* chunks, int n_chunks, const BvhSah* sah,
                                  int* chunk_left, cudaStream_t st);
cudaError_t bvh_launch_partition(const BvhItem* items, BvhItem* out, const BvhChunk* chunks, int n_chunks,
                                 const BvhSah* sah, const int* chunk_left_base, cudaStream_t st);
cudaError_t bvh_launch_copy(BvhItem* items, const BvhItem* from, const BvhChunk* chunks, int n_chunks,
                            cudaStream_t st);
cudaError_t bvh_launch_small(BvhItem* items, BvhItem* scratch, const BvhSmall* smalls, int n_small,
                             bn_bvh_node* nodes, int* node_counts, int* overflow, cudaStream_t st);
cudaError_t bvh_launch_init_acc(BvhSegAcc* acc, int n, cudaStream_t st);
cudaError_t bvh_launch_init_bins(BvhBin* bins, int n, cudaStream_t st);

}  // namespace bn
