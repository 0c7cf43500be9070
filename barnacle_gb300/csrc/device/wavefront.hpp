// Wavefront path state (HBM, structure of arrays) and launch interface.
#pragma once
#include <cuda_runtime.h>

#include "../../../include/barnacle_gpu.h"
#include "dev_types.cuh"

namespace bn {

constexpr int kNumBins = 6;  // 4 material types, miss, no material
// ray-queue sort keys: direction octant (3 bits) over the Morton code of the origin's cell in a
// 2^b x 8 x 2^b grid (x, y, z) over the scene bounds, b from 5 to 8 with the pool (sort_key_bits):
// at most 22 bits
constexpr int kSortBits = 22, kSortBins = 1 << kSortBits;
// b for a pool of path slots: the histogram's fixed scan cost (two passes over its bins per sort)
// grows with the bins, the sort's coherence with the rays per bin.  Measured on the 1,024-instance
// workload: 16-bit keys (b = 5) best at 1 M slots, 20-bit (b = 7) at 16 M, 22-bit (b = 8) at 32 M
// and 64 M
inline int sort_key_bits(long long pool) {
  int lg = 0;
  while ((2LL << lg) <= pool) ++lg;  // floor(log2(pool))
  const int b = (lg - 9) / 2;
  return b < 5 ? 5 : (b > 8 ? 8 : b);
}
enum : int {
  kCntActive = 0,   // ray-queue length
  kCntShadow = 1,   // shadow-queue length
  kCntCont = 2,     // paths continuing after shade
  kCntDone = 3,     // paths that ended this iteration (retired by the next regen)
  kCntIter = 4,     // iterations run
  kCntAgain = 5,    // last control decision (host-driven loop)
  kCntFetchRay = 6, // dynamic-fetch cursors of the extend and shadow kernels
  kCntFetchShadow = 7,
  kCntBin0 = 8,     // 8..13: per-bin hit counts
  // PSSMLT chains: the queues filled in one iteration and traced in the next (k_wf_control moves
  // them into kCntActive / kCntShadow)
  kCntShadowNext = 14,
  kCntActiveNext = 15,
  kCntSize = 16
};

// PSSMLT chains in the wavefront (WfParams::mlt): one path slot per Markov chain; the chain loop
// of PSSMLTIntegrator.RenderSingleChain (PSSMLT.fs:275-377) advances one bounce per iteration.
struct MltWf {
  int n_chains, n_bootstrap, n_dims, mutations;  // mutations per chain, ceil(spp W H / chains)
  int kelemen;                  // 1 Kelemen(eps_min, eps_max), 0 Gaussian(sigma)
  float p_large, sigma, eps_min, eps_max;
  float b, inv_eff_spp;         // bootstrap mean luminance, 1 / effective spp
  const float* alias_prob;      // proportional start table, or null: uniform as the reference
  const int* alias_idx;
  int4* smp;                    // per chain: the MLTSampler's scalar state (MltSampler::pack)
  float4* chain;                // 3 per chain: (L, y), (radiance, pix), (chain sampler, iteration,
                                //   pixel of the mutation in flight, bootstrap id)
  float4* X;                    // n_dims primary samples per chain, chain-major
  float* film;                  // W * H * 3 FP32, splatted
  unsigned long long* accepted;
};

struct WfParams {
  DevScene scene;
  const DevView* views;
  int n_views;
  int spp, max_depth, rr_depth, frame_id;
  int integrator;               // BN_INTEGRATOR_PATH, _NORMAL or _DIRECT
  int pool;                     // path slots
  int max_iters;                // watchdog
  int refill_extend;            // extend lanes refill when at most this many of a warp still walk
  int refill_shadow;            // the same for the shadow kernel
  long long total_paths;
  long long n_pixels;
  // per slot
  // per slot, 32-byte records so that a slot's part of each is one DRAM sector
  float4* ray;                  // 2 per slot: (o, -), (d, pdf of the last BSDF sample)
  float4* bl;                   // 2 per slot: (beta, -), (L, -)
  float4* hit;                  // 2 per slot: (t, u, v, instance | -1 as int bits),
                                //             (triangle or sphere root as int bits, -, -, -)
  int4* meta;                   // (film pixel, depth, sampler state, status)
  // queues
  int* q_active;                // pool entries
  int* q_bins;                  // kNumBins x pool entries
  // spatial sort of both ray queues (counting sort by key, when sort != 0)
  int sort, sort_shadow;
  float4 key_lo, key_scale;     // origin cell = (o - key_lo) * key_scale, in [0, 2^b) x [0, 8) x [0, 2^b)
  int key_bits;                 // b (sort_key_bits): the keys span 2^(2b + 6) bins
  int* slot_key;                // per slot: key of the ray the slot holds (written by shade)
  int* q_key;                   // per ray-queue entry: its key
  int* q_ray;                   // the ray queue in key order (read by extend)
  int* sh_key;                  // per shadow record: its key
  int* q_shadow;                // shadow-record indices in key order (read by shadow)
  unsigned* hist;               // kSortBins counts; zero between uses (the scan clears it)
  unsigned* off;                // kSortBins bucket offsets, then kSortBins / 1024 tile sums
  float4* shadow;               // 4 float4 per record: (o, tmax), (d, owner), a, b
  int* counters;                // kCntSize ints
  void* trace_counters;         // DevCounters (rays, nodes, triangles, instances) of counting walks
  unsigned long long* work_next;
  double* film_acc;             // 3 doubles per pixel
  float* film_out;              // 3 floats per pixel
  cudaGraphConditionalHandle cond;
  int mlt;                      // 1: the slots hold PSSMLT chains (mlt_p), 0: camera paths
  MltWf mlt_p;
};

struct WfLaunch {
  int grid_regen, grid_extend, grid_shade, grid_shadow, grid_scatter;
  int sort_tiles;               // 1,024-bin tiles of the keys' histogram (2^(2b + 6) / 1,024)
  bool watertight;
  bool wide;                    // the scene's wide records (kWalkWide kernels)
  bool sort, sort_shadow;       // ray / shadow queue sorted by ray key before extend / shadow
  bool count;                   // binary walks that count their visits (BN_RENDER_COUNT)
  bool mlt;                     // PSSMLT chains: mlt regen and shade kernels instead of regen / shade
  bool mlt_kelemen;             // their mutation strategy (Kelemen, else Gaussian)
};

// mlt_chains: PSSMLT chains (one slot each); sizes the traversal grids so both fit side by side
WfLaunch wf_launch_shape(bool watertight, bool wide, bool sort, bool sort_shadow, bool count, int blocks_per_sm_cap,
                         bool mlt = false, bool mlt_kelemen = false, long long mlt_chains = 0, int key_bits = 5);
// the chain kernels of the PSSMLT wavefront (k_mlt_wavefront.cu)
cudaError_t mlt_launch_regen(WfParams* dparams, int grid, bool kelemen, cudaStream_t st);
cudaError_t mlt_launch_shade(WfParams* dparams, int grid, bool watertight, bool kelemen, cudaStream_t st);
int mlt_grid_regen();
int mlt_grid_shade(bool watertight);
// a second stream and two events: the PSSMLT iteration traces its shadow and extension rays on
// two streams at once (fork / join)
struct WfFork {
  cudaStream_t side;
  cudaEvent_t fork, join;
};
cudaError_t wf_launch_iteration(WfParams* dparams, const WfLaunch& l, bool use_graph, cudaStream_t st,
                                const WfFork* fk = nullptr);
cudaError_t wf_launch_resolve(WfParams* dparams, cudaStream_t st);

}  // namespace bn
