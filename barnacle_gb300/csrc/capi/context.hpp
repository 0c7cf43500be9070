// bn_context: the device-resident state behind the C-ABI.
#pragma once
#include <cuda_runtime.h>

#include <string>
#include <vector>

#include "../../../include/barnacle_gpu.h"
#include "../device/dev_types.cuh"
#include "../device/launch.hpp"
#include "../device/pssmlt.hpp"

// growable device buffer
struct DevBuf {
  void* ptr = nullptr;
  size_t bytes = 0;
  cudaError_t reserve(size_t n) {
    if (n <= bytes) return cudaSuccess;
    if (ptr) cudaFree(ptr);
    ptr = nullptr;
    bytes = 0;
    cudaError_t e = cudaMalloc(&ptr, n);
    if (e == cudaSuccess) bytes = n;
    return e;
  }
  void release() {
    if (ptr) cudaFree(ptr);
    ptr = nullptr;
    bytes = 0;
  }
  template <class T>
  T* as() const { return static_cast<T*>(ptr); }
};

struct bn_context {
  int device = 0;
  cudaStream_t stream = nullptr;
  cudaEvent_t ev0 = nullptr, ev1 = nullptr, ev2 = nullptr;
  std::string err;

  // scene
  bool has_scene = false;
  bn::DevScene scene{};
  DevBuf nodes, nodes4, tris, inst, mats, lights, light_inst, tri_pdf, tri_lights, error_word, counters;
  std::vector<int32_t> inst_order;     // TLAS order -> descriptor index
  std::vector<bn::DevMaterial> host_mats;
  std::vector<int32_t> host_inst_light;  // per TLAS instance: light index
  int n_lights = 0;
  float scene_lo[3] = {0.f, 0.f, 0.f}, scene_hi[3] = {0.f, 0.f, 0.f};  // TLAS root box
  bool scene_simple = false;  // Lambertian materials, triangle meshes, the uniform light sampler
  // failure-detection limits (bn_set_limits; 0 = the defaults)
  int limit_stack = 0;        // traversal stack entries a walk may use
  int limit_iters = 0;        // wavefront bounce-loop iterations before the watchdog stops it

  // queries
  DevBuf q_in, q_out;

  // render
  DevBuf views, item_offsets, partial, film, wf_state, rgba;
  long long film_floats = 0;
  bn_stats stats{};

  // pssmlt / adjoint scratch
  DevBuf mlt_state, mlt_boot, mlt_chain, adj_params, adj_image, adj_target, adj_grad, adj_aux;

  // wavefront path state, captured graph and tuned launch shape (owned by wavefront.cu)
  void* wf = nullptr;
  void (*wf_release)(void*) = nullptr;
  long long scene_generation = 0;  // bumped by every bn_scene_upload

  int fail(int code, const std::string& msg) {
    err = msg;
    return code;
  }
  int cuda_fail(cudaError_t e, const char* where) {
    err = std::string(where) + ": " + cudaGetErrorString(e);
    return e == cudaErrorMemoryAllocation ? BN_ERR_OUT_OF_MEMORY : BN_ERR_CUDA;
  }
};

namespace bnc {
// host-side view constants (Extensions/Camera/Pinhole.fs:16-22), shared by all render modes
bn::DevView make_dev_view(const bn_view& v, long long pixel_offset, long long path_offset);
int check_device_error(bn_context* ctx);
// The plain megakernel's sample chunks: each work item runs spc consecutive samples of one pixel,
// chunks = ceil(spp / spc) items per pixel.  max_items > 0 caps pixels * chunks (fixed scratch).
struct MegaChunks {
  int chunks = 1, spc = 1;
};
MegaChunks mega_chunks(long long pixels, int spp, long long max_items);
// Launch parameters of the megakernel shared by bn_render and bn_render_noalloc (views, item
// offsets, partial sums, film and counting are filled in by the caller).
bn::MegaParams mega_params(const bn_context* ctx, const bn_render_desc* d, const std::vector<bn::DevView>& views,
                           const MegaChunks& ck, long long items, long long pixels);
int render_wavefront(bn_context* ctx, const bn_render_desc* d, const std::vector<bn::DevView>& views);
// BVHNode.Build on the GPU (bvh_gpu.cu): the host builder's nodes and permutation
int gpu_bvh_build(bn_context* ctx, const float* bounds, int32_t n, std::vector<bn_bvh_node>* nodes,
                  std::vector<int32_t>* perm, int small);
int render_pssmlt(bn_context* ctx, const bn_render_desc* d, const std::vector<bn::DevView>& views);
// the PSSMLT chains in the wavefront (wavefront.cu), after the bootstrap
int render_pssmlt_wavefront(bn_context* ctx, const bn_render_desc* d, const bn::MltParams& mp, int* launches);
}  // namespace bnc
