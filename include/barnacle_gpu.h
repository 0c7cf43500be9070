/*
 * barnacle_gpu.h — C-ABI of the GB300 path-tracing core (libbarnacle_gb300.so).
 *
 * This library replaces the render call of the Barnacle F# renderer:
 *   IntegratorBase.Render : CameraBase * Film * PrimitiveAggregate * LightSamplerBase -> unit
 *     (Base/Integrator.fs:11, called from Extensions/Scene/Render.fs:16)
 * and the queries the render call is built from (Aggregate.Intersect, Material.Eval/Sample,
 * the hash sampler).  The host flattens the scene (instances after Scene.Traverse(0), their
 * matrices, meshes, materials, lights, camera) into the plain structs below and hands them to
 * bn_scene_upload; the library builds the reference-compatible SAH BLAS/TLAS on the host and
 * keeps every device buffer resident until the next upload.
 *
 * Conventions
 *   - every entry point returns an int status: BN_OK (0) or a BN_ERR_* code;
 *     the message of the last failure on a context is available from bn_last_error.
 *   - all pointers are HOST pointers owned by the caller unless a name says _device.
 *   - matrices are System.Numerics.Matrix4x4 in memory order (M11 M12 M13 M14 M21 ... M44),
 *     row-vector convention: p' = p * M, translation in M41..M43.
 *   - one CUDA stream per context; a context is not thread safe, separate contexts are.
 */
#ifndef BARNACLE_GPU_H
#define BARNACLE_GPU_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define BN_ABI_VERSION 1

/* ---- status codes ---------------------------------------------------------------------- */
#define BN_OK 0
#define BN_ERR_INVALID_ARG 1   /* null pointer, bad size, out-of-range index in a descriptor */
#define BN_ERR_CUDA 2          /* a CUDA runtime call failed (message has the CUDA error)     */
#define BN_ERR_NO_SCENE 3      /* a query or render before bn_scene_upload                   */
#define BN_ERR_DEVICE 4        /* a kernel set the device error word (see BN_DEVERR_*)       */
#define BN_ERR_OUT_OF_MEMORY 5 /* device allocation failed                                   */
#define BN_ERR_UNSUPPORTED 6   /* option not supported by this build                         */
#define BN_ERR_IO 7            /* scene/OBJ file could not be read or parsed                 */

/* device error word bits, reported through BN_ERR_DEVICE and bn_get_stats */
#define BN_DEVERR_STACK_OVERFLOW 0x1u /* BVH traversal stack exceeded its fixed depth      */
#define BN_DEVERR_QUEUE_OVERFLOW 0x2u /* a wavefront queue index went past its capacity   */
#define BN_DEVERR_WATCHDOG 0x4u       /* a bounded device loop hit its iteration limit    */
#define BN_DEVERR_BAD_INDEX 0x8u      /* a node/triangle/material index was out of range  */

/* ---- scene description (what the F# host flattens; Base/Scene.fs:38-61) ---------------- */
enum bn_primitive_type { BN_PRIM_MESH = 0, BN_PRIM_SPHERE = 1 };
/* MaterialBase implementations: Extensions/Material/{Lambertian,Mirror,Dielectric,PBR}.fs */
enum bn_material_type { BN_MAT_LAMBERTIAN = 0, BN_MAT_MIRROR = 1, BN_MAT_DIELECTRIC = 2, BN_MAT_PBR = 3 };
/* CameraBase implementations: Extensions/Camera/{Pinhole,ThinLens}.fs */
enum bn_camera_type { BN_CAM_PINHOLE = 0, BN_CAM_THIN_LENS = 1 };
/* LightSamplerBase implementations */
enum bn_light_sampler_type {
  BN_LIGHTS_UNIFORM = 0,        /* Extensions/LightSampler/Uniform.fs: uniform over emissive instances */
  BN_LIGHTS_ALIAS_TRIANGLES = 1 /* new plugin: Vose alias table over all emissive triangles, by power  */
};
/* How the device walks the scene's BVHs.  Both walks return identical hits (same visit order and
 * box decisions as Aggregate/BVH.fs); they differ in speed only.  AUTO takes the 4-wide records
 * for scenes of at least 1,024 BVH nodes, where halving the dependent node loads pays for the
 * wider tests.  Visit counting (BN_TRACE_COUNT, BN_RENDER_COUNT) always walks the binary tree. */
enum bn_bvh_width { BN_BVH_AUTO = 0, BN_BVH_BINARY = 2, BN_BVH_WIDE = 4 };
/* Where bn_scene_upload builds the BLASes and the TLAS; both builders give the same trees
 * (BVHNode.Build, Util/BVH.fs:239-247).  AUTO builds on the GPU from 16,384 boxes on. */
enum bn_bvh_builder { BN_BUILDER_AUTO = 0, BN_BUILDER_HOST = 1, BN_BUILDER_DEVICE = 2 };

/* MeshPrimitive(vertices, indices) (Extensions/Primitive/Mesh.fs:120) */
typedef struct bn_mesh_desc {
  const float* vertices;          /* 3 * n_vertices floats                               */
  const int32_t* indices;         /* 3 * n_triangles vertex indices                      */
  const int32_t* tri_material;    /* optional per-triangle material slot, NULL = none    */
  int32_t n_vertices;
  int32_t n_triangles;
} bn_mesh_desc;

/* ElementalPrimitive: a mesh (index into meshes) or SpherePrimitive(radius) (Sphere.fs:13) */
typedef struct bn_primitive_desc {
  int32_t type;   /* bn_primitive_type */
  int32_t mesh;   /* mesh index when type == BN_PRIM_MESH */
  float radius;   /* sphere radius when type == BN_PRIM_SPHERE */
} bn_primitive_desc;

/* PrimitiveInstance after Node.Traverse (Base/Primitive.fs:99-138, Base/Scene.fs:43-51) */
typedef struct bn_instance_desc {
  int32_t primitive;            /* index into primitives                          */
  int32_t material;             /* index into materials, -1 = no material         */
  int32_t light;                /* index into lights, -1 = not emissive           */
  int32_t pad_;
  float object_to_world[16];    /* PrimitiveInstance.ObjectToWorld                */
  float world_to_object[16];    /* PrimitiveInstance.WorldToObject (its inverse)  */
} bn_instance_desc;

typedef struct bn_material_desc {
  int32_t type;        /* bn_material_type                       */
  float base_color[3]; /* "albedo" (Loader.fs:118-122, default 1) */
  float ior;           /* dielectric IOR (default 1.5)           */
  float roughness;     /* PBR roughness (default 1)              */
  float metallic;      /* PBR metallic (default 0)               */
  float pad_;
} bn_material_desc;

/* DiffuseLight(emission, twoSided) (Base/Light.fs:26-53) */
typedef struct bn_light_desc {
  float emission[3];
  int32_t two_sided;
} bn_light_desc;

/* camera + its world transform (Base/Camera.fs:6-20) */
typedef struct bn_camera_desc {
  int32_t type;            /* bn_camera_type                         */
  float fov_y_degrees;     /* vertical field of view (default 45)    */
  float aspect_ratio;      /* from the scene file, not the film      */
  float aperture;          /* thin lens only                         */
  float focus_distance;    /* thin lens only                         */
  float push_forward;      /* origin pushed along the ray            */
  float camera_to_world[16];
} bn_camera_desc;

typedef struct bn_scene_desc {
  const bn_primitive_desc* primitives; int32_t n_primitives;
  const bn_mesh_desc* meshes;          int32_t n_meshes;
  const bn_instance_desc* instances;   int32_t n_instances;
  const bn_material_desc* materials;   int32_t n_materials;
  const bn_light_desc* lights;         int32_t n_lights;
  int32_t light_sampler;               /* bn_light_sampler_type */
  int32_t bvh_width;                   /* bn_bvh_width (0 = auto) */
  int32_t bvh_builder;                 /* bn_bvh_builder (0 = auto) */
} bn_scene_desc;

/* ---- ray queries (Extensions/Aggregate/BVH.fs:11-58) ----------------------------------- */
typedef struct bn_ray {
  float origin[3];
  float direction[3];
  float t_max;   /* closest hit: initial t (infinity in Li); any hit: the shadow ray's t */
} bn_ray;

typedef struct bn_hit {
  float t;
  float u, v;          /* barycentrics (b1, b2) of the hit triangle; sphere: the uv map  */
  int32_t instance;    /* index into the TLAS-permuted instance order, -1 = miss         */
  int32_t primitive;   /* triangle index within the BLAS-permuted mesh order (the tag)   */
  float normal[3];     /* world-space shading normal (Interaction.Normal)                */
  float position[3];   /* world-space hit point (LocalGeometry.Transform of p)           */
} bn_hit;

#define BN_TRACE_CLOSEST 0x0u       /* PrimitiveAggregate.Intersect(ray, &interaction, &t) */
#define BN_TRACE_ANY 0x1u           /* PrimitiveAggregate.Intersect(ray, t)                */
#define BN_TRACE_WATERTIGHT 0x2u    /* Woop-Benthin-Wald watertight triangle test instead  */
                                    /* of the reference's Moller-Trumbore (Mesh.fs:24-82)   */
#define BN_TRACE_COUNT 0x4u         /* also accumulate node/triangle/instance visit counts  */

/* ---- materials (Base/Material.fs:5-20) ------------------------------------------------- */
typedef struct bn_bsdf_query {
  int32_t material;  /* index into the scene's materials */
  float wo[3];       /* local-frame directions (z = normal) */
  float wi[3];       /* eval: the incident direction       */
  float u_lobe;      /* sample: lobe selector               */
  float u_bsdf[2];   /* sample: 2-D direction sample        */
} bn_bsdf_query;

typedef struct bn_bsdf_result {
  float bsdf[3];     /* f * |cos theta_i| ("bsdf" in BSDFEval)   */
  float pdf;
  float wi[3];       /* sampled direction (sample only)          */
} bn_bsdf_result;

/* ---- render (Base/Integrator.fs:22-55, PathTracing.fs, PSSMLT.fs) ---------------------- */
enum bn_integrator_type {
  BN_INTEGRATOR_PATH = 0,   /* PathTracingIntegrator (Extensions/Integrator/PathTracing.fs)        */
  BN_INTEGRATOR_PSSMLT = 1, /* PSSMLTIntegrator (Extensions/Integrator/PSSMLT.fs)                  */
  BN_INTEGRATOR_NORMAL = 2, /* NormalIntegrator (Extensions/Integrator/Normal.fs): 0.5 (n + 1)     */
  BN_INTEGRATOR_DIRECT = 3  /* DirectIntegrator (Extensions/Integrator/Direct.fs): one light sample */
                            /* and one BSDF sample that scores a light it hits                     */
};
enum bn_render_mode {
  BN_MODE_MEGAKERNEL = 0, /* one thread per pixel-sample path (PSSMLT: per chain, in   */
                          /* lockstep), the plain form                               */
  BN_MODE_WAVEFRONT = 1   /* persistent queues compacted every bounce, many views per */
                          /* launch (PSSMLT: one path slot per chain, same decisions) */
};
enum bn_mutation_type { BN_MUTATION_GAUSSIAN = 0, BN_MUTATION_KELEMEN = 1 };

#define BN_RENDER_WATERTIGHT 0x1u   /* watertight triangle test on the render path            */
#define BN_RENDER_FIXED_ALIAS 0x2u  /* PSSMLT: start chains proportional to bootstrap weight  */
                                    /* (the reference's AliasTable samples uniformly)          */
#define BN_RENDER_NO_GRAPH 0x4u     /* wavefront: launch the bounce loop without a CUDA graph  */
                                    /* (PSSMLT chains always run host-driven iterations)       */
#define BN_RENDER_COUNT 0x8u        /* count rays / BVH nodes / triangles / instances visited  */
                                    /* into bn_stats (a slower instrumented kernel variant)     */
#define BN_RENDER_CULL_SHADOW 0x10u /* megakernel: evaluate a light sample first and trace its   */
                                    /* shadow ray only if it can change the radiance (the same  */
                                    /* image; the wavefront always does this, the plain form    */
                                    /* keeps the reference's trace-then-evaluate order)          */

typedef struct bn_view {
  bn_camera_desc camera;
  int32_t width, height;
} bn_view;

typedef struct bn_render_desc {
  int32_t integrator;        /* bn_integrator_type                                   */
  int32_t mode;              /* bn_render_mode                                        */
  int32_t spp;               /* samples per pixel, or PSSMLT mutations per pixel     */
  int32_t max_depth;         /* default 8                                            */
  int32_t rr_depth;          /* default 5                                            */
  int32_t frame_id;          /* ProgressiveIntegrator.FrameId                        */
  uint32_t flags;            /* BN_RENDER_*                                          */
  /* PSSMLT (Extensions/Integrator/PSSMLT.fs:153-170) */
  int32_t n_bootstrap;
  int32_t n_chains;
  int32_t mutation;          /* bn_mutation_type                                     */
  float large_step_prob;
  float sigma;               /* Gaussian mutation sigma                              */
  float eps_min, eps_max;    /* Kelemen s1, s2                                       */
  /* wavefront launch shape (0 = autotuned or default) */
  int32_t block_size;        /* traversal blocks per SM cap                           */
  int32_t queue_capacity;    /* path slots, 224 B of device memory each; autotuned    */
                             /* from 1 M to 64 M slots, none beyond the render's paths */
  int32_t pad_;
} bn_render_desc;

typedef struct bn_stats {
  uint64_t paths;            /* camera paths (PT) or Markov-chain proposals (PSSMLT)      */
  uint64_t rays;             /* closest-hit + shadow rays traced                          */
  uint64_t nodes_visited;    /* BVH nodes tested (TLAS + BLAS), when counting is enabled  */
  uint64_t tris_tested;
  uint64_t instances_visited;
  uint64_t accepted;         /* PSSMLT accepted mutations                                 */
  uint64_t proposed;         /* PSSMLT proposed mutations                                 */
  double bootstrap_b;        /* PSSMLT normalisation b                                    */
  uint32_t device_error;     /* BN_DEVERR_* bits of the last launch                       */
  float last_kernel_ms;      /* device time of the last render/trace (CUDA events)        */
  float last_dominant_ms;    /* device time of the dominant kernel of the last render     */
  int32_t last_launches;     /* kernels launched by the last render                       */
} bn_stats;

/* ---- context ------------------------------------------------------------------------- */
typedef struct bn_context bn_context;

const char* bn_version(void);
int bn_create(int device, bn_context** out);
int bn_destroy(bn_context* ctx);
/* copies the last error message (NUL-terminated, truncated to len) */
int bn_last_error(const bn_context* ctx, char* buf, size_t len);

/* Scene upload: builds BLAS per mesh + TLAS (Util/BVH.fs:239-247, Aggregate/BVH.fs:9),
 * per-mesh alias tables (Mesh.fs:181-186), the light sampler tables (Uniform.fs,
 * LightSampler.fs:7) and uploads everything.  Replaces the preparation in
 * Extensions/Scene/Render.fs:12-14. */
int bn_scene_upload(bn_context* ctx, const bn_scene_desc* scene);
/* the TLAS permutation: out[k] = index in the descriptor of the k-th instance in TLAS order */
int bn_scene_instance_order(const bn_context* ctx, int32_t* out, int32_t n);

/* Ray queries on the uploaded scene; replaces PrimitiveAggregate.Intersect (both overloads). */
int bn_trace(bn_context* ctx, const bn_ray* rays, int64_t n, uint32_t flags, bn_hit* hits);

/* Batched MaterialBase.Eval / MaterialBase.Sample in the local frame (Base/Material.fs:18-19). */
int bn_bsdf_eval(bn_context* ctx, const bn_bsdf_query* q, int64_t n, bn_bsdf_result* out);
int bn_bsdf_sample(bn_context* ctx, const bn_bsdf_query* q, int64_t n, bn_bsdf_result* out);

/* The hash sampler (Base/Sampler.fs:7-16): for seed triple i, draws n_draws Next1D values.
 * seeds: 3 uint32 per stream (x, y, z); out: n_streams * n_draws floats. */
int bn_sampler_stream(bn_context* ctx, const uint32_t* seeds, int64_t n_streams, int32_t n_draws, float* out);

/* Render: IntegratorBase.Render for one or several views.  out_rgb receives, view after view,
 * width*height*3 floats in Film.Pixels order (row 0 = top row, Base/Film.fs:41-53).
 * out_rgb may be NULL: the image then stays on the device (bn_film_download fetches it). */
int bn_render(bn_context* ctx, const bn_render_desc* desc, const bn_view* views, int32_t n_views,
              float* out_rgb);
int bn_film_download(bn_context* ctx, float* out_rgb, int64_t n_floats);

/* Film output (Base/Film.fs:21-30 PostProcess, :55-66 Save).  bn_film_tonemap maps the film of the
 * last bn_render on the device — identity, ACES fit x(2.51x+0.03)/(x(2.43x+0.59)+0.14) or gamma
 * x^(1/2.2), clamped to [0, 1] — and packs it as ImageSharp's Rgba32(Vector3) does
 * (byte = clamp(255 v + 0.5, 0, 255) truncated; NaN -> 0; alpha 255).  rgba receives 4 bytes per
 * pixel in Film.Pixels order (rows top to bottom) for the first n_pixels of the film (the views
 * one after another; the film's total for all of them). */
enum bn_tone_mapping { BN_TONE_IDENTITY = 0, BN_TONE_ACES = 1, BN_TONE_GAMMA = 2 };
int bn_film_tonemap(bn_context* ctx, int32_t tone_mapping, uint8_t* rgba, int64_t n_pixels);
/* PNG encoding of an RGBA8 image (the encoder Film.Save hands to ImageSharp; stored deflate
 * blocks, so no compression library is needed). */
int bn_image_write_png(const char* path, const uint8_t* rgba, int32_t width, int32_t height);

/* Render without allocating device memory (no counterpart in the reference).
 * For callers that cannot allocate during a render: a host whose device memory all comes from
 * its own arena and whose frame loop must not call cudaMalloc/cudaFree (they synchronise the
 * device), or a caller with a fixed memory budget on a shared GPU.  It renders bn_render's
 * megakernel mode (integrator BN_INTEGRATOR_PATH, mode BN_MODE_MEGAKERNEL only; flags
 * BN_RENDER_WATERTIGHT and BN_RENDER_CULL_SHADOW; BN_RENDER_COUNT returns BN_ERR_UNSUPPORTED) into
 * film_device, a caller-owned buffer of width*height*3 floats per view in DEVICE memory of the
 * context's GPU (anything else returns BN_ERR_INVALID_ARG), views back to back in Film.Pixels
 * order.  The context's own film (bn_film_download, bn_film_tonemap) is not written.  The scene
 * must already be uploaded (bn_scene_upload allocates; do it at set-up time).  Scratch lives in
 * one static device array of the library: 64 view records and 1,048,576 partial sums (16 MiB),
 * held by every GPU that loads the library until exit.  Limits: at most 64 views and 1,048,576
 * pixels in total; larger renders return BN_ERR_INVALID_ARG.  Images are bit-identical to
 * bn_render's while pixels x bn_render's sample chunks per pixel fit the 1,048,576 partial sums;
 * beyond that the call sums each pixel in fewer, longer chunks and the image equals bn_render's up
 * to float summation order.  The first call on a device resolves the array's address (set-up):
 * make it before any stream capture.  Calls share the array, so calls that overlap on the GPU race. */
int bn_render_noalloc(bn_context* ctx, const bn_render_desc* desc, const bn_view* views, int32_t n_views,
                      float* film_device);
int bn_get_stats(const bn_context* ctx, bn_stats* out);
int bn_reset_stats(bn_context* ctx);

/* Failure-detection limits (no reference counterpart; the reference's only failure path is
 * failwith).  stack_entries caps the traversal stack a walk may use (1..200; 0 = the full 200):
 * a walk that needs more stops and sets BN_DEVERR_STACK_OVERFLOW.  max_bounce_iterations caps the
 * wavefront's device-side bounce loop (0 = the default cap derived from the paths and depth): a
 * render that needs more stops and sets BN_DEVERR_WATCHDOG.  Either way the call returns
 * BN_ERR_DEVICE and the context stays usable; tests lower them to drive those paths without
 * faulting the GPU.  The limits hold for the context until changed. */
int bn_set_limits(bn_context* ctx, int32_t stack_entries, int32_t max_bounce_iterations);

/* ---- differentiable materials (new; no reference counterpart) --------------------------
 * A parameter vector of n_slots material slots, each
 *   [albedo r, g, b, roughness, metallic, emission_scale]   (6 floats)
 * drives every PBR material slot of the uploaded scene (material index = slot) and scales
 * light l by the emission_scale of slot bn_adjoint_desc.emissive_slot_base + l.
 * bn_forward renders the image for params; bn_backward runs the path-replay adjoint of
 * 0.5 * sum((image - target)^2) and returns d loss / d params in double precision. */
typedef struct bn_adjoint_desc {
  int32_t n_slots;
  int32_t emissive_slot_base;  /* slot index of light 0's emission scale */
  int32_t width, height;
  int32_t spp;
  int32_t max_depth;
  int32_t rr_depth;
  int32_t frame_id;
  int32_t freeze_sampling;     /* 1: sampling pdfs/RR come from sampling_params (FD checks) */
  int32_t pad_;
  bn_camera_desc camera;
} bn_adjoint_desc;

int bn_forward(bn_context* ctx, const bn_adjoint_desc* desc, const float* params,
               const float* sampling_params, float* out_image);
int bn_backward(bn_context* ctx, const bn_adjoint_desc* desc, const float* params,
                const float* sampling_params, const float* target_image, double* d_params,
                double* loss);

/* ---- host preparation helpers (no GPU needed) ----------------------------------------- */
/* 32-byte BVHNode, the reference layout (Util/BVH.fs:52-73) */
typedef struct bn_bvh_node {
  float bounds_min[3];
  float bounds_max[3];
  int32_t right_or_offset; /* interior: right child index; leaf: first item */
  uint8_t is_leaf;
  int8_t split_axis;
  int8_t count;            /* leaf item count */
  uint8_t visibility_mask;
} bn_bvh_node;

/* BVHNode.Build (Util/BVH.fs:239-247): bounds = n * 6 floats (min xyz, max xyz).
 * nodes_out must hold 2n nodes; perm_out[k] = original index of the k-th item after the
 * in-place permutation. */
int bn_bvh_build(const float* bounds, int32_t n, bn_bvh_node* nodes_out, int32_t* n_nodes_out,
                 int32_t* perm_out);
/* The same build on the GPU of ctx, with the same nodes and permutation: node ranges above 256
 * items are split level by level on the device, smaller ones by one device thread each.  Boxes
 * with a NaN coordinate are built by the host builder. */
int bn_bvh_build_device(bn_context* ctx, const float* bounds, int32_t n, bn_bvh_node* nodes_out,
                        int32_t* n_nodes_out, int32_t* perm_out);
/* Matrix4x4.Invert restated (used by Node.Traverse -> UpdateTransform) */
int bn_mat4_invert(const float m[16], float out[16]);

/* Procedural workloads and the JSON loader produce a library-owned scene + render settings. */
typedef struct bn_scene_bundle bn_scene_bundle;
typedef struct bn_bundle_info {
  const bn_scene_desc* scene;
  const bn_view* views;
  int32_t n_views;
  bn_render_desc render;
  int64_t n_triangles_unique;
  int64_t n_triangles_instanced;
  int32_t n_material_slots;       /* differentiable workload: slots, else 0 */
  int32_t emissive_slot_base;
  const float* slot_params;       /* n_material_slots * 6 ground-truth params, or NULL */
  int32_t tone_mapping;           /* bn_tone_mapping of the film (JSON "tone-mapping"; ACES for the
                                     procedural workloads, as the reference's sample images) */
} bn_bundle_info;

/* name: "cornell" (256^2 64spp d8), "cornell-objects" (512^2 256spp d16, icospheres + mirror),
 *       "instances" (1024 instances of 4 displaced icospheres, 16 views),
 *       "pssmlt" (the cornell-objects scene at 1024^2, 65536 chains),
 *       "materials" (the cornell-objects scene with 32 differentiable material slots). */
int bn_bundle_generate(const char* name, uint32_t seed, bn_scene_bundle** out);
/* Scene.Load (Extensions/Scene/Loader.fs:277-281) + Scene.Traverse(0) */
int bn_bundle_load_json(const char* path, bn_scene_bundle** out);
int bn_bundle_info_get(const bn_scene_bundle* b, bn_bundle_info* out);
int bn_bundle_free(bn_scene_bundle* b);
/* copies the last error of a host helper (bundle, bvh) on this thread */
int bn_host_last_error(char* buf, size_t len);

#ifdef __cplusplus
}
#endif
#endif /* BARNACLE_GPU_H */
