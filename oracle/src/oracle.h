/* ORACLE — test infrastructure only (tests/, the smoke check and bench.py's CPU baseline).
 * CPU restatement of the Barnacle render path; see oracle.cpp for the recorded choices. */
#ifndef BARNACLE_ORACLE_H
#define BARNACLE_ORACLE_H
#include "../../include/barnacle_gpu.h"

#ifdef __cplusplus
extern "C" {
#endif

typedef struct or_scene or_scene;

int or_scene_create(const bn_scene_desc* d, or_scene** out);
void or_scene_free(or_scene* s);
int or_scene_tlas(const or_scene* s, bn_bvh_node* nodes, int32_t* n_nodes, int32_t* order);
int or_scene_blas(const or_scene* s, int32_t mesh, bn_bvh_node* nodes, int32_t* n_nodes, int32_t* perm);
int or_bvh_build(const float* bounds, int32_t n, bn_bvh_node* nodes, int32_t* n_nodes, int32_t* perm);
int or_trace(const or_scene* s, const bn_ray* rays, int64_t n, uint32_t flags, bn_hit* hits, uint64_t* counts);
int or_sampler_stream(const uint32_t* seeds, int64_t n, int32_t draws, float* out);
int or_tonemap(const float* rgb, int64_t n, int32_t tone_mapping, uint8_t* rgba);
uint32_t or_xxhash32_two(uint32_t x, uint32_t y);
uint32_t or_xxhash32_three(uint32_t x, uint32_t y, uint32_t z);
int or_bsdf(const bn_material_desc* materials, const bn_bsdf_query* q, int64_t n, int sample, int use_double,
            double* out7);
int or_render_pt(const or_scene* s, const bn_render_desc* d, const bn_view* view, int32_t x0, int32_t y0, int32_t x1,
                 int32_t y1, int32_t threads, float* out, uint64_t* counts);
int or_render_slots(const or_scene* s, const bn_render_desc* d, const bn_view* view, int32_t n_slots,
                    int32_t emissive_base, const float* params, const float* sparams, int32_t threads, float* out);
int or_render_pssmlt(const or_scene* s, const bn_render_desc* d, const bn_view* view, int32_t threads, float* out,
                     double* stats, float* bootstrap_out);

#ifdef __cplusplus
}
#endif
#endif
