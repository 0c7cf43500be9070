// Device-resident scene layout (HBM), written once by bn_scene_upload.
//
//  nodes      2 x float4 per BVHNode, the reference's 32-byte layout (Util/BVH.fs:52-73):
//             n0 = (min.x, min.y, min.z, max.x), n1 = (max.y, max.z, int right|offset,
//             int bytes [is_leaf, split_axis, count, mask]).  TLAS first (root 0), then every
//             mesh's BLAS at DevInstance::node_base.  Loaded as two 16-byte vector loads.
//             The binary walk reads them when it counts visits (the reference's own work).
//  nodes4     8 x float4 (128 B, one cache line) per interior node that the wide walk enters:
//             the two binary levels below it in one record.  Slots 0-1 hold the left child's
//             children (or the left child itself, slot 1 unused, when it is a leaf), slots 2-3
//             the right child's.  (lo.x[4], lo.y[4], lo.z[4], hi.x[4], hi.y[4], hi.z[4]) slot
//             boxes, int4 ref (node4 index of an interior slot, first item of a leaf slot),
//             int4 meta (x: leaf item count, 8 bits per slot; y: leaf mask bits 0-3, split axis
//             of the node << 4, of its left child << 6, of its right child << 8; z, w: the slot
//             visit order for each of the 8 ray octants, 8 bits = 4 x 2-bit slots per octant,
//             octants 0-3 in z, 4-7 in w).  Unused slots
//             have NaN boxes, which no ray enters.  TLAS records first (root at 0 when the TLAS
//             root is interior), then every BLAS at DevInstance::node4_root.  Built when the
//             scene is walked wide (DevScene::wide).
//  tris       3 x float4 per triangle in BLAS-permuted order, all meshes back to back:
//             (p0, material slot or -1), (p1, original index), (p2, 0).  48 bytes = the 12-byte
//             index + 36 bytes of vertices the reference gathers per tested triangle.
//  instances  DevInstance in TLAS-permuted order (BVHAggregate permutes its array in place).
//  materials  DevMaterial (32 B), lights DevLight (16 B).
//  light tables:
//    uniform (Extensions/LightSampler/Uniform.fs): light_inst[] = emissive instances in TLAS
//      order; tri_pdf[global tri] = the reference AliasTable entry pdf of each mesh triangle
//      (area / sum of areas in object space, Util/AliasTable.fs:14-27 + Mesh.fs:181-186).
//    alias-triangles (new plugin): Vose table over all emissive (instance, triangle) pairs,
//      entries DevTriLight; DevInstance::light_entry_base maps a hit back to its entry.
#pragma once
#include <cstdint>

namespace bn {

enum : int { kPrimMesh = 0, kPrimSphere = 1 };
// entries of a walk's stack of far nodes: a depth-64 TLAS and BLAS, the wide walk stacking up to
// three per record level
constexpr int kStackSize = 200;
enum : int { kMatLambertian = 0, kMatMirror = 1, kMatDielectric = 2, kMatPBR = 3 };

// Two 128-byte lines: the first holds everything a walk reads when it visits the instance (read
// with eight independent 16-byte loads), the second what shading reads.
struct alignas(128) DevInstance {
  float4 bmin;      // world AABB min, .w unused
  float4 bmax;      // world AABB max, .w = sphere radius
  float4 w2o[3];    // w2o[r] = (M1r, M2r, M3r, M4r) of WorldToObject: x'_r = ((x*M1r + y*M2r) + z*M3r) + M4r
  float4 rbmin;     // the BLAS root's box (object space) min, .w unused
  float4 rbmax;     // the BLAS root's box max, .w unused
  int prim_type;    // kPrimMesh / kPrimSphere
  int node_base;    // BLAS root in nodes[]
  int tri_base;     // first triangle of the mesh in tris[]
  int node4_root;   // nodes4 record of the BLAS root; -1: binary scene, leaf root or sphere
  float4 o2w[3];    // as w2o for ObjectToWorld
  int n_tris;
  int material;     // -1 = no material (a light only; the path ends there)
  int light;        // -1 = not emissive
  int light_entry_base;  // alias-triangles: entry index of triangle 0 of this instance, -1 if none
};
static_assert(sizeof(DevInstance) == 256, "DevInstance layout");

struct alignas(16) DevMaterial {
  int type;
  float base[3];
  float ior;
  float alpha;     // max(roughness^2, 1e-3) (PBR.fs:106)
  float metallic;  // clamp(metallic, 0, 1) (PBR.fs:107)
  float roughness;
};
static_assert(sizeof(DevMaterial) == 32, "DevMaterial layout");

struct alignas(16) DevLight {
  float emission[3];
  int two_sided;
};

struct alignas(16) DevTriLight {
  float prob;       // Vose acceptance probability
  int alias;        // Vose alias entry
  float pmf;        // probability of picking this entry
  float area;       // world-space area
  int inst;         // instance (TLAS order)
  int tri;          // triangle within the mesh (BLAS order)
  int pad0, pad1;
};

struct DevView {
  float ul[3], du[3], dv[3];  // pinhole viewport: upper-left, pixel deltas (Pinhole.fs:12-27)
  float c2w[16];              // CameraToWorld
  int width, height;
  int cam_type;
  float aperture, focus_distance, push_forward;
  long long pixel_offset;     // first pixel of this view in the concatenated film
  long long path_offset;      // first path id of this view (pixels * spp before it)
};

struct DevScene {
  const float4* __restrict__ nodes;
  const float4* __restrict__ nodes4;
  const float4* __restrict__ tris;
  const DevInstance* __restrict__ inst;
  const DevMaterial* __restrict__ mats;
  const DevLight* __restrict__ lights;
  const int* __restrict__ light_inst;     // uniform sampler: emissive instances
  const float* __restrict__ tri_pdf;      // uniform sampler: reference alias pdf per triangle
  const DevTriLight* __restrict__ tri_lights;  // alias-triangles sampler
  int n_inst;
  int n_tlas_nodes;
  int n_nodes;
  int n_nodes4;
  int wide;                               // walked through nodes4 (kWalkWide kernels)
  int n_tris;
  int n_light_inst;
  int n_tri_lights;
  int light_sampler;                      // 0 uniform, 1 alias-triangles
  int n_mats;
  int stack_cap;                          // usable stack entries (kStackSize; lower for tests)
  unsigned int* error_word;               // BN_DEVERR_* bits
};

}  // namespace bn
