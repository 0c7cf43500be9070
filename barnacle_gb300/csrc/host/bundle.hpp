// A library-owned scene description plus render settings: what Scene.Load + Scene.Traverse(0)
// produce in the reference (Extensions/Scene/Loader.fs:253-281, Base/Scene.fs:38-61), in the
// flat form of bn_scene_desc.
#pragma once
#include <cstdint>
#include <string>
#include <vector>

#include "../../../include/barnacle_gpu.h"
#include "host_math.hpp"

struct bn_scene_bundle {
  std::vector<std::vector<float>> mesh_vertices;
  std::vector<std::vector<int32_t>> mesh_indices;
  std::vector<std::vector<int32_t>> mesh_trimat;
  std::vector<bn_mesh_desc> meshes;
  std::vector<bn_primitive_desc> primitives;
  std::vector<bn_instance_desc> instances;
  std::vector<bn_material_desc> materials;
  std::vector<bn_light_desc> lights;
  std::vector<bn_view> views;
  bn_scene_desc scene{};
  bn_render_desc render{};
  int32_t light_sampler = BN_LIGHTS_UNIFORM;
  int32_t tone_mapping = BN_TONE_ACES;
  int32_t n_slots = 0;
  int32_t emissive_slot_base = 0;
  std::vector<float> slot_params;
  int64_t tri_unique = 0;
  int64_t tri_instanced = 0;

  int add_mesh(std::vector<float> v, std::vector<int32_t> idx, std::vector<int32_t> trimat = {});
  int add_sphere(float radius);
  int add_material(int type, bnh::V3 color, float ior = 1.5f, float roughness = 1.f, float metallic = 0.f);
  int add_light(bnh::V3 emission, bool two_sided = true);
  int add_instance(int primitive, int material, int light, const bnh::M4& object_to_world);
  void finalize();  // fills the pointer fields of scene / meshes and the triangle counts
};

namespace bnh {
bn_render_desc default_render_desc();
bool generate_bundle(const std::string& name, uint32_t seed, bn_scene_bundle* b, std::string* err);
bool load_json_bundle(const std::string& path, bn_scene_bundle* b, std::string* err);
bool load_obj(const std::string& path, std::vector<float>* v, std::vector<int32_t>* idx, std::string* err);
}  // namespace bnh
