// C-ABI of the host preparation helpers (no GPU involved).
#include <cstring>
#include <string>
#include <vector>

#include "bundle.hpp"
#include "bvh_build.hpp"

namespace {
thread_local std::string g_host_error;
int host_fail(int code, const std::string& msg) {
  g_host_error = msg;
  return code;
}
}  // namespace

// the error channel of bn_host_last_error, for host helpers in other files (png.cpp)
int bnh_host_fail(int code, const std::string& msg) { return host_fail(code, msg); }

extern "C" {

int bn_host_last_error(char* buf, size_t len) {
  if (!buf || len == 0) return static_cast<int>(g_host_error.size());
  std::strncpy(buf, g_host_error.c_str(), len - 1);
  buf[len - 1] = '\0';
  return static_cast<int>(g_host_error.size());
}

int bn_bvh_build(const float* bounds, int32_t n, bn_bvh_node* nodes_out, int32_t* n_nodes_out, int32_t* perm_out) {
  if (n < 0 || (n > 0 && (!bounds || !perm_out)) || !nodes_out || !n_nodes_out)
    return host_fail(BN_ERR_INVALID_ARG, "bn_bvh_build: null pointer or negative count");
  std::vector<bn_bvh_node> nodes;
  std::vector<int32_t> perm;
  const bool ok = bnh::bvh_build(bounds, n, &nodes, &perm);
  if (!ok) return host_fail(BN_ERR_UNSUPPORTED, "bn_bvh_build: a depth-capped leaf holds more than 127 items");
  std::memcpy(nodes_out, nodes.data(), nodes.size() * sizeof(bn_bvh_node));
  if (n > 0) std::memcpy(perm_out, perm.data(), perm.size() * sizeof(int32_t));
  *n_nodes_out = static_cast<int32_t>(nodes.size());
  return BN_OK;
}

int bn_mat4_invert(const float m[16], float out[16]) {
  if (!m || !out) return host_fail(BN_ERR_INVALID_ARG, "bn_mat4_invert: null pointer");
  bnh::M4 a, r;
  std::memcpy(a.m, m, sizeof(a.m));
  const bool ok = bnh::m4_invert(a, &r);
  std::memcpy(out, r.m, sizeof(r.m));
  return ok ? BN_OK : host_fail(BN_ERR_INVALID_ARG, "bn_mat4_invert: singular matrix");
}

int bn_bundle_generate(const char* name, uint32_t seed, bn_scene_bundle** out) {
  if (!name || !out) return host_fail(BN_ERR_INVALID_ARG, "bn_bundle_generate: null pointer");
  auto* b = new bn_scene_bundle();
  std::string err;
  if (!bnh::generate_bundle(name, seed, b, &err)) {
    delete b;
    return host_fail(BN_ERR_INVALID_ARG, err);
  }
  *out = b;
  return BN_OK;
}

int bn_bundle_load_json(const char* path, bn_scene_bundle** out) {
  if (!path || !out) return host_fail(BN_ERR_INVALID_ARG, "bn_bundle_load_json: null pointer");
  auto* b = new bn_scene_bundle();
  std::string err;
  if (!bnh::load_json_bundle(path, b, &err)) {
    delete b;
    return host_fail(BN_ERR_IO, err);
  }
  *out = b;
  return BN_OK;
}

int bn_bundle_info_get(const bn_scene_bundle* b, bn_bundle_info* out) {
  if (!b || !out) return host_fail(BN_ERR_INVALID_ARG, "bn_bundle_info_get: null pointer");
  out->scene = &b->scene;
  out->views = b->views.data();
  out->n_views = static_cast<int32_t>(b->views.size());
  out->render = b->render;
  out->n_triangles_unique = b->tri_unique;
  out->n_triangles_instanced = b->tri_instanced;
  out->n_material_slots = b->n_slots;
  out->emissive_slot_base = b->emissive_slot_base;
  out->slot_params = b->slot_params.empty() ? nullptr : b->slot_params.data();
  out->tone_mapping = b->tone_mapping;
  return BN_OK;
}

int bn_bundle_free(bn_scene_bundle* b) {
  delete b;
  return BN_OK;
}

}  // extern "C"
