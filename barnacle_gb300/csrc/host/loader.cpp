// Scene.Load + Scene.Traverse(0) for the reference's JSON scene schema
// (Extensions/Scene/Loader.fs:14-281, Base/Scene.fs:8-61) and the OBJ reader
// (Extensions/Primitive/Mesh.fs:246-279).
//
// Schema facts kept from the reference:
//  * keyframe matrix = CreateScale * (RotX * RotY * RotZ) * CreateTranslation, rotation values
//    in RADIANS, passed straight to CreateRotationX/Y/Z (Loader.fs:24-45)
//  * Transform.Eval(t): the last keyframe with time <= t; before the first keyframe, the first;
//    between two keyframes KeyFrame.Interpolate (Scene.fs:13-36), with the reference's
//    Transform.Compose that swaps scale and translation (keyframe_interpolate, host_math.cpp).
//    Scene.Render is called with t = 0 (Program.fs:27), so interpolation happens for
//    keyframes on both sides of time 0.
//  * node world matrix = Eval(t) * parent (local . parent, row vectors) (Scene.fs:44)
//  * an instance listed under several nodes appears once per listing, all with the transform
//    of the last traversal (PrimitiveInstance is one mutable object, Primitive.fs:131-138)
//  * the camera takes the world matrix of the last node with "has-camera" (zero matrix if none)
//  * defaults: albedo 1, ior 1.5, roughness 1, metallic 0 (Loader.fs:118-126); two-sided true
//    (:149); spp 1, max-depth 8, rr-depth 5, n-bootstrap 4M, n-chains 1024, Gaussian 1e-2,
//    Kelemen (1/1024, 1/16), large-step 0.5 (:241-262); fov 45, aspect 1, aperture 0,
//    focus 1, push-forward 0 (:275-279)
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <functional>
#include <map>
#include <memory>
#include <sstream>
#include <string>
#include <vector>

#include "bundle.hpp"

namespace bnh {
namespace {

// ------------------------------------------------------------------ minimal JSON
struct JVal {
  enum Kind { Null, Bool, Num, Str, Arr, Obj } kind = Null;
  bool b = false;
  double num = 0;
  std::string str;
  std::vector<JVal> arr;
  std::vector<std::pair<std::string, JVal>> obj;
  const JVal* get(const char* key) const {
    if (kind != Obj) return nullptr;
    for (const auto& kv : obj)
      if (kv.first == key) return kv.second.kind == Null ? nullptr : &kv.second;
    return nullptr;
  }
};

struct JParser {
  const char* p;
  const char* end;
  std::string err;
  void ws() {
    while (p < end && (*p == ' ' || *p == '\n' || *p == '\r' || *p == '\t')) ++p;
  }
  bool fail(const char* m) {
    if (err.empty()) err = m;
    return false;
  }
  bool parse(JVal* v) {
    ws();
    if (p >= end) return fail("unexpected end of JSON");
    const char c = *p;
    if (c == '{') {
      ++p;
      v->kind = JVal::Obj;
      ws();
      if (p < end && *p == '}') { ++p; return true; }
      for (;;) {
        ws();
        JVal key;
        if (p >= end || *p != '"' || !parse_str(&key.str)) return fail("expected object key");
        ws();
        if (p >= end || *p != ':') return fail("expected ':'");
        ++p;
        JVal val;
        if (!parse(&val)) return false;
        v->obj.emplace_back(key.str, std::move(val));
        ws();
        if (p < end && *p == ',') { ++p; continue; }
        if (p < end && *p == '}') { ++p; return true; }
        return fail("expected ',' or '}'");
      }
    }
    if (c == '[') {
      ++p;
      v->kind = JVal::Arr;
      ws();
      if (p < end && *p == ']') { ++p; return true; }
      for (;;) {
        JVal val;
        if (!parse(&val)) return false;
        v->arr.push_back(std::move(val));
        ws();
        if (p < end && *p == ',') { ++p; continue; }
        if (p < end && *p == ']') { ++p; return true; }
        return fail("expected ',' or ']'");
      }
    }
    if (c == '"') { v->kind = JVal::Str; return parse_str(&v->str); }
    if (end - p >= 4 && std::strncmp(p, "true", 4) == 0) { v->kind = JVal::Bool; v->b = true; p += 4; return true; }
    if (end - p >= 5 && std::strncmp(p, "false", 5) == 0) { v->kind = JVal::Bool; p += 5; return true; }
    if (end - p >= 4 && std::strncmp(p, "null", 4) == 0) { v->kind = JVal::Null; p += 4; return true; }
    if (c == '-' || (c >= '0' && c <= '9')) {
      std::string tok;
      while (p < end && (std::strchr("+-.eE", *p) || (*p >= '0' && *p <= '9'))) tok.push_back(*p++);
      char* e = nullptr;
      v->kind = JVal::Num;
      v->num = std::strtod(tok.c_str(), &e);
      if (!e || *e) return fail("bad number");
      return true;
    }
    return fail("unexpected character in JSON");
  }
  bool parse_str(std::string* out) {
    ++p;  // opening quote
    while (p < end && *p != '"') {
      if (*p == '\\') {
        ++p;
        if (p >= end) return fail("bad escape");
        const char e = *p++;
        switch (e) {
          case 'n': out->push_back('\n'); break;
          case 't': out->push_back('\t'); break;
          case 'r': out->push_back('\r'); break;
          case 'b': out->push_back('\b'); break;
          case 'f': out->push_back('\f'); break;
          case 'u': {
            if (end - p < 4) return fail("bad \\u escape");
            const unsigned cp = static_cast<unsigned>(std::strtoul(std::string(p, 4).c_str(), nullptr, 16));
            p += 4;
            if (cp < 0x80) out->push_back(static_cast<char>(cp));
            else if (cp < 0x800) { out->push_back(static_cast<char>(0xC0 | (cp >> 6))); out->push_back(static_cast<char>(0x80 | (cp & 0x3F))); }
            else { out->push_back(static_cast<char>(0xE0 | (cp >> 12))); out->push_back(static_cast<char>(0x80 | ((cp >> 6) & 0x3F))); out->push_back(static_cast<char>(0x80 | (cp & 0x3F))); }
            break;
          }
          default: out->push_back(e);
        }
      } else {
        out->push_back(*p++);
      }
    }
    if (p >= end) return fail("unterminated string");
    ++p;
    return true;
  }
};

float fnum(const JVal* v, float dflt) { return (v && v->kind == JVal::Num) ? static_cast<float>(v->num) : dflt; }
int inum(const JVal* v, int dflt) { return (v && v->kind == JVal::Num) ? static_cast<int>(v->num) : dflt; }
bool jbool(const JVal* v, bool dflt) { return (v && v->kind == JVal::Bool) ? v->b : dflt; }
std::string jstr(const JVal* v) { return (v && v->kind == JVal::Str) ? v->str : std::string(); }
bool farr(const JVal* v, size_t n, float* out) {
  if (!v || v->kind != JVal::Arr || v->arr.size() < n) return false;
  for (size_t i = 0; i < n; ++i) out[i] = static_cast<float>(v->arr[i].num);
  return true;
}

struct Keyframe {
  float time;
  M4 m;
};

M4 keyframe_matrix(const JVal& k) {
  float s[3], r[3], t[3];
  M4 S = farr(k.get("scale"), 3, s) ? m4_scale(s[0], s[1], s[2]) : m4_identity();
  M4 R = m4_identity();
  if (farr(k.get("rotation"), 3, r)) {
    // CreateRotationX(r0) * CreateRotationY(r1) * CreateRotationZ(r2), radians
    R = m4_mul(m4_mul(m4_rot_x(std::cos(r[0]), std::sin(r[0])), m4_rot_y(std::cos(r[1]), std::sin(r[1]))),
               m4_rot_z(std::cos(r[2]), std::sin(r[2])));
  }
  M4 T = farr(k.get("translation"), 3, t) ? m4_translation(t[0], t[1], t[2]) : m4_identity();
  return m4_mul(m4_mul(S, R), T);
}

}  // namespace

bool load_obj(const std::string& path, std::vector<float>* v, std::vector<int32_t>* idx, std::string* err) {
  std::ifstream in(path);
  if (!in) {
    *err = "cannot open OBJ file " + path;
    return false;
  }
  v->clear();
  idx->clear();
  std::string line;
  while (std::getline(in, line)) {
    size_t a = line.find_first_not_of(" \t\r");
    size_t z = line.find_last_not_of(" \t\r");
    if (a == std::string::npos) continue;
    line = line.substr(a, z - a + 1);
    if (line.rfind("v ", 0) == 0) {
      std::istringstream ss(line.substr(2));
      float x, y, w;
      if (!(ss >> x >> y >> w)) { *err = "bad vertex line in " + path; return false; }
      v->push_back(x); v->push_back(y); v->push_back(w);
    } else if (line.rfind("f ", 0) == 0) {
      std::istringstream ss(line.substr(2));
      std::vector<int32_t> f;
      std::string tok;
      const int32_t nv = static_cast<int32_t>(v->size() / 3);
      while (ss >> tok) {
        const size_t slash = tok.find('/');
        const int32_t i = std::atoi(tok.substr(0, slash).c_str());
        f.push_back(i < 0 ? nv + i : i - 1);  // Mesh.fs:262-267
      }
      if (f.size() < 3) { *err = "face with fewer than 3 vertices in " + path; return false; }
      for (size_t k = 2; k < f.size(); ++k) {  // fan triangulation (Mesh.fs:269-277)
        idx->push_back(f[0]); idx->push_back(f[k - 1]); idx->push_back(f[k]);
      }
    }
  }
  return true;
}

bool load_json_bundle(const std::string& path, bn_scene_bundle* b, std::string* err) {
  std::ifstream in(path, std::ios::binary);
  if (!in) { *err = "cannot open scene file " + path; return false; }
  std::stringstream ss;
  ss << in.rdbuf();
  std::string text = ss.str();
  // a UTF-8 byte-order mark is allowed at the start (the reference's cbox.json has one)
  size_t off = (text.size() >= 3 && static_cast<unsigned char>(text[0]) == 0xEF) ? 3 : 0;
  JParser jp{text.data() + off, text.data() + text.size(), {}};
  JVal root;
  if (!jp.parse(&root) || root.kind != JVal::Obj) { *err = "JSON parse error: " + jp.err; return false; }
  const std::string dir = path.find('/') == std::string::npos ? std::string(".") : path.substr(0, path.rfind('/'));

  // transforms (Loader.fs:103-108): keyframes sorted by time
  std::vector<std::vector<Keyframe>> transforms;
  if (const JVal* ts = root.get("transforms"))
    for (const JVal& t : ts->arr) {
      std::vector<Keyframe> ks;
      if (const JVal* kf = t.get("keyframes"))
        for (const JVal& k : kf->arr) ks.push_back({fnum(k.get("time"), 0.f), keyframe_matrix(k)});
      if (ks.empty()) { *err = "KeyFrames cannot be empty"; return false; }
      std::stable_sort(ks.begin(), ks.end(), [](const Keyframe& x, const Keyframe& y) { return x.time < y.time; });
      transforms.push_back(std::move(ks));
    }
  // primitives (Loader.fs:159-176)
  std::vector<int> prim_ids;
  if (const JVal* ps = root.get("primitives"))
    for (const JVal& p : ps->arr) {
      const std::string type = jstr(p.get("type"));
      if (type == "sphere") {
        prim_ids.push_back(b->add_sphere(fnum(p.get("radius"), 1.f)));
      } else if (type == "quad") {
        prim_ids.push_back(b->add_mesh({-1, 0, -1, 1, 0, -1, 1, 0, 1, -1, 0, 1}, {0, 1, 2, 0, 2, 3}));
      } else if (type == "cube") {
        prim_ids.push_back(b->add_mesh({-1, -1, -1, 1, -1, -1, 1, 1, -1, -1, 1, -1, -1, -1, 1, 1, -1, 1, 1, 1, 1, -1, 1, 1},
                                       {0, 2, 1, 0, 3, 2, 4, 5, 6, 4, 6, 7, 0, 1, 5, 0, 5, 4,
                                        3, 7, 6, 3, 6, 2, 0, 4, 7, 0, 7, 3, 1, 2, 6, 1, 6, 5}));
      } else if (type == "mesh") {
        const std::string uri = jstr(p.get("uri"));
        std::vector<float> v;
        std::vector<int32_t> idx;
        if (!uri.empty()) {
          std::string e1;
          if (!load_obj(uri, &v, &idx, &e1) && !load_obj(dir + "/" + uri, &v, &idx, err)) return false;
        } else if (p.get("vertices") && p.get("indices")) {
          for (const JVal& x : p.get("vertices")->arr) v.push_back(static_cast<float>(x.num));
          for (const JVal& x : p.get("indices")->arr) idx.push_back(static_cast<int32_t>(x.num));
          v.resize(v.size() / 3 * 3);
        } else {
          *err = "Invalid mesh primitive";
          return false;
        }
        prim_ids.push_back(b->add_mesh(std::move(v), std::move(idx)));
      } else {
        *err = "Unknown primitive type: " + type;
        return false;
      }
    }
  // materials (Loader.fs:117-133)
  if (const JVal* ms = root.get("materials"))
    for (const JVal& m : ms->arr) {
      float a[3] = {1.f, 1.f, 1.f};
      farr(m.get("albedo"), 3, a);
      const std::string type = jstr(m.get("type"));
      int t;
      if (type == "lambertian") t = BN_MAT_LAMBERTIAN;
      else if (type == "mirror") t = BN_MAT_MIRROR;
      else if (type == "dielectric") t = BN_MAT_DIELECTRIC;
      else if (type == "pbr") t = BN_MAT_PBR;
      else { *err = "Unknown material type: " + type; return false; }
      b->add_material(t, v3(a[0], a[1], a[2]), fnum(m.get("ior"), 1.5f), fnum(m.get("roughness"), 1.f),
                      fnum(m.get("metallic"), 0.f));
    }
  // lights (Loader.fs:140-150)
  if (const JVal* ls = root.get("lights"))
    for (const JVal& l : ls->arr) {
      if (jstr(l.get("type")) != "diffuse") { *err = "Unknown light type: " + jstr(l.get("type")); return false; }
      float e[3] = {0.f, 0.f, 0.f};
      farr(l.get("emission"), 3, e);
      b->add_light(v3(e[0], e[1], e[2]), jbool(l.get("two-sided"), true));
    }
  // instances (Loader.fs:183-205): kept as templates until traversal gives them a transform
  struct InstTemplate { int prim, mat, light; };
  std::vector<InstTemplate> templates;
  if (const JVal* is = root.get("instances"))
    for (const JVal& i : is->arr) {
      const int prim = inum(i.get("primitive"), -1);
      if (prim < 0 || prim >= static_cast<int>(prim_ids.size())) { *err = "instance primitive out of range"; return false; }
      const int mat = inum(i.get("material"), -1), light = inum(i.get("light"), -1);
      if (mat >= static_cast<int>(b->materials.size()) || light >= static_cast<int>(b->lights.size())) {
        *err = "instance material/light out of range";
        return false;
      }
      templates.push_back({prim_ids[prim], mat, light});
    }
  // nodes (Loader.fs:213-228, :327-330) and traversal at t = 0 (Scene.fs:43-61)
  struct NodeT { int transform; std::vector<int> instances, children; bool camera; };
  std::vector<NodeT> nodes;
  if (const JVal* ns = root.get("nodes"))
    for (const JVal& n : ns->arr) {
      NodeT nd{inum(n.get("transform"), -1), {}, {}, jbool(n.get("has-camera"), false)};
      if (const JVal* a = n.get("instances")) for (const JVal& x : a->arr) nd.instances.push_back(static_cast<int>(x.num));
      if (const JVal* a = n.get("children")) for (const JVal& x : a->arr) nd.children.push_back(static_cast<int>(x.num));
      nodes.push_back(std::move(nd));
    }
  if (nodes.empty()) { *err = "scene has no nodes"; return false; }
  const float t_render = 0.f;
  std::vector<int> order;        // instance template per traversal visit
  std::map<int, M4> final_xf;    // last transform written into each instance object
  M4 camera_xf = m4_zero();
  struct Frame { int node; M4 parent; int depth; };
  std::vector<Frame> stack;
  const int root_id = inum(root.get("root"), 0);
  if (root_id < 0 || root_id >= static_cast<int>(nodes.size())) { *err = "root node out of range"; return false; }
  // recursive traversal in reference order: instances of a node, then its children in order
  std::function<bool(int, const M4&, int)> visit = [&](int id, const M4& parent, int depth) -> bool {
    if (depth > 1000) { *err = "node graph is cyclic or too deep"; return false; }
    const NodeT& nd = nodes[id];
    M4 local = m4_identity();
    if (nd.transform >= 0) {
      if (nd.transform >= static_cast<int>(transforms.size())) { *err = "node transform out of range"; return false; }
      const auto& ks = transforms[nd.transform];
      int prev = -1;
      for (int k = static_cast<int>(ks.size()) - 1; k >= 0; --k)
        if (ks[k].time <= t_render) { prev = k; break; }
      if (prev < 0) local = ks[0].m;
      else if (prev == static_cast<int>(ks.size()) - 1) local = ks[prev].m;
      else local = keyframe_interpolate(ks[prev].time, ks[prev].m, ks[prev + 1].time, ks[prev + 1].m, t_render);
    }
    const M4 world = m4_mul(local, parent);
    if (nd.camera) camera_xf = world;
    for (int i : nd.instances) {
      if (i < 0 || i >= static_cast<int>(templates.size())) { *err = "node instance out of range"; return false; }
      final_xf[i] = world;
      order.push_back(i);
    }
    for (int c : nd.children) {
      if (c < 0 || c >= static_cast<int>(nodes.size())) { *err = "node child out of range"; return false; }
      if (!visit(c, world, depth + 1)) return false;
    }
    return true;
  };
  if (!visit(root_id, m4_identity(), 0)) return false;
  for (int i : order) b->add_instance(templates[i].prim, templates[i].mat, templates[i].light, final_xf[i]);

  // integrator (Loader.fs:240-264)
  bn_render_desc r = default_render_desc();
  const JVal* ig = root.get("integrator");
  const std::string itype = ig ? jstr(ig->get("type")) : std::string();
  r.spp = inum(ig ? ig->get("spp") : nullptr, 1);
  r.max_depth = inum(ig ? ig->get("max-depth") : nullptr, 8);
  r.rr_depth = inum(ig ? ig->get("rr-depth") : nullptr, 5);
  if (itype == "path-tracing") {
    r.integrator = BN_INTEGRATOR_PATH;
  } else if (itype == "pssmlt") {
    r.integrator = BN_INTEGRATOR_PSSMLT;
    r.n_bootstrap = inum(ig->get("n-bootstrap"), 4 * 1024 * 1024);
    r.n_chains = inum(ig->get("n-chains"), 1024);
    const std::string ms = jstr(ig->get("mutation-strategy"));
    if (ms.empty() || ms == "Gaussian") { r.mutation = BN_MUTATION_GAUSSIAN; r.sigma = 1e-2f; }
    else if (ms == "Kelemen") { r.mutation = BN_MUTATION_KELEMEN; r.eps_min = 1.f / 1024.f; r.eps_max = 1.f / 16.f; }
    else { *err = "Unknown mutation strategy: " + ms; return false; }
    r.large_step_prob = fnum(ig->get("large-step-prob"), 0.5f);
  } else if (itype == "normal") {
    r.integrator = BN_INTEGRATOR_NORMAL;   // NormalIntegrator(spp) (Loader.fs:186)
  } else if (itype == "direct") {
    r.integrator = BN_INTEGRATOR_DIRECT;   // DirectIntegrator(spp) (Loader.fs:187)
  } else {
    *err = "Unknown integrator type: " + itype;
    return false;
  }
  b->render = r;
  // camera (Loader.fs:274-284) and film (:291-299)
  const JVal* cj = root.get("camera");
  bn_view view{};
  const std::string ctype = cj ? jstr(cj->get("type")) : std::string();
  if (ctype == "pinhole") view.camera.type = BN_CAM_PINHOLE;
  else if (ctype == "thin-lens") view.camera.type = BN_CAM_THIN_LENS;
  else { *err = "Unknown camera type: " + ctype; return false; }
  view.camera.fov_y_degrees = fnum(cj->get("fov"), 45.f);
  view.camera.aspect_ratio = fnum(cj->get("aspect-ratio"), 1.f);
  view.camera.aperture = fnum(cj->get("aperture"), 0.f);
  view.camera.focus_distance = fnum(cj->get("focus-distance"), 1.f);
  view.camera.push_forward = fnum(cj->get("push-forward"), 0.f);
  std::memcpy(view.camera.camera_to_world, camera_xf.m, sizeof(camera_xf.m));
  const JVal* fj = root.get("film");
  if (!fj) { *err = "scene has no film"; return false; }
  const std::string tm = jstr(fj->get("tone-mapping"));
  if (tm == "aces") b->tone_mapping = BN_TONE_ACES;
  else if (tm == "gamma") b->tone_mapping = BN_TONE_GAMMA;
  else if (tm == "identity") b->tone_mapping = BN_TONE_IDENTITY;
  else { *err = "Unknown tone mapping type: " + tm; return false; }
  view.width = inum(fj->get("width"), 0);
  view.height = inum(fj->get("height"), 0);
  if (view.width <= 0 || view.height <= 0) { *err = "film width/height must be positive"; return false; }
  b->views.push_back(view);
  b->light_sampler = BN_LIGHTS_UNIFORM;  // Render.fs:14 hardwires UniformLightSampler
  b->finalize();
  return true;
}

}  // namespace bnh
