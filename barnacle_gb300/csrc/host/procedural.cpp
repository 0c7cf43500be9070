// Procedural, seeded workloads: the Cornell box, the Cornell box with displaced icospheres and
// a mirror, the 1,024-instance scene with 16 views, the PSSMLT setting, and the 32-slot
// differentiable-material scene.  Everything is built from +,-,*,/,sqrt,floor and a
// deterministic sine/cosine, so the same seed gives the same bits on every host; random draws
// are taken one per statement (or declarator), never as several arguments of one call, whose
// evaluation order C++ leaves to the compiler.
#include <cmath>
#include <cstring>
#include <map>
#include <string>
#include <utility>
#include <vector>

#include "bundle.hpp"

using namespace bnh;

// ---------------------------------------------------------------- bundle helpers
int bn_scene_bundle::add_mesh(std::vector<float> v, std::vector<int32_t> idx, std::vector<int32_t> trimat) {
  mesh_vertices.push_back(std::move(v));
  mesh_indices.push_back(std::move(idx));
  mesh_trimat.push_back(std::move(trimat));
  bn_primitive_desc p{};
  p.type = BN_PRIM_MESH;
  p.mesh = static_cast<int32_t>(mesh_vertices.size()) - 1;
  primitives.push_back(p);
  return static_cast<int>(primitives.size()) - 1;
}
int bn_scene_bundle::add_sphere(float radius) {
  bn_primitive_desc p{};
  p.type = BN_PRIM_SPHERE;
  p.mesh = -1;
  p.radius = radius;
  primitives.push_back(p);
  return static_cast<int>(primitives.size()) - 1;
}
int bn_scene_bundle::add_material(int type, V3 c, float ior, float roughness, float metallic) {
  bn_material_desc m{};
  m.type = type;
  m.base_color[0] = c.x; m.base_color[1] = c.y; m.base_color[2] = c.z;
  m.ior = ior; m.roughness = roughness; m.metallic = metallic;
  materials.push_back(m);
  return static_cast<int>(materials.size()) - 1;
}
int bn_scene_bundle::add_light(V3 e, bool two_sided) {
  bn_light_desc l{};
  l.emission[0] = e.x; l.emission[1] = e.y; l.emission[2] = e.z;
  l.two_sided = two_sided ? 1 : 0;
  lights.push_back(l);
  return static_cast<int>(lights.size()) - 1;
}
int bn_scene_bundle::add_instance(int primitive, int material, int light, const M4& o2w) {
  bn_instance_desc d{};
  d.primitive = primitive; d.material = material; d.light = light;
  std::memcpy(d.object_to_world, o2w.m, sizeof(d.object_to_world));
  M4 inv;
  m4_invert(o2w, &inv);
  std::memcpy(d.world_to_object, inv.m, sizeof(d.world_to_object));
  instances.push_back(d);
  return static_cast<int>(instances.size()) - 1;
}
void bn_scene_bundle::finalize() {
  meshes.resize(mesh_vertices.size());
  tri_unique = 0;
  for (size_t i = 0; i < meshes.size(); ++i) {
    bn_mesh_desc& m = meshes[i];
    m.vertices = mesh_vertices[i].data();
    m.indices = mesh_indices[i].data();
    m.tri_material = mesh_trimat[i].empty() ? nullptr : mesh_trimat[i].data();
    m.n_vertices = static_cast<int32_t>(mesh_vertices[i].size() / 3);
    m.n_triangles = static_cast<int32_t>(mesh_indices[i].size() / 3);
    tri_unique += m.n_triangles;
  }
  tri_instanced = 0;
  for (const auto& in : instances) {
    const bn_primitive_desc& p = primitives[in.primitive];
    if (p.type == BN_PRIM_MESH) tri_instanced += static_cast<int64_t>(mesh_indices[p.mesh].size() / 3);
  }
  scene.primitives = primitives.data(); scene.n_primitives = static_cast<int32_t>(primitives.size());
  scene.meshes = meshes.data(); scene.n_meshes = static_cast<int32_t>(meshes.size());
  scene.instances = instances.data(); scene.n_instances = static_cast<int32_t>(instances.size());
  scene.materials = materials.data(); scene.n_materials = static_cast<int32_t>(materials.size());
  scene.lights = lights.data(); scene.n_lights = static_cast<int32_t>(lights.size());
  scene.light_sampler = light_sampler;
}

namespace bnh {

bn_render_desc default_render_desc() {
  // defaults of IntegratorInfo.ToIntegrator (Extensions/Scene/Loader.fs:170-204)
  bn_render_desc r{};
  r.integrator = BN_INTEGRATOR_PATH;
  r.mode = BN_MODE_MEGAKERNEL;
  r.spp = 1;
  r.max_depth = 8;
  r.rr_depth = 5;
  r.frame_id = 0;
  r.n_bootstrap = 4 * 1024 * 1024;
  r.n_chains = 1024;
  r.mutation = BN_MUTATION_GAUSSIAN;
  r.large_step_prob = 0.5f;
  r.sigma = 1e-2f;
  r.eps_min = 1.f / 1024.f;
  r.eps_max = 1.f / 16.f;
  return r;
}

namespace {

// splitmix64 stream
struct Rng {
  uint64_t s;
  explicit Rng(uint64_t seed) : s(seed * 0x9E3779B97F4A7C15ull + 0x632BE59BD9B4E019ull) {}
  uint64_t next() {
    uint64_t z = (s += 0x9E3779B97F4A7C15ull);
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
  }
  double uniform() { return static_cast<double>(next() >> 11) * (1.0 / 9007199254740992.0); }
  float uniformf(float lo, float hi) { return static_cast<float>(lo + (hi - lo) * uniform()); }
  int below(int n) { return static_cast<int>(uniform() * n); }
};

M4 rot_y_degrees(double deg) {
  double s, c;
  det_sincos(deg * 3.14159265358979323846 / 180.0, &s, &c);
  return m4_rot_y(static_cast<float>(c), static_cast<float>(s));
}

// uniform random rotation: a unit quaternion from rejection sampling in the 4-cube
M4 random_rotation(Rng& r) {
  double q[4], n2;
  do {
    for (double& x : q) x = 2.0 * r.uniform() - 1.0;
    n2 = q[0] * q[0] + q[1] * q[1] + q[2] * q[2] + q[3] * q[3];
  } while (n2 > 1.0 || n2 < 1e-6);
  const double inv = 1.0 / std::sqrt(n2);
  const double x = q[0] * inv, y = q[1] * inv, z = q[2] * inv, w = q[3] * inv;
  M4 m = m4_identity();
  m.m[0] = static_cast<float>(1 - 2 * (y * y + z * z));
  m.m[1] = static_cast<float>(2 * (x * y + z * w));
  m.m[2] = static_cast<float>(2 * (x * z - y * w));
  m.m[4] = static_cast<float>(2 * (x * y - z * w));
  m.m[5] = static_cast<float>(1 - 2 * (x * x + z * z));
  m.m[6] = static_cast<float>(2 * (y * z + x * w));
  m.m[8] = static_cast<float>(2 * (x * z + y * w));
  m.m[9] = static_cast<float>(2 * (y * z - x * w));
  m.m[10] = static_cast<float>(1 - 2 * (x * x + y * y));
  return m;
}

// camera-to-world for a camera at eye looking at target (camera looks down -z, y up)
M4 look_at(V3 eye, V3 target, V3 up) {
  V3 f = normalize(target - eye);
  V3 r = normalize(cross(f, up));
  V3 u = cross(r, f);
  M4 m = m4_identity();
  m.m[0] = r.x; m.m[1] = r.y; m.m[2] = r.z;
  m.m[4] = u.x; m.m[5] = u.y; m.m[6] = u.z;
  m.m[8] = -f.x; m.m[9] = -f.y; m.m[10] = -f.z;
  m.m[12] = eye.x; m.m[13] = eye.y; m.m[14] = eye.z;
  return m;
}

bn_view make_view(const M4& c2w, float fov, int w, int h) {
  bn_view v{};
  v.camera.type = BN_CAM_PINHOLE;
  v.camera.fov_y_degrees = fov;
  v.camera.aspect_ratio = static_cast<float>(w) / static_cast<float>(h);
  v.camera.aperture = 0.f;
  v.camera.focus_distance = 1.f;
  v.camera.push_forward = 0.f;
  std::memcpy(v.camera.camera_to_world, c2w.m, sizeof(c2w.m));
  v.width = w;
  v.height = h;
  return v;
}

// ------------------------------------------------------------ value noise (4 octaves)
uint32_t lattice_hash(int32_t x, int32_t y, int32_t z, uint32_t seed) {
  uint32_t h = seed * 0x27d4eb2du;
  h ^= static_cast<uint32_t>(x) * 0x85ebca6bu;
  h = (h << 13) | (h >> 19);
  h ^= static_cast<uint32_t>(y) * 0xc2b2ae35u;
  h = (h << 11) | (h >> 21);
  h ^= static_cast<uint32_t>(z) * 0x9e3779b1u;
  h ^= h >> 16; h *= 0x7feb352du; h ^= h >> 15; h *= 0x846ca68bu; h ^= h >> 16;
  return h;
}
double lattice_value(int32_t x, int32_t y, int32_t z, uint32_t seed) {
  return static_cast<double>(lattice_hash(x, y, z, seed) >> 8) * (2.0 / 16777216.0) - 1.0;
}
double value_noise(double x, double y, double z, uint32_t seed) {
  const double fx = std::floor(x), fy = std::floor(y), fz = std::floor(z);
  const int32_t ix = static_cast<int32_t>(fx), iy = static_cast<int32_t>(fy), iz = static_cast<int32_t>(fz);
  auto smooth = [](double t) { return t * t * (3.0 - 2.0 * t); };
  const double tx = smooth(x - fx), ty = smooth(y - fy), tz = smooth(z - fz);
  double c[2][2][2];
  for (int a = 0; a < 2; ++a)
    for (int b = 0; b < 2; ++b)
      for (int d = 0; d < 2; ++d) c[a][b][d] = lattice_value(ix + a, iy + b, iz + d, seed);
  auto lerp = [](double a, double b, double t) { return a + (b - a) * t; };
  const double x00 = lerp(c[0][0][0], c[1][0][0], tx), x10 = lerp(c[0][1][0], c[1][1][0], tx);
  const double x01 = lerp(c[0][0][1], c[1][0][1], tx), x11 = lerp(c[0][1][1], c[1][1][1], tx);
  return lerp(lerp(x00, x10, ty), lerp(x01, x11, ty), tz);
}
double fbm4(double x, double y, double z, uint32_t seed) {
  double sum = 0.0, amp = 1.0, freq = 2.0, norm = 0.0;
  for (int o = 0; o < 4; ++o) {
    sum += amp * value_noise(x * freq, y * freq, z * freq, seed + 101u * static_cast<uint32_t>(o));
    norm += amp;
    amp *= 0.5;
    freq *= 2.0;
  }
  return sum / norm;
}

// ------------------------------------------------------------ geodesic spheres
// Frequency-n geodesic subdivision of the icosahedron: 20 n^2 triangles, 10 n^2 + 2 vertices.
// Points on an icosahedron edge are computed once from the edge's two corners in canonical
// order, so neighbouring faces share vertices exactly (the mesh is closed).
void geodesic_sphere(int n, double amplitude, uint32_t noise_seed, std::vector<float>* vout,
                     std::vector<int32_t>* iout) {
  const double t = (1.0 + std::sqrt(5.0)) / 2.0;
  const double base[12][3] = {{-1, t, 0}, {1, t, 0}, {-1, -t, 0}, {1, -t, 0}, {0, -1, t}, {0, 1, t},
                              {0, -1, -t}, {0, 1, -t}, {t, 0, -1}, {t, 0, 1}, {-t, 0, -1}, {-t, 0, 1}};
  const int faces[20][3] = {{0, 11, 5}, {0, 5, 1}, {0, 1, 7}, {0, 7, 10}, {0, 10, 11}, {1, 5, 9}, {5, 11, 4},
                            {11, 10, 2}, {10, 7, 6}, {7, 1, 8}, {3, 9, 4}, {3, 4, 2}, {3, 2, 6}, {3, 6, 8},
                            {3, 8, 9}, {4, 9, 5}, {2, 4, 11}, {6, 2, 10}, {8, 6, 7}, {9, 8, 1}};
  std::vector<double> pos;  // unit-sphere positions, xyz
  auto push = [&](double x, double y, double z) {
    const double l = std::sqrt(x * x + y * y + z * z);
    pos.push_back(x / l); pos.push_back(y / l); pos.push_back(z / l);
    return static_cast<int32_t>(pos.size() / 3) - 1;
  };
  for (auto& b : base) push(b[0], b[1], b[2]);
  std::map<std::pair<int, int>, std::vector<int32_t>> edge_points;  // (lo, hi) -> points k=1..n-1 from lo
  auto edge_point = [&](int a, int b, int k_from_a) -> int32_t {
    const int lo = a < b ? a : b, hi = a < b ? b : a;
    const int k = a < b ? k_from_a : n - k_from_a;  // steps from lo
    auto it = edge_points.find({lo, hi});
    if (it == edge_points.end()) {
      std::vector<int32_t> ids(n + 1, -1);
      for (int s = 1; s < n; ++s) {
        const double w = static_cast<double>(s) / n;
        ids[s] = push(base[lo][0] * (1 - w) + base[hi][0] * w, base[lo][1] * (1 - w) + base[hi][1] * w,
                      base[lo][2] * (1 - w) + base[hi][2] * w);
      }
      it = edge_points.emplace(std::make_pair(lo, hi), std::move(ids)).first;
    }
    return it->second[k];
  };
  std::vector<int32_t>& idx = *iout;
  idx.clear();
  for (auto& f : faces) {
    const int A = f[0], B = f[1], C = f[2];
    // grid[i][j]: weight i toward B, j toward C
    std::vector<std::vector<int32_t>> grid(n + 1, std::vector<int32_t>(n + 1, -1));
    for (int i = 0; i <= n; ++i)
      for (int j = 0; i + j <= n; ++j) {
        const int wa = n - i - j;
        int32_t id;
        if (i == 0 && j == 0) id = A;
        else if (i == n) id = B;
        else if (j == n) id = C;
        else if (j == 0) id = edge_point(A, B, i);
        else if (i == 0) id = edge_point(A, C, j);
        else if (wa == 0) id = edge_point(B, C, j);
        else {
          const double a = static_cast<double>(wa) / n, b = static_cast<double>(i) / n, c = static_cast<double>(j) / n;
          id = push(base[A][0] * a + base[B][0] * b + base[C][0] * c, base[A][1] * a + base[B][1] * b + base[C][1] * c,
                    base[A][2] * a + base[B][2] * b + base[C][2] * c);
        }
        grid[i][j] = id;
      }
    for (int i = 0; i < n; ++i)
      for (int j = 0; i + j < n; ++j) {
        idx.push_back(grid[i][j]); idx.push_back(grid[i + 1][j]); idx.push_back(grid[i][j + 1]);
        if (i + j + 1 < n) {
          idx.push_back(grid[i + 1][j]); idx.push_back(grid[i + 1][j + 1]); idx.push_back(grid[i][j + 1]);
        }
      }
  }
  const size_t nv = pos.size() / 3;
  vout->resize(nv * 3);
  for (size_t v = 0; v < nv; ++v) {
    const double x = pos[3 * v], y = pos[3 * v + 1], z = pos[3 * v + 2];
    const double r = amplitude > 0 ? 1.0 + amplitude * fbm4(x, y, z, noise_seed) : 1.0;
    (*vout)[3 * v] = static_cast<float>(x * r);
    (*vout)[3 * v + 1] = static_cast<float>(y * r);
    (*vout)[3 * v + 2] = static_cast<float>(z * r);
  }
}

// axis-aligned quad from its 4 corners (two triangles 0-1-2, 0-2-3)
int add_quad(bn_scene_bundle* b, V3 a, V3 c1, V3 c2, V3 c3) {
  std::vector<float> v = {a.x, a.y, a.z, c1.x, c1.y, c1.z, c2.x, c2.y, c2.z, c3.x, c3.y, c3.z};
  return b->add_mesh(std::move(v), {0, 1, 2, 0, 2, 3});
}

// the unit cube of MeshPrimitive.Cube (Extensions/Primitive/Mesh.fs:136-155)
int add_unit_cube(bn_scene_bundle* b) {
  std::vector<float> v = {-1, -1, -1, 1, -1, -1, 1, 1, -1, -1, 1, -1, -1, -1, 1, 1, -1, 1, 1, 1, 1, -1, 1, 1};
  std::vector<int32_t> i = {0, 2, 1, 0, 3, 2, 4, 5, 6, 4, 6, 7, 0, 1, 5, 0, 5, 4,
                            3, 7, 6, 3, 6, 2, 0, 4, 7, 0, 7, 3, 1, 2, 6, 1, 6, 5};
  return b->add_mesh(std::move(v), std::move(i));
}

struct CornellIds {
  int white, red, green;
};

// The Cornell box in the unit cube: floor/ceiling/back white, left red, right green, two white
// boxes (0.3 and 0.6 tall, rotated -17 and +17 degrees about y), a 0.25 x 0.2 one-sided ceiling
// light of emission (17,12,4) just below the ceiling.  36 triangles.  light_quads > 1 splits the
// light into a 2x2 grid.
CornellIds build_cornell(bn_scene_bundle* b, int light_quads, std::vector<int>* light_instances) {
  CornellIds ids{};
  ids.white = b->add_material(BN_MAT_LAMBERTIAN, v3(0.73f, 0.73f, 0.73f));
  ids.red = b->add_material(BN_MAT_LAMBERTIAN, v3(0.65f, 0.05f, 0.05f));
  ids.green = b->add_material(BN_MAT_LAMBERTIAN, v3(0.12f, 0.45f, 0.15f));
  const M4 I = m4_identity();
  int p;
  p = add_quad(b, v3(0, 0, 0), v3(1, 0, 0), v3(1, 0, 1), v3(0, 0, 1));  // floor
  b->add_instance(p, ids.white, -1, I);
  p = add_quad(b, v3(0, 1, 0), v3(0, 1, 1), v3(1, 1, 1), v3(1, 1, 0));  // ceiling
  b->add_instance(p, ids.white, -1, I);
  p = add_quad(b, v3(0, 0, 0), v3(0, 1, 0), v3(1, 1, 0), v3(1, 0, 0));  // back
  b->add_instance(p, ids.white, -1, I);
  p = add_quad(b, v3(0, 0, 0), v3(0, 0, 1), v3(0, 1, 1), v3(0, 1, 0));  // left
  b->add_instance(p, ids.red, -1, I);
  p = add_quad(b, v3(1, 0, 0), v3(1, 1, 0), v3(1, 1, 1), v3(1, 0, 1));  // right
  b->add_instance(p, ids.green, -1, I);
  const int cube = add_unit_cube(b);
  b->add_instance(cube, ids.white, -1,
                  m4_mul(m4_mul(m4_scale(0.15f, 0.15f, 0.15f), rot_y_degrees(-17.0)), m4_translation(0.66f, 0.15f, 0.62f)));
  b->add_instance(cube, ids.white, -1,
                  m4_mul(m4_mul(m4_scale(0.15f, 0.30f, 0.15f), rot_y_degrees(17.0)), m4_translation(0.34f, 0.30f, 0.36f)));
  const float y = 0.998f, x0 = 0.375f, x1 = 0.625f, z0 = 0.4f, z1 = 0.6f;
  const int g = light_quads > 1 ? 2 : 1;
  for (int a = 0; a < g; ++a)
    for (int c = 0; c < g; ++c) {
      const float xa = x0 + (x1 - x0) * a / g, xb = x0 + (x1 - x0) * (a + 1) / g;
      const float za = z0 + (z1 - z0) * c / g, zb = z0 + (z1 - z0) * (c + 1) / g;
      const int q = add_quad(b, v3(xa, y, za), v3(xb, y, za), v3(xb, y, zb), v3(xa, y, zb));
      // one-sided: the quad's winding gives a -y normal, so it emits downward only
      const int l = b->add_light(v3(17.f, 12.f, 4.f), false);
      const int inst = b->add_instance(q, -1, l, I);
      if (light_instances) light_instances->push_back(inst);
    }
  return ids;
}

M4 cornell_camera() { return look_at(v3(0.5f, 0.5f, 2.4f), v3(0.5f, 0.5f, 0.f), v3(0, 1, 0)); }

// Cornell box + displaced PBR icosphere (level 6), dielectric icosphere (level 5), mirror quad
void add_cornell_objects(bn_scene_bundle* b, Rng& rng, int pbr_material_override) {
  std::vector<float> v;
  std::vector<int32_t> idx;
  geodesic_sphere(64, 0.05, 7u, &v, &idx);  // level 6: 81,920 triangles
  const int ico6 = b->add_mesh(std::move(v), std::move(idx));
  const float br = rng.uniformf(0.2f, 0.9f), bg = rng.uniformf(0.2f, 0.9f), bb = rng.uniformf(0.2f, 0.9f);
  const V3 bc = v3(br, bg, bb);
  const float metallic = rng.uniform() < 0.5 ? 0.f : 1.f;
  const float roughness = rng.uniformf(0.05f, 0.8f);
  int pbr = pbr_material_override >= 0 ? pbr_material_override
                                       : b->add_material(BN_MAT_PBR, bc, 1.5f, roughness, metallic);
  b->add_instance(ico6, pbr, -1, m4_mul(m4_scale(0.12f, 0.12f, 0.12f), m4_translation(0.66f, 0.42f, 0.62f)));
  std::vector<float> v5;
  std::vector<int32_t> i5;
  geodesic_sphere(32, 0.0, 0u, &v5, &i5);  // level 5: 20,480 triangles
  const int ico5 = b->add_mesh(std::move(v5), std::move(i5));
  int glass = pbr_material_override >= 0 ? pbr_material_override
                                         : b->add_material(BN_MAT_DIELECTRIC, v3(1, 1, 1), 1.5f);
  b->add_instance(ico5, glass, -1, m4_mul(m4_scale(0.12f, 0.12f, 0.12f), m4_translation(0.25f, 0.12f, 0.75f)));
  const int mq = add_quad(b, v3(0.55f, 0.35f, 0.002f), v3(0.9f, 0.35f, 0.002f), v3(0.9f, 0.75f, 0.002f),
                          v3(0.55f, 0.75f, 0.002f));
  int mirror = pbr_material_override >= 0 ? pbr_material_override
                                          : b->add_material(BN_MAT_MIRROR, v3(0.95f, 0.95f, 0.95f));
  b->add_instance(mq, mirror, -1, m4_identity());
}

bool gen_cornell(bn_scene_bundle* b, uint32_t) {
  build_cornell(b, 1, nullptr);
  b->light_sampler = BN_LIGHTS_UNIFORM;
  b->views.push_back(make_view(cornell_camera(), 40.f, 256, 256));
  b->render = default_render_desc();
  b->render.spp = 64;
  b->render.max_depth = 8;
  b->render.rr_depth = 5;
  return true;
}

bool gen_cornell_objects(bn_scene_bundle* b, uint32_t seed, int res, int spp) {
  Rng rng(seed);
  build_cornell(b, 1, nullptr);
  add_cornell_objects(b, rng, -1);
  b->light_sampler = BN_LIGHTS_ALIAS_TRIANGLES;
  b->views.push_back(make_view(cornell_camera(), 40.f, res, res));
  b->render = default_render_desc();
  b->render.spp = spp;
  b->render.max_depth = 16;
  b->render.rr_depth = 5;
  return true;
}

bool gen_pssmlt(bn_scene_bundle* b, uint32_t seed) {
  gen_cornell_objects(b, seed, 1024, 16);
  b->render.integrator = BN_INTEGRATOR_PSSMLT;
  b->render.spp = 16;  // mutations per pixel
  b->render.n_bootstrap = 1 << 20;
  b->render.n_chains = 65536;
  b->render.large_step_prob = 0.3f;
  b->render.mutation = BN_MUTATION_KELEMEN;
  b->render.eps_min = 1.f / 1024.f;
  b->render.eps_max = 1.f / 64.f;
  return true;
}

bool gen_instances(bn_scene_bundle* b, uint32_t seed) {
  Rng rng(seed);
  const int freqs[4] = {32, 64, 100, 128};  // 20,480 / 81,920 / 200,000 / 327,680 triangles
  int blas[4];
  for (int k = 0; k < 4; ++k) {
    std::vector<float> v;
    std::vector<int32_t> idx;
    geodesic_sphere(freqs[k], 0.05, 1000u + 17u * static_cast<uint32_t>(k) + seed, &v, &idx);
    blas[k] = b->add_mesh(std::move(v), std::move(idx));
  }
  const int ground_mat = b->add_material(BN_MAT_LAMBERTIAN, v3(0.5f, 0.5f, 0.5f));
  const int ground = add_quad(b, v3(-100, 0, -100), v3(-100, 0, 100), v3(100, 0, 100), v3(100, 0, -100));
  b->add_instance(ground, ground_mat, -1, m4_identity());
  for (int i = 0; i < 1024; ++i) {
    const int k = rng.below(4);
    const float s = rng.uniformf(0.5f, 2.0f);
    const M4 R = random_rotation(rng);
    const float x = rng.uniformf(-60.f, 60.f), z = rng.uniformf(-60.f, 60.f), y = s + rng.uniformf(0.f, 20.f);
    const int type = rng.below(4);
    int mat;
    const float cr = rng.uniformf(0.2f, 0.9f), cg = rng.uniformf(0.2f, 0.9f), cb = rng.uniformf(0.2f, 0.9f);
    const V3 c = v3(cr, cg, cb);
    if (type == BN_MAT_LAMBERTIAN) mat = b->add_material(BN_MAT_LAMBERTIAN, c);
    else if (type == BN_MAT_MIRROR) mat = b->add_material(BN_MAT_MIRROR, c);
    else if (type == BN_MAT_DIELECTRIC) mat = b->add_material(BN_MAT_DIELECTRIC, v3(1, 1, 1), 1.5f);
    else {
      const float roughness = rng.uniformf(0.05f, 0.8f);
      const float metallic = rng.uniform() < 0.5 ? 0.f : 1.f;
      mat = b->add_material(BN_MAT_PBR, c, 1.5f, roughness, metallic);
    }
    b->add_instance(blas[k], mat, -1, m4_mul(m4_mul(m4_scale(s, s, s), R), m4_translation(x, y, z)));
  }
  // 64 emissive triangles: one shared triangle mesh, 64 instances
  const int tri = b->add_mesh({-1.f, 0.f, -0.577f, 1.f, 0.f, -0.577f, 0.f, 0.f, 1.155f}, {0, 1, 2});
  for (int i = 0; i < 64; ++i) {
    const float e = rng.uniformf(5.f, 20.f);
    const int l = b->add_light(v3(e, e, e), true);
    const float s = rng.uniformf(2.f, 5.f);
    const float x = rng.uniformf(-70.f, 70.f), z = rng.uniformf(-70.f, 70.f), y = rng.uniformf(30.f, 45.f);
    b->add_instance(tri, -1, l, m4_mul(m4_mul(m4_scale(s, s, s), random_rotation(rng)), m4_translation(x, y, z)));
  }
  b->light_sampler = BN_LIGHTS_ALIAS_TRIANGLES;
  const int res[12][2] = {{256, 256}, {320, 240}, {512, 512}, {640, 360}, {640, 480}, {800, 600},
                          {1024, 576}, {1024, 768}, {1280, 720}, {1280, 1024}, {1600, 900}, {1920, 1080}};
  for (int v = 0; v < 16; ++v) {
    const int k = rng.below(12);
    double s, c;
    det_sincos(2.0 * 3.14159265358979323846 * (v + rng.uniform() * 0.5) / 16.0, &s, &c);
    const float rad = rng.uniformf(70.f, 95.f);
    const V3 eye = v3(static_cast<float>(c) * rad, rng.uniformf(12.f, 35.f), static_cast<float>(s) * rad);
    const float tx = rng.uniformf(-15.f, 15.f), ty = rng.uniformf(2.f, 10.f), tz = rng.uniformf(-15.f, 15.f);
    const V3 target = v3(tx, ty, tz);
    b->views.push_back(make_view(look_at(eye, target, v3(0, 1, 0)), rng.uniformf(35.f, 60.f), res[k][0], res[k][1]));
  }
  b->render = default_render_desc();
  b->render.spp = 64;
  b->render.max_depth = 12;
  b->render.rr_depth = 3;
  b->render.mode = BN_MODE_WAVEFRONT;
  return true;
}

bool gen_materials(bn_scene_bundle* b, uint32_t seed) {
  Rng rng(seed);
  std::vector<int> lights;
  // geometry of the cornell-objects scene, the ceiling light split into 4 emissive quads
  build_cornell(b, 4, &lights);
  Rng obj_rng(seed);
  add_cornell_objects(b, obj_rng, 0);
  const int n_slots = 32, n_emissive = 4, base_e = n_slots - n_emissive;
  // materials 0..31 are the slots (PBR); build_cornell created 3 lambertians first: replace
  b->materials.clear();
  b->slot_params.assign(static_cast<size_t>(n_slots) * 6, 0.f);
  for (int s = 0; s < n_slots; ++s) {
    float* p = &b->slot_params[static_cast<size_t>(s) * 6];
    p[0] = rng.uniformf(0.05f, 0.95f); p[1] = rng.uniformf(0.05f, 0.95f); p[2] = rng.uniformf(0.05f, 0.95f);
    p[3] = rng.uniformf(0.05f, 0.9f);
    p[4] = rng.uniformf(0.f, 1.f);
    p[5] = s >= base_e ? rng.uniformf(0.5f, 1.5f) : 1.f;
    b->add_material(BN_MAT_PBR, v3(p[0], p[1], p[2]), 1.5f, p[3], p[4]);
  }
  // per-triangle slot ids on every non-emissive mesh
  for (size_t i = 0; i < b->instances.size(); ++i) {
    bn_instance_desc& in = b->instances[i];
    if (in.light >= 0) continue;
    in.material = 0;
    const int mesh = b->primitives[in.primitive].mesh;
    if (mesh < 0 || !b->mesh_trimat[mesh].empty()) continue;
    const size_t nt = b->mesh_indices[mesh].size() / 3;
    std::vector<int32_t> tm(nt);
    for (size_t t = 0; t < nt; ++t) tm[t] = rng.below(base_e);
    b->mesh_trimat[mesh] = std::move(tm);
  }
  b->n_slots = n_slots;
  b->emissive_slot_base = base_e;
  b->light_sampler = BN_LIGHTS_ALIAS_TRIANGLES;
  b->views.push_back(make_view(cornell_camera(), 40.f, 256, 256));
  b->render = default_render_desc();
  b->render.spp = 16;
  b->render.max_depth = 8;
  b->render.rr_depth = 5;
  return true;
}

}  // namespace

bool generate_bundle(const std::string& name, uint32_t seed, bn_scene_bundle* b, std::string* err) {
  bool ok;
  if (name == "cornell") ok = gen_cornell(b, seed);
  else if (name == "cornell-objects") ok = gen_cornell_objects(b, seed, 512, 256);
  else if (name == "instances") ok = gen_instances(b, seed);
  else if (name == "pssmlt") ok = gen_pssmlt(b, seed);
  else if (name == "materials") ok = gen_materials(b, seed);
  else {
    *err = "unknown workload '" + name + "' (cornell, cornell-objects, instances, pssmlt, materials)";
    return false;
  }
  b->finalize();
  return ok;
}

}  // namespace bnh
