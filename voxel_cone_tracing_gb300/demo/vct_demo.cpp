// vct_demo.cpp -- headless stand-in for the reference's application
// (src/main.cpp): the same scene, camera, light and per-frame calls on the
// engine's `vct::Renderer`, with every frame written to a binary PPM instead
// of swapped to a GLFW window.
//
//   vct_demo [--assets DIR] [--out PREFIX] [--frames N] [--width W]
//            [--height H] [--grid N] [--rotate RAD] [--sampler hw|exact]
//            [--dump-matrices FILE]
//
// --sampler selects the texture unit (default) or FP32 software filtering;
// --dump-matrices writes, per frame, the view, projection and the object's
// model matrix the frame used (48 floats, column-major, text) so that a
// checker can rebuild the same frame.
//
// Scene (main.cpp:85-118): assets/CornellBox-Glossy.obj at the identity, and
// assets/suzanne.obj at (0, 1.1, -0.5), scale 0.3, with the glossy
// transmissive material of main.cpp:88-97; grid size 3; camera at
// (0, 0.9, 3), pitch 0, yaw -90 degrees, glm::perspective(45, aspect, 0.1,
// 100) -- 45 is taken as radians, as glm does; one ceiling light at
// (0, 1.4, 0).  Without --assets (or when the files are missing) a built-in
// box of the same extent with red / green side walls and an icosphere in
// place of suzanne are used.  Each frame turns the object by --rotate
// radians about +y (the keyboard rotation of main.cpp), and the voxel debug
// view is off (set_voxel_view_dir(7, lod), main.cpp:300).
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

#include "vct_renderer.hpp"

namespace {

using vct::mat4;

struct V3 {
  float x, y, z;
};
V3 sub(V3 a, V3 b) { return {a.x - b.x, a.y - b.y, a.z - b.z}; }
V3 add(V3 a, V3 b) { return {a.x + b.x, a.y + b.y, a.z + b.z}; }
V3 scl(V3 a, float s) { return {a.x * s, a.y * s, a.z * s}; }
float dot(V3 a, V3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
V3 cross(V3 a, V3 b) { return {a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x}; }
V3 normalize(V3 a) { return scl(a, 1.0f / std::sqrt(dot(a, a))); }

mat4 mul(const mat4& a, const mat4& b) {  // column-major a * b
  mat4 r;
  for (int c = 0; c < 4; ++c)
    for (int k = 0; k < 4; ++k) {
      float s = 0.0f;
      for (int j = 0; j < 4; ++j) s += a.m[j * 4 + k] * b.m[c * 4 + j];
      r.m[c * 4 + k] = s;
    }
  return r;
}

// glm::lookAt (right-handed).
mat4 look_at(V3 eye, V3 center, V3 up) {
  const V3 f = normalize(sub(center, eye));
  const V3 s = normalize(cross(f, up));
  const V3 u = cross(s, f);
  mat4 m = mat4::identity();
  m.m[0] = s.x; m.m[4] = s.y; m.m[8] = s.z;
  m.m[1] = u.x; m.m[5] = u.y; m.m[9] = u.z;
  m.m[2] = -f.x; m.m[6] = -f.y; m.m[10] = -f.z;
  m.m[12] = -dot(s, eye); m.m[13] = -dot(u, eye); m.m[14] = dot(f, eye);
  return m;
}

// glm::perspective (right-handed, clip z in [-1, 1]); fovy in radians.
mat4 perspective(float fovy, float aspect, float n, float f) {
  const float t = std::tan(fovy / 2.0f);
  mat4 m;
  std::memset(m.m, 0, sizeof(m.m));
  m.m[0] = 1.0f / (aspect * t);
  m.m[5] = 1.0f / t;
  m.m[10] = -(f + n) / (f - n);
  m.m[11] = -1.0f;
  m.m[14] = -(2.0f * f * n) / (f - n);
  return m;
}

mat4 translate(V3 t) {
  mat4 m = mat4::identity();
  m.m[12] = t.x; m.m[13] = t.y; m.m[14] = t.z;
  return m;
}
mat4 rotate_y(float a) {
  mat4 m = mat4::identity();
  m.m[0] = std::cos(a); m.m[8] = std::sin(a);
  m.m[2] = -std::sin(a); m.m[10] = std::cos(a);
  return m;
}
mat4 scale(float s) {
  mat4 m = mat4::identity();
  m.m[0] = m.m[5] = m.m[10] = s;
  return m;
}

bool file_exists(const std::string& p) {
  FILE* f = std::fopen(p.c_str(), "rb");
  if (f) std::fclose(f);
  return f != nullptr;
}

vct::material_data_t diffuse_material(float r, float g, float b) {
  vct::material_data_t m;
  std::memset(&m, 0, sizeof(m));
  m.ambient[0] = m.ambient[1] = m.ambient[2] = m.ambient[3] = 1.0f;
  m.diffuse[0] = r; m.diffuse[1] = g; m.diffuse[2] = b; m.diffuse[3] = 1.0f;
  m.shininess = 10.0f;
  m.ior = 1.0f;
  m.dissolve = 1.0f;
  m.illum = 2;
  return m;
}

// Built-in stand-in for CornellBox-Glossy.obj: floor, ceiling and back wall
// (white), left wall (red), right wall (green), x in [-1, 1], y in [0, 2],
// z in [-1, 1], normals facing the inside.
vct::model_id_t builtin_box(vct::Renderer& r) {
  const vct::material_id_t white = [&] { auto m = diffuse_material(0.73f, 0.73f, 0.73f); return r.add_material(m); }();
  const vct::material_id_t red = [&] { auto m = diffuse_material(0.63f, 0.06f, 0.04f); return r.add_material(m); }();
  const vct::material_id_t green = [&] { auto m = diffuse_material(0.15f, 0.48f, 0.09f); return r.add_material(m); }();
  struct Quad {
    V3 a, b, c, d, n;
    vct::material_id_t mat;
  };
  const Quad quads[5] = {
      {{-1, 0, -1}, {1, 0, -1}, {1, 0, 1}, {-1, 0, 1}, {0, 1, 0}, white},     // floor
      {{-1, 2, -1}, {-1, 2, 1}, {1, 2, 1}, {1, 2, -1}, {0, -1, 0}, white},    // ceiling
      {{-1, 0, -1}, {-1, 2, -1}, {1, 2, -1}, {1, 0, -1}, {0, 0, 1}, white},   // back
      {{-1, 0, -1}, {-1, 0, 1}, {-1, 2, 1}, {-1, 2, -1}, {1, 0, 0}, red},     // left
      {{1, 0, -1}, {1, 2, -1}, {1, 2, 1}, {1, 0, 1}, {-1, 0, 0}, green},      // right
  };
  std::vector<vct::vert_data_t> v;
  std::vector<uint32_t> idx;
  std::vector<vct_draw_obj> objs;
  for (const Quad& q : quads) {
    const uint32_t base = (uint32_t)v.size();
    for (V3 p : {q.a, q.b, q.c, q.d}) {
      vct::vert_data_t vd;
      std::memset(&vd, 0, sizeof(vd));
      vd.pos[0] = p.x; vd.pos[1] = p.y; vd.pos[2] = p.z;
      vd.norm[0] = q.n.x; vd.norm[1] = q.n.y; vd.norm[2] = q.n.z;
      v.push_back(vd);
    }
    vct_draw_obj o;
    o.first_index = (uint32_t)idx.size();
    o.index_count = 6;
    o.material_id = (uint32_t)q.mat;
    objs.push_back(o);
    for (uint32_t k : {0u, 1u, 2u, 0u, 2u, 3u}) idx.push_back(base + k);
  }
  return r.load_mesh(v.data(), (uint32_t)v.size(), idx.data(), (uint32_t)idx.size(), objs.data(),
                     (uint32_t)objs.size());
}

// Built-in stand-in for suzanne.obj: a unit icosphere (3 subdivisions).
vct::model_id_t builtin_object(vct::Renderer& r) {
  const float t = (1.0f + std::sqrt(5.0f)) / 2.0f;
  std::vector<V3> p = {{-1, t, 0}, {1, t, 0}, {-1, -t, 0}, {1, -t, 0}, {0, -1, t}, {0, 1, t},
                       {0, -1, -t}, {0, 1, -t}, {t, 0, -1}, {t, 0, 1}, {-t, 0, -1}, {-t, 0, 1}};
  std::vector<uint32_t> f = {0, 11, 5, 0, 5, 1, 0, 1, 7, 0, 7, 10, 0, 10, 11, 1, 5, 9, 5, 11, 4, 11, 10, 2, 10, 7, 6,
                             7, 1, 8, 3, 9, 4, 3, 4, 2, 3, 2, 6, 3, 6, 8, 3, 8, 9, 4, 9, 5, 2, 4, 11, 6, 2, 10, 8,
                             6, 7, 9, 8, 1};
  for (V3& q : p) q = normalize(q);
  for (int s = 0; s < 3; ++s) {
    std::vector<uint32_t> g;
    for (size_t i = 0; i < f.size(); i += 3) {
      const uint32_t a = f[i], b = f[i + 1], c = f[i + 2];
      const uint32_t ab = (uint32_t)p.size(), bc = ab + 1, ca = ab + 2;
      p.push_back(normalize(add(p[a], p[b])));
      p.push_back(normalize(add(p[b], p[c])));
      p.push_back(normalize(add(p[c], p[a])));
      for (uint32_t k : {a, ab, ca, b, bc, ab, c, ca, bc, ab, bc, ca}) g.push_back(k);
    }
    f.swap(g);
  }
  std::vector<vct::vert_data_t> v(p.size());
  for (size_t i = 0; i < p.size(); ++i) {
    std::memset(&v[i], 0, sizeof(v[i]));
    v[i].pos[0] = v[i].norm[0] = p[i].x;
    v[i].pos[1] = v[i].norm[1] = p[i].y;
    v[i].pos[2] = v[i].norm[2] = p[i].z;
  }
  vct_draw_obj o;
  o.first_index = 0;
  o.index_count = (uint32_t)f.size();
  o.material_id = 0;
  return r.load_mesh(v.data(), (uint32_t)v.size(), f.data(), (uint32_t)f.size(), &o, 1);
}

bool write_ppm(const std::string& path, const std::vector<uint8_t>& rgba, int w, int h) {
  FILE* fp = std::fopen(path.c_str(), "wb");
  if (!fp) return false;
  std::fprintf(fp, "P6\n%d %d\n255\n", w, h);
  std::vector<uint8_t> row((size_t)w * 3);
  for (int y = h - 1; y >= 0; --y) {  // row 0 of the frame is the bottom
    for (int x = 0; x < w; ++x)
      for (int c = 0; c < 3; ++c) row[(size_t)x * 3 + c] = rgba[((size_t)y * w + x) * 4 + c];
    std::fwrite(row.data(), 1, row.size(), fp);
  }
  return std::fclose(fp) == 0;
}

}  // namespace

int main(int argc, char** argv) {
  std::string assets, out = "vct_frame";
  int frames = 1, width = 800, height = 600, grid = 128;  // main.cpp:28-29; renderer.cpp:146
  float rot_step = 0.05f;
  int sampler = VCT_SAMPLER_HW;
  std::string dump;
  for (int i = 1; i < argc; ++i) {
    const std::string a = argv[i];
    auto next = [&]() -> const char* {
      if (i + 1 >= argc) { std::fprintf(stderr, "%s needs a value\n", a.c_str()); std::exit(2); }
      return argv[++i];
    };
    if (a == "--assets") assets = next();
    else if (a == "--out") out = next();
    else if (a == "--frames") frames = std::atoi(next());
    else if (a == "--width") width = std::atoi(next());
    else if (a == "--height") height = std::atoi(next());
    else if (a == "--grid") grid = std::atoi(next());
    else if (a == "--rotate") rot_step = (float)std::atof(next());
    else if (a == "--dump-matrices") dump = next();
    else if (a == "--sampler") {
      const std::string v = next();
      if (v == "hw") sampler = VCT_SAMPLER_HW;
      else if (v == "exact") sampler = VCT_SAMPLER_EXACT;
      else { std::fprintf(stderr, "--sampler takes hw or exact\n"); return 2; }
    }
    else { std::fprintf(stderr, "unknown argument %s\n", a.c_str()); return 2; }
  }

  vct_config cfg;
  vct_config_default(&cfg);
  cfg.grid_res = grid;
  cfg.sampler = sampler;
  vct::Renderer renderer(width, height, &cfg);
  if (renderer.last_status() != VCT_OK) {
    std::fprintf(stderr, "vct_demo: %s\n", vct_last_error());
    return 1;
  }

  const std::string box_path = assets + "/CornellBox-Glossy.obj", obj_path = assets + "/suzanne.obj";
  const bool have_assets = !assets.empty() && file_exists(box_path) && file_exists(obj_path);
  const vct::model_id_t box = have_assets ? renderer.load_model(box_path.c_str()) : builtin_box(renderer);
  const vct::model_id_t dynamic_object =
      have_assets ? renderer.load_model(obj_path.c_str()) : builtin_object(renderer);
  if (box == (vct::model_id_t)VCT_INVALID_ID || dynamic_object == (vct::model_id_t)VCT_INVALID_ID) {
    std::fprintf(stderr, "vct_demo: scene load failed: %s\n", vct_last_error());
    return 1;
  }

  vct::material_data_t dm;  // main.cpp:88-97
  std::memset(&dm, 0, sizeof(dm));
  for (int k = 0; k < 4; ++k) {
    dm.ambient[k] = 1.0f;
    dm.diffuse[k] = 0.0f;
    dm.specular[k] = 1.0f;
    dm.transmittance[k] = 1.0f;
  }
  dm.emission[0] = 0.0f; dm.emission[1] = 0.0f; dm.emission[2] = 0.25f;
  dm.shininess = 1000.0f;
  dm.ior = 5.0f;
  dm.dissolve = 0.1f;
  dm.illum = 4;
  const vct::material_id_t dm_id = renderer.add_material(dm);
  renderer.set_model_material(dm_id, dynamic_object);
  const V3 dynamic_object_position = {0.0f, 1.1f, -0.5f};
  const float dynamic_object_scale = 0.3f;
  float dynamic_object_rot = 0.0f;

  renderer.set_grid_size(3.0f);
  // Camera(glm::vec3(0, .9, 3), 0, -90): front = (cos(-90 deg), 0, sin(-90 deg)).
  const V3 eye = {0.0f, 0.9f, 3.0f};
  const float yaw = -90.0f * 3.14159265358979f / 180.0f;
  const V3 front = normalize(V3{std::cos(yaw), 0.0f, std::sin(yaw)});
  mat4 view = look_at(eye, add(eye, front), V3{0.0f, 1.0f, 0.0f});
  mat4 proj = perspective(45.0f, (float)width / (float)height, 0.1f, 100.0f);
  renderer.set_camera_transform(view, proj);

  vct::point_light_t ceiling_light;  // main.cpp:115-118
  ceiling_light.position[0] = 0.0f; ceiling_light.position[1] = 1.4f; ceiling_light.position[2] = 0.0f;
  ceiling_light.color[0] = ceiling_light.color[1] = ceiling_light.color[2] = 1.0f;
  ceiling_light.intensity = 1.0f;

  FILE* dump_fp = nullptr;
  if (!dump.empty() && !(dump_fp = std::fopen(dump.c_str(), "w"))) {
    std::fprintf(stderr, "vct_demo: cannot write %s\n", dump.c_str());
    return 1;
  }
  std::vector<uint8_t> rgba((size_t)width * height * 4);
  for (int f = 0; f < frames; ++f) {
    renderer.set_voxel_view_dir(7, 0.0f);
    const mat4 m = mul(mul(translate(dynamic_object_position), rotate_y(dynamic_object_rot)),
                       scale(dynamic_object_scale));  // main.cpp:369-372
    renderer.set_model_transform(dynamic_object, m);
    if (dump_fp) {
      for (const mat4* q : {(const mat4*)&view, (const mat4*)&proj, &m})
        for (int k = 0; k < 16; ++k) std::fprintf(dump_fp, "%.9g%c", q->m[k], k == 15 ? '\n' : ' ');
    }
    renderer.set_model_transform(box, mat4::identity());
    renderer.queue_model(box);
    renderer.queue_model(dynamic_object);
    renderer.queue_point_light(ceiling_light);
    renderer.render();
    if (renderer.read_frame(rgba.data()) != VCT_OK) {
      std::fprintf(stderr, "vct_demo: frame %d: %s\n", f, vct_last_error());
      return 1;
    }
    vct_stage_times t;
    vct_get_stage_times(renderer.handle(), &t);
    char name[64];
    std::snprintf(name, sizeof(name), "_%04d.ppm", f);
    if (!write_ppm(out + name, rgba, width, height)) {
      std::fprintf(stderr, "vct_demo: cannot write %s%s\n", out.c_str(), name);
      return 1;
    }
    std::printf("frame %d: voxelize %.3f ms, mipmap %.3f ms, gbuffer %.3f ms, trace %.3f ms -> %s%s\n", f,
                t.voxelize, t.mipmap, t.gbuffer, t.trace, out.c_str(), name);
    dynamic_object_rot += rot_step;
  }
  if (dump_fp && std::fclose(dump_fp) != 0) {
    std::fprintf(stderr, "vct_demo: cannot write %s\n", dump.c_str());
    return 1;
  }
  return 0;
}
