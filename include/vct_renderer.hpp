// vct_renderer.hpp -- C++ `Renderer` with the method names and signatures of
// src/renderer.h:122-196 and the Texture3D helpers of src/texture_3d.h:6-10,
// implemented over the C ABI of vct.h (header only; link libvct.so).
//
// glm::mat4 / glm::vec3 become vct::mat4 / vct::vec3 with the same memory
// layout (column-major float[16], float[3]); GLuint handles become uint32_t.
// Methods that return void in the reference keep returning void and report a
// failure through last_status() / vct_last_error(), so existing call sites
// compile unchanged.
#pragma once

#include <cstddef>
#include <cstring>

#include "vct.h"

namespace vct {

struct vec3 {
  float x, y, z;
};
struct mat4 {
  float m[16];  // column-major, as glm::mat4
  static mat4 identity() {
    mat4 r;
    std::memset(r.m, 0, sizeof(r.m));
    r.m[0] = r.m[5] = r.m[10] = r.m[15] = 1.0f;
    return r;
  }
};

typedef uint64_t model_id_t;     // renderer.h:23
typedef uint64_t shader_id_t;    // renderer.h:24
typedef uint64_t material_id_t;  // renderer.h:25
typedef vct_point_light point_light_t;
typedef vct_material_data material_data_t;
typedef vct_vert_data vert_data_t;

#ifndef INVALID_ID
#define INVALID_ID (~0)  // renderer.h:22
#endif

class Renderer {
 public:
  Renderer(int width, int height, const vct_config* cfg = nullptr) {
    status_ = vct_renderer_create(width, height, cfg, &r_);
  }
  ~Renderer() { vct_renderer_destroy(r_); }
  Renderer(const Renderer&) = delete;
  Renderer& operator=(const Renderer&) = delete;

  // Resource
  model_id_t load_model(const char* filename) { return vct_load_model(r_, filename); }
  model_id_t load_mesh(const vert_data_t* v, uint32_t nv, const uint32_t* idx, uint32_t ni, const vct_draw_obj* objs,
                       uint32_t no) {
    model_id_t id = VCT_INVALID_ID;
    status_ = vct_load_mesh(r_, v, nv, idx, ni, objs, no, &id);
    return id;
  }
  shader_id_t load_shader(const char* vertex_shader_name, const char* fragment_shader_name,
                          const char* geometry_shader_name = nullptr) {
    return vct_load_shader(r_, vertex_shader_name, fragment_shader_name, geometry_shader_name);
  }
  material_id_t add_material(material_data_t& material_data) { return vct_add_material(r_, &material_data); }
  void upload_material_data(material_data_t& material_data, material_id_t material_id) {
    status_ = vct_upload_material_data(r_, &material_data, material_id);
  }
  void set_model_material(material_id_t material_id, model_id_t model_id) {
    status_ = vct_set_model_material(r_, material_id, model_id);
  }
  vec3 get_model_dimensions(model_id_t model) {
    vec3 d = {0, 0, 0};
    status_ = vct_get_model_dimensions(r_, model, &d.x);
    return d;
  }
  void set_grid_resolution(unsigned int res) { status_ = vct_set_grid_resolution(r_, res); }
  void set_grid_size(float size) { status_ = vct_set_grid_size(r_, size); }
  void set_camera_transform(mat4& lookat, mat4& projection) {
    status_ = vct_set_camera_transform(r_, lookat.m, projection.m);
  }
  void set_model_transform(model_id_t model_id, mat4 model_matrix) {
    status_ = vct_set_model_transform(r_, model_id, model_matrix.m);
  }
  // The reference returns material_t& (its UBO handle); the data is returned here.
  material_data_t get_material(material_id_t material_id) {
    material_data_t m;
    std::memset(&m, 0, sizeof(m));
    status_ = vct_get_material(r_, material_id, &m);
    return m;
  }

  // Render
  void set_rendering_phases(bool direct, bool diffuse, bool specular, bool shadow) {
    status_ = vct_set_rendering_phases(r_, direct, diffuse, specular, shadow);
  }
  void set_voxel_view_dir(int dir, float lod) { status_ = vct_set_voxel_view_dir(r_, dir, lod); }
  void queue_model(model_id_t model_id) { status_ = vct_queue_model(r_, model_id); }
  void queue_point_light(point_light_t& point_light) { status_ = vct_queue_point_light(r_, &point_light); }
  void render() { status_ = vct_render(r_); }

  // Engine additions: deferred light injection, synchronisation, read-back, status.
  void set_light_injection(bool enable) { status_ = vct_set_light_injection(r_, enable ? 1 : 0); }
  vct_status read_frame(void* rgba8) { return status_ = vct_read_frame(r_, rgba8, VCT_FRAME_RGBA8); }
  vct_status synchronize() { return status_ = vct_synchronize(r_); }
  vct_status last_status() const { return status_; }
  vct_renderer* handle() { return r_; }

 private:
  vct_renderer* r_ = nullptr;
  vct_status status_ = VCT_OK;
};

// Many independent scenes per frame (vct_batch_*; no reference counterpart).
class Batch {
 public:
  Batch(const vct_batch_scene* scenes, uint32_t n, const vct_batch_config* cfg = nullptr) {
    status_ = vct_batch_create(scenes, n, cfg, &b_);
  }
  ~Batch() { vct_batch_destroy(b_); }
  Batch(const Batch&) = delete;
  Batch& operator=(const Batch&) = delete;

  void set_camera(uint32_t scene, mat4& lookat, mat4& projection) {
    status_ = vct_batch_set_camera(b_, scene, lookat.m, projection.m);
  }
  void render() { status_ = vct_batch_render(b_); }
  vct_status synchronize() { return status_ = vct_batch_synchronize(b_); }
  vct_status read_frame(uint32_t scene, void* rgba8) { return status_ = vct_batch_read_frame(b_, scene, rgba8); }
  vct_status autotune(int frames, vct_batch_shape* best = nullptr) {
    return status_ = vct_batch_autotune(b_, frames, best, nullptr, nullptr);
  }
  vct_status last_status() const { return status_; }
  vct_batch* handle() { return b_; }

 private:
  vct_batch* b_ = nullptr;
  vct_status status_ = VCT_OK;
};

// Texture3D, texture_3d.h:6-10.
inline uint32_t create_tex_3d(int width, int height, int depth, int levels) {
  return vct_create_tex_3d(width, height, depth, levels);
}
inline void destroy_tex_3d(uint32_t tex) { vct_destroy_tex_3d(tex); }
inline void activate_tex_3d(uint32_t program, uint32_t tex, uint32_t unit) { vct_activate_tex_3d(program, tex, unit); }
inline void clear_tex_3d(uint32_t tex, float clear_color[4]) { vct_clear_tex_3d(tex, clear_color); }
inline void mip_tex_3d(uint32_t tex) { vct_mip_tex_3d(tex); }

}  // namespace vct
