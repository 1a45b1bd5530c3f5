// api_obj.cpp -- vct_load_model: Wavefront OBJ/MTL reader feeding
// vct_load_mesh, in place of the tinyobjloader call of Renderer::load_model
// (renderer.cpp:407-603).
//
// Follows the reference's use of the parsed data: polygons are triangulated
// as fans (LoadObj(..., triangulate=true), renderer.cpp:417); every
// (position, normal, uv) corner is deduplicated into one vertex
// (renderer.cpp:464-515); per shape, consecutive faces with the same material
// form one draw object (renderer.cpp:519-556); the file's materials are
// appended to the renderer's material list (renderer.cpp:423-430, fields of
// create_material :49-81) and a face without material uses the file's first
// material (DEFAULT_MATERIAL_INDEX + base, :527-528,537) -- or the renderer's
// default material 0 when the file has none.
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <map>
#include <sstream>
#include <string>
#include <unordered_map>
#include <vector>

#include "api_common.h"

using namespace vct;

namespace {

struct Key {
  int v, t, n;
  bool operator==(const Key& o) const { return v == o.v && t == o.t && n == o.n; }
};
struct KeyHash {
  size_t operator()(const Key& k) const {
    return ((size_t)(uint32_t)k.v * 73856093u) ^ ((size_t)(uint32_t)k.t * 19349663u) ^ ((size_t)(uint32_t)k.n * 83492791u);
  }
};

int fix_index(long i, size_t n) {  // OBJ: 1-based, negative = relative
  if (i > 0) return (int)(i - 1);
  if (i < 0) return (int)((long)n + i);
  return -1;
}

bool parse_corner(const std::string& tok, size_t nv, size_t nt, size_t nn, Key& k) {
  k.v = k.t = k.n = -1;
  const char* s = tok.c_str();
  char* end;
  long v = std::strtol(s, &end, 10);
  if (end == s) return false;
  k.v = fix_index(v, nv);
  if (*end == '/') {
    s = end + 1;
    if (*s != '/') {
      long t = std::strtol(s, &end, 10);
      if (end != s) k.t = fix_index(t, nt);
      s = end;
    }
    if (*s == '/') {
      s++;
      long n = std::strtol(s, &end, 10);
      if (end != s) k.n = fix_index(n, nn);
    }
  }
  return k.v >= 0 && (size_t)k.v < nv && k.t < (int)nt && k.n < (int)nn;
}

void load_mtl(const std::string& path, std::vector<vct_material_data>& mats, std::map<std::string, int>& names) {
  std::ifstream f(path);
  if (!f) {
    std::fprintf(stderr, "vct_load_model: cannot open material library %s\n", path.c_str());
    return;
  }
  std::string line;
  vct_material_data* m = nullptr;
  bool has_d = false;  // tinyobjloader: `d` wins over `Tr` in either order
  while (std::getline(f, line)) {
    std::istringstream ss(line);
    std::string tag;
    if (!(ss >> tag) || tag[0] == '#') continue;
    if (tag == "newmtl") {
      std::string name;
      ss >> name;
      vct_material_data d;
      std::memset(&d, 0, sizeof(d));
      // tinyobj defaults: dissolve 1, ior 1, shininess 1, transmittance 0.
      d.dissolve = 1.0f;
      d.ior = 1.0f;
      d.shininess = 1.0f;
      names[name] = (int)mats.size();
      mats.push_back(d);
      m = &mats.back();
      has_d = false;
      continue;
    }
    if (!m) continue;
    auto rd3 = [&](float* o) { ss >> o[0] >> o[1] >> o[2]; };
    if (tag == "Ka") rd3(m->ambient);
    else if (tag == "Kd") rd3(m->diffuse);
    else if (tag == "Ks") rd3(m->specular);
    else if (tag == "Kt" || tag == "Tf") rd3(m->transmittance);
    else if (tag == "Ke") rd3(m->emission);
    else if (tag == "Ns") ss >> m->shininess;
    else if (tag == "Ni") ss >> m->ior;
    else if (tag == "d") { ss >> m->dissolve; has_d = true; }
    else if (tag == "Tr") { float tr = 0.0f; ss >> tr; if (!has_d) m->dissolve = 1.0f - tr; }
    else if (tag == "illum") ss >> m->illum;
    else if (tag == "Pr") ss >> m->roughness;
    else if (tag == "Pm") ss >> m->metallic;
    else if (tag == "Ps") ss >> m->sheen;
    else if (tag == "Pc") ss >> m->clearcoat_thickness;
    else if (tag == "Pcr") ss >> m->clearcoat_roughness;
    else if (tag == "aniso") ss >> m->anisotropy;
    else if (tag == "anisor") ss >> m->anisotropy_rotation;
  }
}

}  // namespace

extern "C" vct_model_id vct_load_model(vct_renderer* r, const char* filename) {
  clear_error();
  if (!r || !filename) {
    set_error(VCT_ERR_INVALID_VALUE, "NULL argument");
    return VCT_INVALID_ID;
  }
  std::ifstream f(filename);
  if (!f) {
    std::fprintf(stderr, "Error loading file %s\n", filename);  // renderer.cpp:419
    set_error(VCT_ERR_IO, "cannot open %s", filename);
    return VCT_INVALID_ID;
  }
  const std::string fn = filename;
  const std::string basepath = fn.substr(0, fn.find_last_of("\\/") + 1);
  std::vector<float> P, T, Nn;
  std::vector<vct_material_data> mats;
  std::map<std::string, int> names;
  struct Face { Key c[3]; int mat; int shape; };
  std::vector<Face> faces;
  int cur_mat = -1, shape = 0;
  bool shape_has_faces = false;
  std::string line;
  while (std::getline(f, line)) {
    std::istringstream ss(line);
    std::string tag;
    if (!(ss >> tag) || tag[0] == '#') continue;
    if (tag == "v") { float x = 0, y = 0, z = 0; ss >> x >> y >> z; P.insert(P.end(), {x, y, z}); }
    else if (tag == "vn") { float x = 0, y = 0, z = 0; ss >> x >> y >> z; Nn.insert(Nn.end(), {x, y, z}); }
    else if (tag == "vt") { float u = 0, v = 0; ss >> u >> v; T.insert(T.end(), {u, v}); }
    else if (tag == "o" || tag == "g") {
      if (shape_has_faces) { ++shape; shape_has_faces = false; }
    } else if (tag == "mtllib") {
      std::string lib;
      while (ss >> lib) load_mtl(basepath + lib, mats, names);
    } else if (tag == "usemtl") {
      std::string name;
      ss >> name;
      auto it = names.find(name);
      cur_mat = it == names.end() ? -1 : it->second;
    } else if (tag == "f") {
      std::vector<Key> poly;
      std::string tok;
      while (ss >> tok) {
        Key k;
        if (!parse_corner(tok, P.size() / 3, T.size() / 2, Nn.size() / 3, k)) {
          set_error(VCT_ERR_IO, "%s: bad face corner '%s'", filename, tok.c_str());
          std::fprintf(stderr, "Error loading file %s\n", filename);
          return VCT_INVALID_ID;
        }
        poly.push_back(k);
      }
      for (size_t i = 1; i + 1 < poly.size(); ++i) faces.push_back({{poly[0], poly[i], poly[i + 1]}, cur_mat, shape});
      shape_has_faces = true;
    }
  }
  const uint32_t base = material_count(r);
  for (const auto& m : mats) vct_add_material(r, &m);
  std::vector<vct_vert_data> verts;
  std::vector<uint32_t> idx;
  std::unordered_map<Key, uint32_t, KeyHash> uniq;
  std::vector<vct_draw_obj> objs;
  for (size_t i = 0; i < faces.size(); ++i) {
    const Face& fc = faces[i];
    for (int k = 0; k < 3; ++k) {
      auto it = uniq.find(fc.c[k]);
      uint32_t vi;
      if (it == uniq.end()) {
        vct_vert_data v;
        std::memset(&v, 0, sizeof(v));
        std::memcpy(v.pos, &P[3 * fc.c[k].v], 12);
        if (fc.c[k].n >= 0) std::memcpy(v.norm, &Nn[3 * fc.c[k].n], 12);
        if (fc.c[k].t >= 0) std::memcpy(v.tex, &T[2 * fc.c[k].t], 8);
        vi = (uint32_t)verts.size();
        uniq.emplace(fc.c[k], vi);
        verts.push_back(v);
      } else {
        vi = it->second;
      }
      idx.push_back(vi);
    }
    const uint32_t mat = fc.mat >= 0 ? base + (uint32_t)fc.mat : (mats.empty() ? 0u : base);
    if (objs.empty() || objs.back().material_id != mat || i == 0 || faces[i - 1].shape != fc.shape)
      objs.push_back({(uint32_t)(3 * i), 0u, mat});
    objs.back().index_count += 3;
  }
  vct_model_id id = VCT_INVALID_ID;
  if (vct_load_mesh(r, verts.data(), (uint32_t)verts.size(), idx.data(), (uint32_t)idx.size(), objs.data(),
                    (uint32_t)objs.size(), &id) != VCT_OK)
    return VCT_INVALID_ID;
  return id;
}
