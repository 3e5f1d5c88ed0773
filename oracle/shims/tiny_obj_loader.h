// Oracle stand-in for the tinyobjloader types and ObjReader calls the
// reference uses (core/src/Scene.cpp:31-56,66-118,122-189,202-255,
// core/src/tinyobj.cpp:7-89), backed by the oracle's OBJ/MTL reader.
#pragma once
#include <string>
#include <vector>
#include "../port/hor_io.hpp"

namespace tinyobj {
typedef float real_t;
struct index_t { int vertex_index = -1, normal_index = -1, texcoord_index = -1; };
struct mesh_t {
  std::vector<index_t> indices;
  std::vector<unsigned char> num_face_vertices;
  std::vector<int> material_ids;
  std::vector<unsigned int> smoothing_group_ids;
};
struct shape_t { std::string name; mesh_t mesh; };
struct attrib_t { std::vector<real_t> vertices, normals, texcoords; };
struct material_t {
  std::string name;
  real_t ambient[3], diffuse[3], specular[3], transmittance[3], emission[3];
  real_t shininess, ior, dissolve, anisotropy;
  int illum;
  std::string diffuse_texname, specular_highlight_texname, bump_texname, metallic_texname;
};
struct ObjReaderConfig {
  bool triangulate = true;
  bool vertex_color = true;
  std::string mtl_search_path;
};
class ObjReader {
 public:
  bool ParseFromFile(const std::string& filename, const ObjReaderConfig& cfg) {
    hor::ObjData d;
    if (!hor::parse_obj(filename, cfg.mtl_search_path, d, error_)) return false;
    warning_ = d.warning;
    attrib_.vertices = d.vertices; attrib_.normals = d.normals; attrib_.texcoords = d.texcoords;
    for (const hor::ObjShape& s : d.shapes) {
      shape_t sh; sh.name = s.name;
      for (const hor::ObjIndex& ix : s.indices) { index_t t; t.vertex_index = ix.v; t.normal_index = ix.vn; t.texcoord_index = ix.vt; sh.mesh.indices.push_back(t); }
      sh.mesh.num_face_vertices = s.num_face_vertices;
      sh.mesh.material_ids = s.material_ids;
      sh.mesh.smoothing_group_ids = s.smoothing_group_ids;
      shapes_.push_back(sh);
    }
    for (const hor::ObjMaterial& m : d.materials) {
      material_t t; t.name = m.name;
      for (int c = 0; c < 3; ++c) {
        t.ambient[c] = m.ambient[c]; t.diffuse[c] = m.diffuse[c]; t.specular[c] = m.specular[c];
        t.transmittance[c] = m.transmittance[c]; t.emission[c] = m.emission[c];
      }
      t.shininess = m.shininess; t.ior = m.ior; t.dissolve = m.dissolve; t.anisotropy = m.anisotropy; t.illum = m.illum;
      t.diffuse_texname = m.diffuse_texname; t.specular_highlight_texname = m.specular_highlight_texname;
      t.bump_texname = m.bump_texname; t.metallic_texname = m.metallic_texname;
      materials_.push_back(t);
    }
    return true;
  }
  const attrib_t& GetAttrib() const { return attrib_; }
  const std::vector<shape_t>& GetShapes() const { return shapes_; }
  const std::vector<material_t>& GetMaterials() const { return materials_; }
  const std::string& Error() const { return error_; }
  const std::string& Warning() const { return warning_; }
 private:
  attrib_t attrib_;
  std::vector<shape_t> shapes_;
  std::vector<material_t> materials_;
  std::string error_, warning_;
};
}  // namespace tinyobj
