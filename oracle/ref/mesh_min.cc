// mesh_min.cc -- TEST INFRASTRUCTURE ONLY.
//
// The ugu::Mesh members the rasterizer's translation units call (construct,
// destroy, read and set the SoA arrays).  The reference's own src/mesh.cc
// cannot be compiled here (it needs nlohmann/json, tinyobjloader and Eigen's
// sparse module, all absent), so these trivial accessors are written out for
// the class declared in include/ugu/mesh.h.  Normals are supplied by the
// caller, computed by the restatement of Mesh::CalcNormal in the oracle.
#include "ugu/mesh.h"

namespace ugu {

Mesh::Mesh() {}
Mesh::~Mesh() {}
Mesh::Mesh(const Mesh& src) = default;

const std::vector<Eigen::Vector3f>& Mesh::vertices() const { return vertices_; }
const std::vector<Eigen::Vector3f>& Mesh::vertex_colors() const { return vertex_colors_; }
const std::vector<Eigen::Vector3i>& Mesh::vertex_indices() const { return vertex_indices_; }
const std::vector<Eigen::Vector3f>& Mesh::normals() const { return normals_; }
const std::vector<Eigen::Vector3f>& Mesh::face_normals() const { return face_normals_; }
const std::vector<Eigen::Vector3i>& Mesh::normal_indices() const { return normal_indices_; }
const std::vector<Eigen::Vector2f>& Mesh::uv() const { return uv_; }
const std::vector<Eigen::Vector3i>& Mesh::uv_indices() const { return uv_indices_; }
const std::vector<int>& Mesh::material_ids() const { return material_ids_; }
const std::vector<ObjMaterial>& Mesh::materials() const { return materials_; }

bool Mesh::set_vertices(const std::vector<Eigen::Vector3f>& v) { vertices_ = v; return true; }
bool Mesh::set_vertex_colors(const std::vector<Eigen::Vector3f>& v) { vertex_colors_ = v; return true; }
bool Mesh::set_vertex_indices(const std::vector<Eigen::Vector3i>& v) { vertex_indices_ = v; return true; }
bool Mesh::set_normals(const std::vector<Eigen::Vector3f>& v) { normals_ = v; return true; }
bool Mesh::set_face_normals(const std::vector<Eigen::Vector3f>& v) { face_normals_ = v; return true; }
bool Mesh::set_normal_indices(const std::vector<Eigen::Vector3i>& v) { normal_indices_ = v; return true; }
bool Mesh::set_uv(const std::vector<Eigen::Vector2f>& v) { uv_ = v; return true; }
bool Mesh::set_uv_indices(const std::vector<Eigen::Vector3i>& v) { uv_indices_ = v; return true; }
bool Mesh::set_material_ids(const std::vector<int>& v) { material_ids_ = v; return true; }
bool Mesh::set_materials(const std::vector<ObjMaterial>& v) { materials_ = v; return true; }

}  // namespace ugu
