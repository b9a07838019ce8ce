// Host-side scene: the reference's scene JSON (clovers-cli/src/scenefile.rs)
// flattened into the structure-of-arrays layout of device_types.h.
#pragma once

#include <cstdint>
#include <string>
#include <vector>

#include "device_types.h"

namespace clv {

struct HostScene {
  std::vector<ClvNode> nodes;
  std::vector<ClvPlanar> tris, quads;
  std::vector<float> spheres;  // 4 floats each
  std::vector<ClvObj> objs;
  std::vector<uint32_t> obj_children;
  std::vector<uint32_t> tri_gid, quad_gid, sphere_gid, obj_gid;
  std::vector<uint32_t> tri_mat, quad_mat, sphere_mat;
  std::vector<float> tri_area, quad_area;
  std::vector<float> tri_verts;  // 12 per triangle: the three vertices as given (x, y, z, 0)
  std::vector<ClvMaterial> materials;
  std::vector<float> spd;  // 400 floats per table
  std::vector<ClvMisNode> mis_nodes;
  uint32_t root = CLV_REF_EMPTY, mis_root = CLV_REF_EMPTY;
  float root_box[6] = {0, 0, 0, 0, 0, 0};
  uint32_t background_spd = 0;
  float background_xyz[3] = {0, 0, 0};
  ClvCamera camera{};
  uint32_t width = 0, height = 0;
  uint32_t tree_depth = 0, mis_depth = 0;
  uint64_t object_count = 0;
  float time_0 = 0.0f, time_1 = 1.0f;
};

// Loads a clovers scene file (JSON).  width/height set the camera aspect ratio
// (clovers-cli/src/scenefile.rs:47-57).  Throws std::runtime_error.
// lam: the longest-axis-midpoint builder (BvhAlgorithm::Lam) for both trees instead of the SAH builder.
HostScene load_scene_json(const std::string& path, uint32_t width, uint32_t height, bool lam = false);
HostScene load_scene_text(const std::string& text, uint32_t width, uint32_t height, const std::string& base_dir,
                          bool lam = false);

// A scene made only of triangles given as a vertex buffer and u32 index
// triples (Triangle::from_coordinates, clovers/src/objects/triangle.rs:106-117),
// all with the default material; no camera or priority list.
HostScene mesh_scene(const float* verts, uint32_t nverts, const uint32_t* idx, uint32_t ntris);

}  // namespace clv
