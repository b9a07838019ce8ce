// GPU-resident scene layout shared by the host flattener (scene.cpp) and the
// CUDA kernels.  Everything is plain-old-data in structure-of-arrays form.
//
// BVH: binary, exactly the tree the reference's SAH builder produces
// (clovers/src/bvh/build/surface_area_heuristic.rs), flattened depth-first.
// A node carries the boxes of BOTH children so one 64-byte fetch gives
// everything BVHNode::hit needs at that node (own box comes from the parent's
// record, or the scene root box).
//
// Child references (u32):
//   REF_EMPTY                 Hitable::Empty
//   kind << 29 | index        kind = REF_NODE, REF_TRI, REF_QUAD, REF_SPHERE or REF_OBJ
#pragma once
#include <stdint.h>

#define CLV_REF_EMPTY 0xFFFFFFFFu
#define CLV_REF_NODE 0u
#define CLV_REF_TRI 1u
#define CLV_REF_QUAD 2u
#define CLV_REF_SPHERE 3u
#define CLV_REF_OBJ 4u
#define CLV_REF_KIND(r) ((r) >> 29)
#define CLV_REF_INDEX(r) ((r) & 0x1FFFFFFFu)
#define CLV_MAKE_REF(kind, idx) (((uint32_t)(kind) << 29) | (uint32_t)(idx))

// Boxes: {xmin, xmax, ymin, ymax, zmin, zmax}
struct __attribute__((aligned(16))) ClvNode {
  float lbox[6];
  float rbox[6];
  uint32_t left, right;
  uint32_t pad0, pad1;
};

// Triangle and quad record: the fields of clovers/src/objects/triangle.rs:36-55
// (q, u, v, normal, d, w), 16 floats = 64 bytes:
//   f4[0] = q.x q.y q.z u.x | f4[1] = u.y u.z v.x v.y
//   f4[2] = v.z n.x n.y n.z | f4[3] = d   w.x w.y w.z
struct __attribute__((aligned(16))) ClvPlanar {
  float f[16];
};

// Complex objects (wrappers and compound shapes), evaluated by a small
// depth-bounded interpreter on the device.
enum ClvObjKind {
  CLV_OBJ_BOXY = 0,       // a: first of 6 consecutive quads
  CLV_OBJ_LIST = 1,       // a: first child slot in obj_children, b: count
  CLV_OBJ_TRANSLATE = 2,  // a: child ref, p[0..2] offset
  CLV_OBJ_ROTATEY = 3,    // a: child ref, p[0] sin, p[1] cos
  CLV_OBJ_MEDIUM = 4,     // a: boundary ref, b: material, p[0] -1/density
  CLV_OBJ_MOVING = 5,     // b: material, p[0..2] c0, p[3..5] c1, p[6] t0, p[7] t1, p[8] radius
};
struct __attribute__((aligned(16))) ClvObj {
  uint32_t kind, a, b, pad;
  float p[12];
};

// Materials (clovers/src/materials.rs:141-156) and textures (textures.rs:17-109).
enum ClvMatKind {
  CLV_MAT_DIELECTRIC = 0,
  CLV_MAT_DISPERSIVE = 1,
  CLV_MAT_LAMBERTIAN = 2,
  CLV_MAT_CONELIGHT = 3,
  CLV_MAT_DIFFUSELIGHT = 4,
  CLV_MAT_METAL = 5,
  CLV_MAT_ISOTROPIC = 6,
};
enum ClvTexKind { CLV_TEX_SOLID = 0, CLV_TEX_SPATIAL = 1, CLV_TEX_SURFACE = 2, CLV_TEX_ILLUMINANT = 3 };
struct __attribute__((aligned(16))) ClvMaterial {
  uint32_t kind;
  uint32_t tex_kind;
  uint32_t spd_even;    // SPD table index (SolidColor / checker even / Dielectric colour)
  uint32_t spd_odd;     // checker odd
  float density;        // checker density
  uint32_t illuminant;  // illuminant table index
  float intensity;
  float fuzz;
  float refractive_index;
  float cauchy_a, cauchy_b;
  uint32_t sellmeier;
  float sell_b[3];
  float sell_c[3];
  float spread;
  uint32_t thin_film;
  float tf_ior, tf_thickness;
  uint32_t wavelength_dependent;
  uint32_t pad[3];
};

// MIS ("priority") tree, clovers-cli/src/scenefile.rs:106-108: same binary
// tree shape as the main BVH but only pdf_value / random are evaluated.
struct ClvMisNode {
  uint32_t left, right;  // refs; REF_NODE indexes mis_nodes
};

struct ClvCamera {
  float llc[3], horizontal[3], vertical[3], origin[3], u[3], v[3], w[3];
  float lens_radius;
};

// Everything a kernel needs, passed by value.
struct ClvDeviceScene {
  const ClvNode* nodes;
  const ClvPlanar* tris;
  const ClvPlanar* quads;
  const float* spheres;  // 4 floats per sphere: center.xyz, radius
  const ClvObj* objs;
  const uint32_t* obj_children;
  const uint32_t* tri_gid;
  const uint32_t* quad_gid;
  const uint32_t* sphere_gid;
  const uint32_t* obj_gid;
  const uint32_t* tri_mat;
  const uint32_t* quad_mat;
  const uint32_t* sphere_mat;
  const float* tri_area;
  const float* quad_area;
  const ClvMaterial* materials;
  const float* spd;         // [n_spd][400]
  const float* illuminant;  // [n_illuminants][400]
  const float* cmf;         // [400][3] wavelength_into_xyz table
  const ClvMisNode* mis_nodes;
  uint32_t root;            // ref of the main BVH root (a node, or a single leaf)
  uint32_t mis_root;        // ref of the MIS root
  float root_box[6];
  uint32_t background_spd;
  uint32_t n_nodes, n_tris, n_quads, n_spheres, n_objs, n_materials;
  uint32_t max_depth_tree;  // depth of the main BVH (stack bound)
  uint32_t compound_level;  // 0 primitives only, 1 wrapper chains, 2 media / lists present
  uint32_t boxes_div_safe;  // every BVH box coordinate is 0 or of magnitude in [2^-70, 2^59]
  uint32_t mis_depth;
  uint32_t watertight;      // triangles use the watertight test (tri_verts set)
  const float* tri_verts;   // 12 per triangle: the vertices as given, xyz0 (watertight test only)
  ClvCamera camera;
};
