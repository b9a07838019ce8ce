// Scene flattening for the GB300 renderer: JSON -> SoA device arrays, plus the
// binary SAH build of clovers/src/bvh/build/surface_area_heuristic.rs.
//
// All f32 arithmetic that decides geometry (triangle/quad precomputation,
// boxes, centroids, SAH costs) follows the reference's operation order, so the
// tree and the primitive records are bit-identical to what the reference
// builds.  Compile with -ffp-contract=off.

#include "scene.hpp"

#include <algorithm>
#include <cctype>
#include <cmath>
#include <cstring>
#include <fstream>
#include <memory>
#include <sstream>
#include <stdexcept>

#include "json.hpp"
#include "spectral.hpp"

namespace clv {
namespace {

struct V3 {
  float x = 0, y = 0, z = 0;
  V3() {}
  V3(float a, float b, float c) : x(a), y(b), z(c) {}
  float operator[](int i) const { return i == 0 ? x : (i == 1 ? y : z); }
};
inline V3 operator+(V3 a, V3 b) { return V3(a.x + b.x, a.y + b.y, a.z + b.z); }
inline V3 operator-(V3 a, V3 b) { return V3(a.x - b.x, a.y - b.y, a.z - b.z); }
inline V3 operator-(V3 a) { return V3(-a.x, -a.y, -a.z); }
inline V3 operator*(float s, V3 a) { return V3(s * a.x, s * a.y, s * a.z); }
inline V3 operator/(V3 a, float s) { return V3(a.x / s, a.y / s, a.z / s); }
inline float dot(V3 a, V3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
inline V3 cross(V3 a, V3 b) { return V3(a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x); }
inline float length(V3 a) { return std::sqrt(dot(a, a)); }
inline V3 unit(V3 a) { return a / length(a); }

const float kPi = 3.14159265358979323846f;
const float kDegToRad = 3.14159265358979323846f / 180.0f;  // f32::to_radians
const float kRectEps = 0.0001f;                            // EPSILON_RECT_THICKNESS

// ---- boxes {xmin,xmax,ymin,ymax,zmin,zmax}; Interval::new orders its ends
struct Box {
  float b[6] = {0, 0, 0, 0, 0, 0};  // AABB::default() is the zero box
};
inline Box box_from(V3 a, V3 c) {
  Box r;
  for (int k = 0; k < 3; ++k) {
    r.b[2 * k] = std::fmin(a[k], c[k]);
    r.b[2 * k + 1] = std::fmax(a[k], c[k]);
  }
  return r;
}
inline void box_grow(Box& a, const Box& o) {
  for (int k = 0; k < 3; ++k) {
    a.b[2 * k] = std::fmin(a.b[2 * k], o.b[2 * k]);
    a.b[2 * k + 1] = std::fmax(a.b[2 * k + 1], o.b[2 * k + 1]);
  }
}
inline float box_area(const Box& a) {  // aabb.rs:159-163
  const float ex = a.b[1] - a.b[0], ey = a.b[3] - a.b[2], ez = a.b[5] - a.b[4];
  return 2.0f * (ex * ey + ey * ez + ex * ez);
}
inline V3 box_center(const Box& a) {  // Interval::center = min + 0.5*size
  return V3(a.b[0] + 0.5f * (a.b[1] - a.b[0]), a.b[2] + 0.5f * (a.b[3] - a.b[2]), a.b[4] + 0.5f * (a.b[5] - a.b[4]));
}
inline void box_pad(Box& a) {  // aabb.rs:99-119
  for (int k = 0; k < 3; ++k) {
    float lo = a.b[2 * k], hi = a.b[2 * k + 1];
    if (!(hi - lo >= kRectEps)) {
      float nlo = lo - kRectEps, nhi = hi + kRectEps;
      a.b[2 * k] = std::fmin(nlo, nhi);
      a.b[2 * k + 1] = std::fmax(nlo, nhi);
    }
  }
}

// ---- BVH builds over items with a box and a centroid.
struct Item {
  Box box;
  V3 c;
};
// child codes: >= 0 node index, kEmpty, or item i as -(i + 2)
const int64_t kEmpty = -1;
struct Built {
  int64_t left = kEmpty, right = kEmpty;
  Box box;
};
struct BuildResult {
  std::vector<Built> nodes;
  uint32_t depth = 0;
};

BuildResult sah_build(const std::vector<Item>& items) {
  BuildResult out;
  const size_t n = items.size();
  if (n == 0) throw std::runtime_error("BVH build over an empty list (the reference's builder panics)");
  std::vector<uint32_t> ids(n), tmp;
  for (size_t i = 0; i < n; ++i) ids[i] = (uint32_t)i;
  struct Task {
    size_t b, e;
    int64_t parent;
    int side;  // 0 left, 1 right
    uint32_t depth;
  };
  std::vector<Task> stack;
  stack.push_back({0, n, -1, 0, 1});
  auto item_code = [](uint32_t i) { return -(int64_t)i - 2; };
  while (!stack.empty()) {
    Task t = stack.back();
    stack.pop_back();
    const int64_t me = (int64_t)out.nodes.size();
    out.nodes.emplace_back();
    out.depth = std::max(out.depth, t.depth);
    if (t.parent >= 0) (t.side == 0 ? out.nodes[t.parent].left : out.nodes[t.parent].right) = me;
    // vec_bounding_box (bvh/build/utils.rs:42-74)
    Box bb = items[ids[t.b]].box;
    for (size_t i = t.b + 1; i < t.e; ++i) box_grow(bb, items[ids[i]].box);
    out.nodes[me].box = bb;
    const size_t count = t.e - t.b;
    if (count == 1) {
      out.nodes[me].left = item_code(ids[t.b]);
      continue;
    }
    if (count == 2) {
      out.nodes[me].left = item_code(ids[t.b]);
      out.nodes[me].right = item_code(ids[t.b + 1]);
      continue;
    }
    // find_best_split (surface_area_heuristic.rs:81-132).  The 8 candidates
    // of an axis are scored in one pass: an item is left of candidate i iff
    // c <= cand[i], and min/max box growth is exact, so binning reproduces
    // evaluate_sah's sums bit for bit.
    int best_axis = 0;
    float best_pos = 0.0f, best_cost = INFINITY;
    for (int axis = 0; axis < 3; ++axis) {
      float bmin = INFINITY, bmax = -INFINITY;
      for (size_t i = t.b; i < t.e; ++i) {
        const float cv = items[ids[i]].c[axis];
        bmin = std::fmin(bmin, cv);
        bmax = std::fmax(bmax, cv);
      }
      if (bmin == bmax) continue;
      const float scale = (bmax - bmin) / 8.0f;
      float cand[8];
      for (int i = 0; i < 8; ++i) cand[i] = bmin + (float)i * scale;
      Box binb[9];
      bool used[9] = {false, false, false, false, false, false, false, false, false};
      uint64_t binc[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0};
      for (size_t i = t.b; i < t.e; ++i) {
        const Item& it = items[ids[i]];
        const float cv = it.c[axis];
        int k = 0;
        while (k < 8 && !(cv <= cand[k])) ++k;  // first candidate with cv <= cand
        if (used[k]) box_grow(binb[k], it.box);
        else { binb[k] = it.box; used[k] = true; }
        binc[k]++;
      }
      for (int i = 0; i < 8; ++i) {
        Box lb, rb;  // both start from the zero box, as in evaluate_sah
        uint64_t lc = 0, rc = 0;
        for (int k = 0; k <= 8; ++k) {
          if (!used[k]) continue;
          if (k <= i) { box_grow(lb, binb[k]); lc += binc[k]; }
          else { box_grow(rb, binb[k]); rc += binc[k]; }
        }
        const float cost = (float)lc * box_area(lb) + (float)rc * box_area(rb);
        if (cost < best_cost) {
          best_pos = cand[i];
          best_axis = axis;
          best_cost = cost;
        }
      }
    }
    // order-preserving partition on centroid[axis] <= pos
    tmp.clear();
    size_t w = t.b;
    for (size_t i = t.b; i < t.e; ++i) {
      const uint32_t id = ids[i];
      if (items[id].c[best_axis] <= best_pos) ids[w++] = id;
      else tmp.push_back(id);
    }
    std::copy(tmp.begin(), tmp.end(), ids.begin() + (std::ptrdiff_t)w);
    const size_t mid = w;
    if (mid == t.b) {  // left empty: peel the first of the right list
      out.nodes[me].left = item_code(ids[t.b]);
      stack.push_back({t.b + 1, t.e, me, 1, t.depth + 1});
      continue;
    }
    if (mid == t.e) {  // right empty: peel the first of the left list
      out.nodes[me].right = item_code(ids[t.b]);
      stack.push_back({t.b + 1, t.e, me, 0, t.depth + 1});
      continue;
    }
    stack.push_back({mid, t.e, me, 1, t.depth + 1});  // popped after the left subtree: preorder
    stack.push_back({t.b, mid, me, 0, t.depth + 1});
  }
  return out;
}

// ---- JSON helpers
using clv_json::Value;
V3 vec3_of(const Value& v, const char* what) {
  if (v.is_array() && v.arr.size() == 3) return V3(v.arr[0].as_f32(what), v.arr[1].as_f32(what), v.arr[2].as_f32(what));
  if (v.is_object() && v.has("x")) return V3(v.at("x").as_f32(what), v.at("y").as_f32(what), v.at("z").as_f32(what));
  throw std::runtime_error(std::string("expected a 3-vector for `") + what + "`");
}
void rgb_of(const Value& v, float out[3], const char* what) {
  if (v.is_array() && v.arr.size() == 3) {
    for (int i = 0; i < 3; ++i) out[i] = v.arr[i].as_f32(what);
    return;
  }
  if (v.is_object() && v.has("red")) {
    out[0] = v.at("red").as_f32(what);
    out[1] = v.at("green").as_f32(what);
    out[2] = v.at("blue").as_f32(what);
    return;
  }
  throw std::runtime_error(std::string("expected an RGB triple for `") + what + "`");
}
int hex_digit(char c) {
  if (c >= '0' && c <= '9') return c - '0';
  if (c >= 'a' && c <= 'f') return c - 'a' + 10;
  if (c >= 'A' && c <= 'F') return c - 'A' + 10;
  throw std::runtime_error("bad hex colour");
}
// ColorInit -> Xyz<E>, clovers/src/colorinit.rs:45-60
void color_xyz(const Value& v, float out[3]) {
  float t[3];
  if (v.is_array()) {
    rgb_of(v, t, "color");
    srgb_to_xyz_e(t, out);
    return;
  }
  if (!v.is_object() || v.obj.size() != 1) throw std::runtime_error("unsupported colour form");
  const std::string& k = v.obj[0].first;
  const Value& c = v.obj[0].second;
  if (k == "hex") {
    std::string s = c.as_string("hex");
    if (!s.empty() && s[0] == '#') s = s.substr(1);
    if (s.size() == 3) s = std::string{s[0], s[0], s[1], s[1], s[2], s[2]};
    if (s.size() != 6) throw std::runtime_error("bad hex colour");
    for (int i = 0; i < 3; ++i) t[i] = (float)(hex_digit(s[2 * i]) * 16 + hex_digit(s[2 * i + 1])) / 255.0f;
    srgb_to_xyz_e(t, out);
  } else if (k == "srgb") {
    rgb_of(c, t, "srgb");
    srgb_to_xyz_e(t, out);
  } else if (k == "lin_srgb") {
    rgb_of(c, t, "lin_srgb");
    linsrgb_to_xyz_e(t, out);
  } else if (k == "xyz_e") {
    V3 x = vec3_of(c, "xyz_e");
    out[0] = x.x; out[1] = x.y; out[2] = x.z;
  } else if (k == "xyz_d65") {
    V3 x = vec3_of(c, "xyz_d65");
    const float in[3] = {x.x, x.y, x.z};
    xyz_d65_to_xyz_e(in, out);
  } else {
    throw std::runtime_error("unsupported colour kind `" + k + "`");
  }
}

// PLY reader for objects/ply.rs: the vertex element's x, y, z and the face
// element's vertex_indices, from an ASCII or binary (either byte order) body.
// Value conversions follow ply.rs's property_to_float / property_to_vec_u32.
class PlyReader {
 public:
  std::vector<float> verts;     // x, y, z per vertex
  std::vector<uint64_t> faces;  // first three indices of each face
  PlyReader(const std::vector<char>& d, const std::string& path) : d_(d), path_(path) { parse(); }

 private:
  enum Type { I8, U8, I16, U16, I32, U32, F32, F64, NONE };
  struct Prop {
    std::string name;
    Type type = NONE, count = NONE;
    bool list = false;
  };
  struct Elem {
    std::string name;
    uint64_t count = 0;
    std::vector<Prop> props;
  };
  const std::vector<char>& d_;
  std::string path_;
  size_t pos_ = 0;
  int format_ = 0;  // 0 ascii, 1 binary little endian, 2 binary big endian

  [[noreturn]] void bad(const std::string& m) const { throw std::runtime_error("PLY file `" + path_ + "`: " + m); }
  static Type type_of(const std::string& t) {
    if (t == "char" || t == "int8") return I8;
    if (t == "uchar" || t == "uint8") return U8;
    if (t == "short" || t == "int16") return I16;
    if (t == "ushort" || t == "uint16") return U16;
    if (t == "int" || t == "int32") return I32;
    if (t == "uint" || t == "uint32") return U32;
    if (t == "float" || t == "float32") return F32;
    if (t == "double" || t == "float64") return F64;
    return NONE;
  }
  static int size_of(Type t) { return t <= U8 ? 1 : t <= U16 ? 2 : t <= F32 ? 4 : 8; }
  std::string line() {
    if (pos_ >= d_.size()) bad("header ends early");
    size_t e = pos_;
    while (e < d_.size() && d_[e] != '\n') ++e;
    std::string l(d_.data() + pos_, e - pos_);
    pos_ = e < d_.size() ? e + 1 : e;
    if (!l.empty() && l.back() == '\r') l.pop_back();
    return l;
  }
  static std::vector<std::string> words(const std::string& l) {
    std::vector<std::string> w;
    size_t i = 0;
    while (i < l.size()) {
      while (i < l.size() && (l[i] == ' ' || l[i] == '\t')) ++i;
      size_t j = i;
      while (j < l.size() && l[j] != ' ' && l[j] != '\t') ++j;
      if (j > i) w.emplace_back(l.substr(i, j - i));
      i = j;
    }
    return w;
  }
  std::string token() {  // ASCII body
    while (pos_ < d_.size() && std::isspace((unsigned char)d_[pos_])) ++pos_;
    const size_t b = pos_;
    while (pos_ < d_.size() && !std::isspace((unsigned char)d_[pos_])) ++pos_;
    if (b == pos_) bad("body ends early");
    return std::string(d_.data() + b, pos_ - b);
  }
  void raw(Type t, unsigned char* out) {  // binary body, host byte order
    const int n = size_of(t);
    if (pos_ + n > d_.size()) bad("body ends early");
    unsigned char b[8];
    std::memcpy(b, d_.data() + pos_, n);
    pos_ += n;
    const uint16_t one = 1;
    const bool host_le = *reinterpret_cast<const unsigned char*>(&one) == 1;
    const bool file_le = format_ == 1;
    for (int k = 0; k < n; ++k) out[k] = b[host_le == file_le ? k : n - 1 - k];
  }
  // an integer-valued property (list counts, indices); signed values as read
  int64_t integer(Type t) {
    if (t == F32 || t == F64 || t == NONE) bad("non-integer list count or index");
    if (format_ == 0) return std::strtoll(token().c_str(), nullptr, 10);
    unsigned char b[8];
    raw(t, b);
    switch (t) {
      case I8: { int8_t v; std::memcpy(&v, b, 1); return v; }
      case U8: return b[0];
      case I16: { int16_t v; std::memcpy(&v, b, 2); return v; }
      case U16: { uint16_t v; std::memcpy(&v, b, 2); return v; }
      case I32: { int32_t v; std::memcpy(&v, b, 4); return v; }
      default: { uint32_t v; std::memcpy(&v, b, 4); return v; }
    }
  }
  // property_to_float: int, uint, float and double properties, as f32
  float coord(Type t) {
    if (t == F32) {
      if (format_ == 0) return std::strtof(token().c_str(), nullptr);
      float v;
      unsigned char b[4];
      raw(t, b);
      std::memcpy(&v, b, 4);
      return v;
    }
    if (t == F64) {
      if (format_ == 0) return (float)std::strtod(token().c_str(), nullptr);
      double v;
      unsigned char b[8];
      raw(t, b);
      std::memcpy(&v, b, 8);
      return (float)v;
    }
    if (t == I32 || t == U32) return (float)integer(t);
    bad("unsupported vertex coordinate type");
  }
  void skip(Type t) {
    if (format_ == 0) token();
    else {
      unsigned char b[8];
      raw(t, b);
    }
  }
  void parse() {
    if (line() != "ply") bad("not a PLY file");
    std::vector<Elem> elems;
    while (true) {
      const std::vector<std::string> w = words(line());
      if (w.empty()) continue;
      if (w[0] == "end_header") break;
      if (w[0] == "comment" || w[0] == "obj_info") continue;
      if (w[0] == "format") {
        if (w.size() < 2) bad("bad format line");
        format_ = w[1] == "ascii" ? 0 : w[1] == "binary_little_endian" ? 1 : w[1] == "binary_big_endian" ? 2 : -1;
        if (format_ < 0) bad("unknown format " + w[1]);
      } else if (w[0] == "element") {
        if (w.size() < 3) bad("bad element line");
        Elem e;
        e.name = w[1];
        e.count = std::strtoull(w[2].c_str(), nullptr, 10);
        elems.push_back(e);
      } else if (w[0] == "property") {
        if (elems.empty()) bad("property before element");
        Prop p;
        if (w.size() >= 5 && w[1] == "list") {
          p.list = true;
          p.count = type_of(w[2]);
          p.type = type_of(w[3]);
          p.name = w[4];
        } else if (w.size() >= 3) {
          p.type = type_of(w[1]);
          p.name = w[2];
        } else {
          bad("bad property line");
        }
        if (p.type == NONE || (p.list && p.count == NONE)) bad("unknown property type");
        elems.back().props.push_back(p);
      } else {
        bad("unknown header line `" + w[0] + "`");
      }
    }
    bool have_v = false, have_f = false;
    for (const Elem& e : elems) {
      const bool vert = e.name == "vertex", face = e.name == "face";
      int xyz[3] = {-1, -1, -1}, vi = -1;
      for (size_t k = 0; k < e.props.size(); ++k) {
        const Prop& p = e.props[k];
        if (vert && !p.list && (p.name == "x" || p.name == "y" || p.name == "z")) xyz[p.name[0] - 'x'] = (int)k;
        if (face && p.list && p.name == "vertex_indices") vi = (int)k;
      }
      if (vert) {
        if (xyz[0] < 0 || xyz[1] < 0 || xyz[2] < 0) bad("vertex element without x, y, z");
        if (e.count > (1ull << 32)) bad("too many vertices");
        verts.assign(3 * e.count, 0.0f);
        have_v = true;
      }
      if (face) {
        if (vi < 0) bad("face element without vertex_indices");
        const Type it = e.props[vi].type;
        if (it == I8 || it == F32 || it == F64) bad("unsupported vertex_indices type");
        if (e.count > (1ull << 32)) bad("too many faces");
        faces.reserve(3 * e.count);
        have_f = true;
      }
      for (uint64_t r = 0; r < e.count; ++r) {
        for (size_t k = 0; k < e.props.size(); ++k) {
          const Prop& p = e.props[k];
          if (p.list) {
            const int64_t n = integer(p.count);
            if (n < 0) bad("negative list length");
            const bool take = face && (int)k == vi;
            if (take && n < 3) bad("face with fewer than 3 vertices");
            for (int64_t j = 0; j < n; ++j) {
              if (take && j < 3) {
                const int64_t v = integer(p.type);
                faces.push_back((uint64_t)(v < 0 ? -v : v));  // signed lists: unsigned_abs
              } else {
                skip(p.type);
              }
            }
          } else if (vert && ((int)k == xyz[0] || (int)k == xyz[1] || (int)k == xyz[2])) {
            verts[3 * r + (p.name[0] - 'x')] = coord(p.type);
          } else {
            skip(p.type);
          }
        }
      }
    }
    if (!have_v || !have_f) bad("vertex or face element missing");
  }
};

struct Emitted {
  uint32_t ref = CLV_REF_EMPTY;
  bool has_box = false;
  Box box;
  V3 c;
  bool can_sample = false;  // HitableTrait::random is implemented
  bool is_list = false;
  std::vector<Emitted> items;  // ObjectList / STL members, flattened at top level
};

class Builder {
 public:
  HostScene& S;
  std::string base_dir;
  std::vector<std::pair<std::string, uint32_t>> shared;
  uint32_t fallback = 0;

  explicit Builder(HostScene& s) : S(s) {}

  uint32_t add_spd(const float xyz[3]) {
    const size_t off = S.spd.size();
    S.spd.resize(off + 400);
    spd_table(xyz, &S.spd[off]);
    return (uint32_t)(off / 400);
  }
  uint32_t grey_spd() {
    const float g[3] = {0.5f, 0.5f, 0.5f};
    return add_spd(g);
  }

  // Texture (clovers/src/textures.rs:17-109) into the material's texture slots.
  void texture(const Value* v, ClvMaterial& m) {
    if (!v) {  // Texture::default(): SolidColor of XYZ(E) (0.5, 0.5, 0.5)
      m.tex_kind = CLV_TEX_SOLID;
      m.spd_even = grey_spd();
      return;
    }
    const std::string& kind = v->at("kind").as_string("texture kind");
    if (kind == "SolidColor") {
      float xyz[3];
      color_xyz(v->at("color"), xyz);
      m.tex_kind = CLV_TEX_SOLID;
      m.spd_even = add_spd(xyz);
    } else if (kind == "SpatialChecker" || kind == "SurfaceChecker") {
      float ev[3] = {0.8f, 0.8f, 0.8f}, od[3] = {0.5f, 0.5f, 0.5f};
      if (v->has("even")) color_xyz(v->at("even"), ev);
      if (v->has("odd")) color_xyz(v->at("odd"), od);
      m.tex_kind = kind == "SpatialChecker" ? CLV_TEX_SPATIAL : CLV_TEX_SURFACE;
      m.spd_even = add_spd(ev);
      m.spd_odd = add_spd(od);
      m.density = v->has("density") ? v->at("density").as_f32("density") : (kind == "SpatialChecker" ? 1.0f : 10.0f);
    } else if (kind.rfind("Illuminant", 0) == 0) {
      std::string suffix = kind.substr(10);
      if (suffix.rfind("Led", 0) == 0) suffix = "LED_" + suffix.substr(3);
      int found = -1;
      for (int i = 0; i < clv_tables::kNumIlluminants; ++i)
        if (suffix == clv_tables::kIlluminantNames[i]) found = i;
      if (found < 0) throw std::runtime_error("unknown texture kind `" + kind + "`");
      m.tex_kind = CLV_TEX_ILLUMINANT;
      m.illuminant = (uint32_t)found;
      m.intensity = v->has("intensity") ? v->at("intensity").as_f32("intensity") : 1.0f;
    } else {
      throw std::runtime_error("unknown texture kind `" + kind + "`");
    }
  }

  // Material (clovers/src/materials.rs:50-103)
  uint32_t material(const Value& v) {
    ClvMaterial m;
    std::memset(&m, 0, sizeof m);
    m.refractive_index = 1.5f;
    m.cauchy_a = 1.5046f;
    m.cauchy_b = 0.0042f;
    m.spread = 10.0f;
    const std::string& kind = v.at("kind").as_string("material kind");
    if (kind == "Lambertian" || kind == "Isotropic") {
      m.kind = kind == "Lambertian" ? CLV_MAT_LAMBERTIAN : CLV_MAT_ISOTROPIC;
      texture(v.find("albedo"), m);
    } else if (kind == "Metal") {
      m.kind = CLV_MAT_METAL;
      texture(v.find("albedo"), m);
      m.fuzz = v.has("fuzz") ? v.at("fuzz").as_f32("fuzz") : 0.0f;  // serde path: no clamp (metal.rs:57-62)
    } else if (kind == "Dielectric") {
      m.kind = CLV_MAT_DIELECTRIC;
      if (v.has("refractive_index")) m.refractive_index = v.at("refractive_index").as_f32("refractive_index");
      float c[3] = {1.0f, 1.0f, 1.0f};
      if (v.has("color")) {
        V3 x = vec3_of(v.at("color"), "color");
        c[0] = x.x; c[1] = x.y; c[2] = x.z;
      }
      m.spd_even = add_spd(c);
    } else if (kind == "Dispersive") {
      m.kind = CLV_MAT_DISPERSIVE;
      if (v.has("cauchy_a")) m.cauchy_a = v.at("cauchy_a").as_f32("cauchy_a");
      if (v.has("cauchy_b")) m.cauchy_b = v.at("cauchy_b").as_f32("cauchy_b");
      if (v.has("sellmeier_b") || v.has("sellmeier_c")) {  // extension: Sellmeier form
        V3 b = vec3_of(v.at("sellmeier_b"), "sellmeier_b"), c = vec3_of(v.at("sellmeier_c"), "sellmeier_c");
        m.sellmeier = 1;
        for (int i = 0; i < 3; ++i) { m.sell_b[i] = b[i]; m.sell_c[i] = c[i]; }
      }
    } else if (kind == "DiffuseLight") {
      m.kind = CLV_MAT_DIFFUSELIGHT;
      texture(&v.at("emit"), m);
    } else if (kind == "ConeLight") {
      m.kind = CLV_MAT_CONELIGHT;
      m.spread = v.at("spread").as_f32("spread");
      texture(&v.at("emit"), m);
    } else {
      throw std::runtime_error("unknown material kind `" + kind + "`");
    }
    const Value* tf = v.find("thin_film");
    if (tf && !tf->is_null()) {
      m.thin_film = 1;
      m.tf_ior = tf->has("refractive_index") ? tf->at("refractive_index").as_f32("refractive_index") : 1.5f;
      m.tf_thickness = tf->has("thickness") ? tf->at("thickness").as_f32("thickness") : 500.0f;
    }
    m.wavelength_dependent = (m.thin_film || m.kind == CLV_MAT_DISPERSIVE) ? 1u : 0u;
    S.materials.push_back(m);
    return (uint32_t)(S.materials.size() - 1);
  }

  uint32_t default_material() {  // SharedMaterial::default(): Lambertian, grey
    ClvMaterial m;
    std::memset(&m, 0, sizeof m);
    m.kind = CLV_MAT_LAMBERTIAN;
    m.tex_kind = CLV_TEX_SOLID;
    m.spd_even = grey_spd();
    m.refractive_index = 1.5f;
    m.cauchy_a = 1.5046f;
    m.cauchy_b = 0.0042f;
    m.spread = 10.0f;
    S.materials.push_back(m);
    return (uint32_t)(S.materials.size() - 1);
  }

  // MaterialInit (materials.rs:31-45): a shared name or an inline material
  uint32_t material_ref(const Value* v, bool strict = false) {
    if (!v || v->is_string()) {
      const std::string name = v ? v->str : std::string();
      for (auto& kv : shared)
        if (kv.first == name) return kv.second;
      if (strict) throw std::runtime_error("material `" + name + "` not found");
      for (auto& kv : shared)
        if (kv.first.empty()) return kv.second;
      return fallback;
    }
    return material(*v);
  }

  // corners: a triangle's vertices as given (from_coordinates); otherwise q,
  // q + u, q + v.  They feed only the optional watertight test.
  Emitted planar(V3 q, V3 u, V3 v, uint32_t mat, bool tri, bool top, const V3* corners = nullptr) {
    // triangle.rs:61-101 / quad.rs:61-83
    const V3 n = cross(u, v);
    const V3 nn = unit(n);
    const float d = -(dot(nn, q));
    const V3 w = n / dot(n, n);
    ClvPlanar r;
    const float f[16] = {q.x, q.y, q.z, u.x, u.y, u.z, v.x, v.y, v.z, nn.x, nn.y, nn.z, d, w.x, w.y, w.z};
    std::memcpy(r.f, f, sizeof f);
    Emitted e;
    if (tri) {
      const V3 c1 = q, c2 = q + u, c3 = q + v;
      e.box.b[0] = std::fmin(std::fmin(c1.x, c2.x), c3.x); e.box.b[1] = std::fmax(std::fmax(c1.x, c2.x), c3.x);
      e.box.b[2] = std::fmin(std::fmin(c1.y, c2.y), c3.y); e.box.b[3] = std::fmax(std::fmax(c1.y, c2.y), c3.y);
      e.box.b[4] = std::fmin(std::fmin(c1.z, c2.z), c3.z); e.box.b[5] = std::fmax(std::fmax(c1.z, c2.z), c3.z);
      e.c = q + (u / 4.0f) + (v / 4.0f);
      S.tris.push_back(r);
      const V3 vs[3] = {corners ? corners[0] : c1, corners ? corners[1] : c2, corners ? corners[2] : c3};
      for (const V3& p : vs) {
        S.tri_verts.push_back(p.x);
        S.tri_verts.push_back(p.y);
        S.tri_verts.push_back(p.z);
        S.tri_verts.push_back(0.0f);
      }
      S.tri_mat.push_back(mat);
      S.tri_gid.push_back(CLV_REF_EMPTY);
      S.tri_area.push_back(length(n) / 2.0f);
      e.ref = CLV_MAKE_REF(CLV_REF_TRI, S.tris.size() - 1);
    } else {
      e.box = box_from(q, q + u + v);
      e.c = q + (u / 2.0f) + (v / 2.0f);
      S.quads.push_back(r);
      S.quad_mat.push_back(mat);
      S.quad_gid.push_back(CLV_REF_EMPTY);
      S.quad_area.push_back(length(n));
      e.ref = CLV_MAKE_REF(CLV_REF_QUAD, S.quads.size() - 1);
    }
    box_pad(e.box);
    e.has_box = true;
    e.can_sample = true;
    (void)top;
    return e;
  }

  Emitted sphere(V3 c, float r, uint32_t mat) {  // sphere.rs:40-54
    S.spheres.insert(S.spheres.end(), {c.x, c.y, c.z, r});
    S.sphere_mat.push_back(mat);
    S.sphere_gid.push_back(CLV_REF_EMPTY);
    Emitted e;
    e.ref = CLV_MAKE_REF(CLV_REF_SPHERE, S.spheres.size() / 4 - 1);
    e.box = box_from(c - V3(r, r, r), c + V3(r, r, r));
    e.has_box = true;
    e.c = c;
    e.can_sample = true;
    return e;
  }

  uint32_t push_obj(const ClvObj& o) {
    S.objs.push_back(o);
    S.obj_gid.push_back(CLV_REF_EMPTY);
    return CLV_MAKE_REF(CLV_REF_OBJ, S.objs.size() - 1);
  }
  static ClvObj blank_obj(uint32_t kind) {
    ClvObj o;
    std::memset(&o, 0, sizeof o);
    o.kind = kind;
    return o;
  }

  // Rotation3::from_euler_angles(roll, pitch, yaw) in degrees, row-major
  static void euler_matrix(const V3& rot, float R[9]) {
    const float sr = std::sin(rot.x * kDegToRad), cr = std::cos(rot.x * kDegToRad);
    const float sp = std::sin(rot.y * kDegToRad), cp = std::cos(rot.y * kDegToRad);
    const float sy = std::sin(rot.z * kDegToRad), cy = std::cos(rot.z * kDegToRad);
    const float M[9] = {cy * cp, cy * sp * sr - sy * cr, cy * sp * cr + sy * sr,
                        sy * cp, sy * sp * sr + cy * cr, sy * sp * cr - cy * sr,
                        -sp,     cp * sr,                cp * cr};
    std::memcpy(R, M, sizeof M);
  }

  std::vector<char> read_file(const std::string& path, const char* what) {
    std::ifstream f(path, std::ios::binary);
    if (!f && !base_dir.empty()) f.open(base_dir + "/" + path, std::ios::binary);
    if (!f) throw std::runtime_error(std::string("cannot open ") + what + " file `" + path + "`");
    return std::vector<char>((std::istreambuf_iterator<char>(f)), std::istreambuf_iterator<char>());
  }

  // objects/ply.rs:55-118: vertices x, y, z (int, uint, float or double
  // properties), faces from the first three `vertex_indices` of each face
  // (unsigned lists as read, signed lists by absolute value), rotated, scaled
  // and offset like STL triangles.  Binary (either byte order) and ASCII bodies.
  void ply_triangles(const Value& o, std::vector<Emitted>& out) {
    const std::string path = o.at("path").as_string("path");
    const std::vector<char> data = read_file(path, "PLY");
    PlyReader ply(data, path);
    const uint32_t mat = material_ref(o.find("material"), true);
    const float scale = o.at("scale").as_f32("scale");
    const V3 center = vec3_of(o.at("center"), "center");
    float R[9];
    euler_matrix(vec3_of(o.at("rotation"), "rotation"), R);
    for (size_t f = 0; f < ply.faces.size(); f += 3) {
      V3 p[3];
      for (int k = 0; k < 3; ++k) {
        const uint64_t vi = ply.faces[f + k];
        if (vi >= ply.verts.size() / 3) throw std::runtime_error("PLY face index out of range in `" + path + "`");
        const V3 a(ply.verts[3 * vi], ply.verts[3 * vi + 1], ply.verts[3 * vi + 2]);
        const V3 r(R[0] * a.x + R[1] * a.y + R[2] * a.z, R[3] * a.x + R[4] * a.y + R[5] * a.z,
                   R[6] * a.x + R[7] * a.y + R[8] * a.z);
        p[k] = V3(r.x * scale, r.y * scale, r.z * scale) + center;
      }
      out.push_back(planar(p[0], p[1] - p[0], p[2] - p[0], mat, true, false, p));
    }
  }

  void stl_triangles(const Value& o, std::vector<Emitted>& out) {  // objects/stl.rs:52-104
    const std::string path = o.at("path").as_string("path");
    const std::vector<char> data = read_file(path, "STL");
    if (data.size() < 84) throw std::runtime_error("STL file too short");
    uint32_t n;
    std::memcpy(&n, data.data() + 80, 4);
    if (data.size() < 84 + (size_t)n * 50) throw std::runtime_error("STL file truncated (binary STL expected)");
    const uint32_t mat = material_ref(o.find("material"), true);
    const float scale = o.at("scale").as_f32("scale");
    const V3 center = vec3_of(o.at("center"), "center");
    float R[9];
    euler_matrix(vec3_of(o.at("rotation"), "rotation"), R);
    for (uint32_t i = 0; i < n; ++i) {
      const char* rec = data.data() + 84 + (size_t)i * 50;
      V3 p[3];
      for (int k = 0; k < 3; ++k) {
        float c[3];
        std::memcpy(c, rec + 12 + 12 * k, 12);
        const V3 a(c[0], c[1], c[2]);
        const V3 r(R[0] * a.x + R[1] * a.y + R[2] * a.z, R[3] * a.x + R[4] * a.y + R[5] * a.z,
                   R[6] * a.x + R[7] * a.y + R[8] * a.z);
        p[k] = V3(r.x * scale, r.y * scale, r.z * scale) + center;
      }
      out.push_back(planar(p[0], p[1] - p[0], p[2] - p[0], mat, true, false, p));
    }
  }

  // object_to_hitable, clovers/src/objects.rs:91-157
  Emitted object(const Value& o) {
    const std::string& kind = o.at("kind").as_string("object kind");
    if (kind == "Sphere")
      return sphere(vec3_of(o.at("center"), "center"), o.at("radius").as_f32("radius"), material_ref(o.find("material")));
    if (kind == "Quad" || kind == "Triangle")
      return planar(vec3_of(o.at("q"), "q"), vec3_of(o.at("u"), "u"), vec3_of(o.at("v"), "v"),
                    material_ref(o.find("material")), kind == "Triangle", false);
    if (kind == "Boxy") {  // boxy.rs:40-73
      const V3 c0 = vec3_of(o.at("corner_0"), "corner_0"), c1 = vec3_of(o.at("corner_1"), "corner_1");
      const uint32_t mat = material_ref(o.find("material"));
      const V3 mn(std::fmin(c0.x, c1.x), std::fmin(c0.y, c1.y), std::fmin(c0.z, c1.z));
      const V3 mx(std::fmax(c0.x, c1.x), std::fmax(c0.y, c1.y), std::fmax(c0.z, c1.z));
      const V3 dx(mx.x - mn.x, 0, 0), dy(0, mx.y - mn.y, 0), dz(0, 0, mx.z - mn.z);
      const uint32_t first = (uint32_t)S.quads.size();
      planar(V3(mn.x, mn.y, mx.z), dx, dy, mat, false, false);
      planar(V3(mx.x, mn.y, mx.z), -dz, dy, mat, false, false);
      planar(V3(mx.x, mn.y, mn.z), -dx, dy, mat, false, false);
      planar(V3(mn.x, mn.y, mn.z), dz, dy, mat, false, false);
      planar(V3(mn.x, mx.y, mx.z), dx, -dz, mat, false, false);
      planar(V3(mn.x, mn.y, mn.z), dx, dz, mat, false, false);
      ClvObj ob = blank_obj(CLV_OBJ_BOXY);
      ob.a = first;
      Emitted e;
      e.ref = push_obj(ob);
      e.box = box_from(c0, c1);
      e.has_box = true;
      e.c = box_center(e.box);
      return e;
    }
    if (kind == "MovingSphere") {  // moving_sphere.rs:52-82, times fixed to 0..1 (objects.rs:101-104)
      const V3 c0 = vec3_of(o.at("center_0"), "center_0"), c1 = vec3_of(o.at("center_1"), "center_1");
      const float r = o.at("radius").as_f32("radius");
      ClvObj ob = blank_obj(CLV_OBJ_MOVING);
      ob.b = material_ref(o.find("material"));
      const float p[9] = {c0.x, c0.y, c0.z, c1.x, c1.y, c1.z, 0.0f, 1.0f, r};
      std::memcpy(ob.p, p, sizeof p);
      Emitted e;
      e.ref = push_obj(ob);
      Box b0 = box_from(c0 - V3(r, r, r), c0 + V3(r, r, r));
      const Box b1 = box_from(c1 - V3(r, r, r), c1 + V3(r, r, r));
      box_grow(b0, b1);
      e.box = b0;
      e.has_box = true;
      e.c = c0 + ((0.5f - 0.0f) / (1.0f - 0.0f)) * (c1 - c0);
      return e;
    }
    if (kind == "ObjectList" || kind == "STL" || kind == "PLY") {
      Emitted e;
      e.is_list = true;
      if (kind == "STL") stl_triangles(o, e.items);
      else if (kind == "PLY") ply_triangles(o, e.items);
      else
        for (auto& c : o.at("objects").arr) e.items.push_back(object(c));
      // HitableList::new (hitable.rs:139-143)
      bool first = true;
      for (auto& it : e.items) {
        if (!it.has_box) throw std::runtime_error("No bounding box for hitables");
        if (first) { e.box = it.box; first = false; }
        else box_grow(e.box, it.box);
      }
      if (first) throw std::runtime_error("No bounding box for hitables");
      e.has_box = true;
      e.c = box_center(e.box);
      // as a nested object (inside a wrapper) the list is a real object
      ClvObj ob = blank_obj(CLV_OBJ_LIST);
      ob.a = (uint32_t)S.obj_children.size();
      ob.b = (uint32_t)e.items.size();
      for (auto& it : e.items) S.obj_children.push_back(it.ref);
      e.ref = push_obj(ob);
      return e;
    }
    if (kind == "Translate") {  // translate.rs:33-78
      Emitted inner = object(o.at("object"));
      const V3 off = vec3_of(o.at("offset"), "offset");
      if (!inner.has_box) throw std::runtime_error("Translate of an object without a bounding box");
      ClvObj ob = blank_obj(CLV_OBJ_TRANSLATE);
      ob.a = inner.ref;
      ob.p[0] = off.x; ob.p[1] = off.y; ob.p[2] = off.z;
      Emitted e;
      e.ref = push_obj(ob);
      e.has_box = true;
      for (int k = 0; k < 3; ++k) {
        const float a = inner.box.b[2 * k] + off[k], b = inner.box.b[2 * k + 1] + off[k];
        e.box.b[2 * k] = std::fmin(a, b);
        e.box.b[2 * k + 1] = std::fmax(a, b);
      }
      e.c = inner.c + off;
      return e;
    }
    if (kind == "RotateY") {  // rotate.rs:32-72
      Emitted inner = object(o.at("object"));
      const float rad = o.at("angle").as_f32("angle") * kDegToRad;
      const float s = std::sin(rad), c = std::cos(rad);
      ClvObj ob = blank_obj(CLV_OBJ_ROTATEY);
      ob.a = inner.ref;
      ob.p[0] = s;
      ob.p[1] = c;
      Emitted e;
      e.ref = push_obj(ob);
      e.c = inner.c;
      if (inner.has_box) {
        V3 mn(INFINITY, INFINITY, INFINITY), mx(-INFINITY, -INFINITY, -INFINITY);
        float mnv[3] = {INFINITY, INFINITY, INFINITY}, mxv[3] = {-INFINITY, -INFINITY, -INFINITY};
        const Box& bb = inner.box;
        for (int i = 0; i < 2; ++i)
          for (int j = 0; j < 2; ++j)
            for (int k = 0; k < 2; ++k) {
              const float fi = (float)i, fj = (float)j, fk = (float)k;
              const float x = fi * bb.b[1] + (1.0f - fi) * bb.b[0];
              const float y = fj * bb.b[3] + (1.0f - fj) * bb.b[2];
              const float z = fk * bb.b[5] + (1.0f - fk) * bb.b[4];
              const float t[3] = {c * x + s * z, y, -s * x + c * z};
              for (int a = 0; a < 3; ++a) {
                mnv[a] = std::fmin(mnv[a], t[a]);
                mxv[a] = std::fmax(mxv[a], t[a]);
              }
            }
        (void)mn; (void)mx;
        e.box = box_from(V3(mnv[0], mnv[1], mnv[2]), V3(mxv[0], mxv[1], mxv[2]));
        e.has_box = true;
      }
      return e;
    }
    if (kind == "ConstantMedium") {  // constant_medium.rs:51-61
      Emitted inner = object(o.at("boundary"));
      const float density = o.has("density") ? o.at("density").as_f32("density") : 0.1f;
      ClvMaterial m;
      std::memset(&m, 0, sizeof m);
      m.kind = CLV_MAT_ISOTROPIC;
      m.refractive_index = 1.5f;
      m.spread = 10.0f;
      texture(o.find("texture"), m);
      S.materials.push_back(m);
      ClvObj ob = blank_obj(CLV_OBJ_MEDIUM);
      ob.a = inner.ref;
      ob.b = (uint32_t)(S.materials.size() - 1);
      ob.p[0] = -1.0f / density;
      Emitted e;
      e.ref = push_obj(ob);
      e.has_box = inner.has_box;
      e.box = inner.box;
      e.c = inner.c;
      return e;
    }
    throw std::runtime_error("unsupported object kind `" + kind + "`");
  }
};

void set_gid(HostScene& S, uint32_t ref, uint32_t gid) {
  const uint32_t k = CLV_REF_KIND(ref), i = CLV_REF_INDEX(ref);
  if (k == CLV_REF_TRI) S.tri_gid[i] = gid;
  else if (k == CLV_REF_QUAD) S.quad_gid[i] = gid;
  else if (k == CLV_REF_SPHERE) S.sphere_gid[i] = gid;
  else if (k == CLV_REF_OBJ) S.obj_gid[i] = gid;
}

// longest_axis_midpoint.rs:12-93: the list sorted by box minimum along the
// axis of largest span, split at its middle (one object and a node of two at
// three objects).  The reference's comparator (bvh/build/utils.rs:7-21)
// answers Less only for a strictly smaller minimum: a stable sort keeps ties
// in list order, and the two-object case, which compares the pair directly,
// puts the second object first on a tie.  Nodes in preorder, like sah_build.
BuildResult lam_build(const std::vector<Item>& items) {
  BuildResult out;
  const size_t n = items.size();
  if (n == 0) throw std::runtime_error("BVH build over an empty list (the reference's builder panics)");
  std::vector<uint32_t> ids(n);
  for (size_t i = 0; i < n; ++i) ids[i] = (uint32_t)i;
  struct Task {
    size_t b, e;
    int64_t parent;
    int side;
    uint32_t depth;
  };
  std::vector<Task> stack;
  stack.push_back({0, n, -1, 0, 1});
  auto item_code = [](uint32_t i) { return -(int64_t)i - 2; };
  while (!stack.empty()) {
    const Task t = stack.back();
    stack.pop_back();
    const int64_t me = (int64_t)out.nodes.size();
    out.nodes.emplace_back();
    out.depth = std::max(out.depth, t.depth);
    if (t.parent >= 0) (t.side == 0 ? out.nodes[t.parent].left : out.nodes[t.parent].right) = me;
    Box bb = items[ids[t.b]].box;
    for (size_t i = t.b + 1; i < t.e; ++i) box_grow(bb, items[ids[i]].box);
    out.nodes[me].box = bb;
    const float sx = bb.b[1] - bb.b[0], sy = bb.b[3] - bb.b[2], sz = bb.b[5] - bb.b[4];
    const float largest = std::fmax(std::fmax(sx, sy), sz);
    const int axis = sx == largest ? 0 : (sy == largest ? 1 : (sz == largest ? 2 : -1));
    if (axis < 0) throw std::runtime_error("no axis of largest span (NaN box)");
    auto key = [&](uint32_t i) { return items[i].box.b[2 * axis]; };
    const size_t count = t.e - t.b;
    if (count == 1) {
      out.nodes[me].left = item_code(ids[t.b]);
      continue;
    }
    if (count == 2) {
      const uint32_t a = ids[t.b], c = ids[t.b + 1];
      const bool keep = key(a) < key(c);
      out.nodes[me].left = item_code(keep ? a : c);
      out.nodes[me].right = item_code(keep ? c : a);
      continue;
    }
    std::stable_sort(ids.begin() + (std::ptrdiff_t)t.b, ids.begin() + (std::ptrdiff_t)t.e,
                     [&](uint32_t a, uint32_t c) { return key(a) < key(c); });
    if (count == 3) {
      out.nodes[me].left = item_code(ids[t.b]);
      const int64_t r = (int64_t)out.nodes.size();
      out.nodes.emplace_back();
      out.nodes[me].right = r;
      Box rb = items[ids[t.b + 1]].box;
      box_grow(rb, items[ids[t.b + 2]].box);
      out.nodes[r].box = rb;
      out.nodes[r].left = item_code(ids[t.b + 1]);
      out.nodes[r].right = item_code(ids[t.b + 2]);
      out.depth = std::max(out.depth, t.depth + 1);
      continue;
    }
    const size_t mid = t.b + count / 2;
    stack.push_back({mid, t.e, me, 1, t.depth + 1});  // popped after the left subtree: preorder
    stack.push_back({t.b, mid, me, 0, t.depth + 1});
  }
  return out;
}

void store_box(float dst[6], const Box& b) { std::memcpy(dst, b.b, sizeof b.b); }

// Main BVH: nodes carry both children's boxes.
void flatten_main(HostScene& S, const std::vector<Emitted>& tops, bool lam = false) {
  std::vector<Item> items(tops.size());
  for (size_t i = 0; i < tops.size(); ++i) {
    if (!tops[i].has_box) throw std::runtime_error("an unbounded object cannot be placed in the BVH");
    items[i].box = tops[i].box;
    items[i].c = tops[i].c;
  }
  BuildResult br = lam ? lam_build(items) : sah_build(items);
  S.nodes.resize(br.nodes.size());
  auto child = [&](int64_t code, float box[6]) -> uint32_t {
    if (code == kEmpty) { std::memset(box, 0, 6 * sizeof(float)); return CLV_REF_EMPTY; }
    if (code >= 0) { store_box(box, br.nodes[(size_t)code].box); return CLV_MAKE_REF(CLV_REF_NODE, code); }
    const size_t it = (size_t)(-code - 2);
    store_box(box, items[it].box);
    return tops[it].ref;
  };
  for (size_t i = 0; i < br.nodes.size(); ++i) {
    ClvNode& n = S.nodes[i];
    std::memset(&n, 0, sizeof n);
    n.left = child(br.nodes[i].left, n.lbox);
    n.right = child(br.nodes[i].right, n.rbox);
  }
  S.root = CLV_MAKE_REF(CLV_REF_NODE, 0);
  store_box(S.root_box, br.nodes[0].box);
  S.tree_depth = br.depth;
}

void flatten_mis(HostScene& S, const std::vector<Emitted>& prio, bool lam = false) {
  std::vector<Item> items(prio.size());
  for (size_t i = 0; i < prio.size(); ++i) {
    if (!prio[i].has_box) throw std::runtime_error("an unbounded priority object cannot be placed in the MIS BVH");
    if (!prio[i].can_sample)
      throw std::runtime_error(
          "a priority object has no HitableTrait::random (only spheres, quads and triangles do; the reference "
          "panics when it samples one)");
    items[i].box = prio[i].box;
    items[i].c = prio[i].c;
  }
  BuildResult br = lam ? lam_build(items) : sah_build(items);
  S.mis_nodes.resize(br.nodes.size());
  auto child = [&](int64_t code) -> uint32_t {
    if (code == kEmpty) return CLV_REF_EMPTY;
    if (code >= 0) return CLV_MAKE_REF(CLV_REF_NODE, code);
    return prio[(size_t)(-code - 2)].ref;
  };
  for (size_t i = 0; i < br.nodes.size(); ++i) {
    S.mis_nodes[i].left = child(br.nodes[i].left);
    S.mis_nodes[i].right = child(br.nodes[i].right);
  }
  S.mis_root = CLV_MAKE_REF(CLV_REF_NODE, 0);
  S.mis_depth = br.depth;
}

void camera_init(ClvCamera& cam, V3 look_from, V3 look_at, V3 up, float vfov, float aspect, float aperture,
                 float focus) {  // camera.rs:59-99
  cam.lens_radius = aperture / 2.0f;
  const float theta = vfov * kPi / 180.0f;
  const float hh = std::tan(theta / 2.0f);
  const float hw = aspect * hh;
  const V3 origin = look_from;
  const V3 w = unit(look_from - look_at);
  const V3 u = unit(cross(up, w));
  const V3 v = unit(cross(w, u));
  const V3 llc = origin - (hw * focus) * u - (hh * focus) * v - focus * w;
  const V3 hor = (2.0f * hw * focus) * u;
  const V3 ver = (2.0f * hh * focus) * v;
  auto put = [](float* d, V3 a) { d[0] = a.x; d[1] = a.y; d[2] = a.z; };
  put(cam.llc, llc);
  put(cam.horizontal, hor);
  put(cam.vertical, ver);
  put(cam.origin, origin);
  put(cam.u, u);
  put(cam.v, v);
  put(cam.w, w);
}

}  // namespace

HostScene load_scene_text(const std::string& text, uint32_t width, uint32_t height, const std::string& base_dir,
                          bool lam) {
  if (width == 0 || height == 0) throw std::runtime_error("width and height must be positive");
  const Value root = clv_json::parse(text);
  HostScene S;
  S.width = width;
  S.height = height;
  Builder B(S);
  B.base_dir = base_dir;
  S.time_0 = root.at("time_0").as_f32("time_0");
  S.time_1 = root.at("time_1").as_f32("time_1");
  // background: Srgb -> Xyz(D65) -> Xyz<E> (scenefile.rs:43-44)
  float bg[3];
  rgb_of(root.at("background_color"), bg, "background_color");
  srgb_to_xyz_e(bg, S.background_xyz);
  S.background_spd = B.add_spd(S.background_xyz);
  const Value& cam = root.at("camera");
  camera_init(S.camera, vec3_of(cam.at("look_from"), "look_from"), vec3_of(cam.at("look_at"), "look_at"),
              vec3_of(cam.at("up"), "up"), cam.at("vertical_fov").as_f32("vertical_fov"),
              (float)width / (float)height, cam.at("aperture").as_f32("aperture"),
              cam.at("focus_distance").as_f32("focus_distance"));
  if (const Value* mats = root.find("materials")) {
    if (!mats->is_array()) throw std::runtime_error("`materials` must be an array");
    for (auto& m : mats->arr) {
      const uint32_t id = B.material(m);
      B.shared.emplace_back(m.at("name").as_string("name"), id);
    }
  }
  B.fallback = B.default_material();
  B.shared.emplace_back(std::string(), B.fallback);

  // scenefile.rs:62-103: flatten one level of lists, collect priority objects
  std::vector<Emitted> tops, prio;
  for (auto& o : root.at("objects").arr) {
    const bool p = o.has("priority") && o.at("priority").as_bool("priority");
    Emitted e = B.object(o);
    if (e.is_list) {
      for (auto& it : e.items) {
        if (it.is_list) throw std::runtime_error("Recursing too hard in scene initialization");
        if (p) prio.push_back(it);
        tops.push_back(it);
      }
    } else {
      if (p) prio.push_back(e);
      tops.push_back(e);
    }
  }
  if (tops.empty()) throw std::runtime_error("the scene has no objects");
  if (prio.empty())
    throw std::runtime_error("the scene has no priority objects (the reference's MIS BVH build panics)");
  for (size_t i = 0; i < tops.size(); ++i) set_gid(S, tops[i].ref, (uint32_t)i);
  S.object_count = tops.size();
  flatten_main(S, tops, lam);  // scenefile.rs:106-108: both trees with the same algorithm
  flatten_mis(S, prio, lam);
  return S;
}

HostScene load_scene_json(const std::string& path, uint32_t width, uint32_t height, bool lam) {
  std::ifstream f(path);
  if (!f) throw std::runtime_error("cannot open scene file `" + path + "`");
  std::stringstream ss;
  ss << f.rdbuf();
  const size_t slash = path.find_last_of('/');
  return load_scene_text(ss.str(), width, height, slash == std::string::npos ? std::string(".") : path.substr(0, slash),
                         lam);
}

HostScene mesh_scene(const float* verts, uint32_t nverts, const uint32_t* idx, uint32_t ntris) {
  if (ntris == 0) throw std::runtime_error("the mesh has no triangles");
  HostScene S;
  Builder B(S);
  const float black[3] = {0, 0, 0};
  S.background_spd = B.add_spd(black);
  const uint32_t mat = B.default_material();
  std::vector<Emitted> tops;
  tops.reserve(ntris);
  S.tris.reserve(ntris);
  for (uint32_t i = 0; i < ntris; ++i) {
    const uint32_t ia = idx[3 * (size_t)i], ib = idx[3 * (size_t)i + 1], ic = idx[3 * (size_t)i + 2];
    if (ia >= nverts || ib >= nverts || ic >= nverts) throw std::runtime_error("vertex index out of range");
    const V3 a(verts[3 * (size_t)ia], verts[3 * (size_t)ia + 1], verts[3 * (size_t)ia + 2]);
    const V3 b(verts[3 * (size_t)ib], verts[3 * (size_t)ib + 1], verts[3 * (size_t)ib + 2]);
    const V3 c(verts[3 * (size_t)ic], verts[3 * (size_t)ic + 1], verts[3 * (size_t)ic + 2]);
    const V3 corners[3] = {a, b, c};
    tops.push_back(B.planar(a, b - a, c - a, mat, true, true, corners));
    S.tri_gid.back() = i;
  }
  S.object_count = ntris;
  flatten_main(S, tops);
  return S;
}

}  // namespace clv
