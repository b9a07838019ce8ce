// Device-side hot path of the clovers renderer on GB300 (sm_103a).
//
// Everything here follows the reference's f32 operation order (the file is
// compiled with -fmad=false, so no multiply-add is fused) so that ray casts
// return bit-identical hit ids and distances:
//   * AABB::hit (reciprocal slabs) and AABB::distance (true divisions),
//     clovers/src/aabb.rs:54-86 and 135-155;
//   * BVHNode::hit's visiting order, clovers/src/bvh/hitable_trait.rs:15-81:
//     own box first, both children's entry distances, nearer child first
//     (left on ties), far child skipped when the near subtree's hit is closer
//     than the far box's entry distance, the far child's hit preferred on
//     equal distance;
//   * Sphere/Quad/Triangle::hit, clovers/src/objects/{sphere,quad,triangle}.rs.
// The recursion of the reference becomes an explicit per-thread stack whose
// entries hold the deferred far child, its entry distance, its slab interval
// (for its own-box test when it is popped) and the hit count at push time
// (to know whether the near subtree produced a hit).
#pragma once

#include <cuda_runtime.h>
#include <math_constants.h>
#include <stdint.h>

#include "clv_log.h"
#include "device_types.h"
#include "rng.cuh"

namespace clvd {

#define CLV_PI 3.14159265358979323846f
#define CLV_EPS_ACNE 0.001f
#define CLV_EPS_RECT 0.0001f
#define CLV_EPS_MEDIUM 0.0001f
#define CLV_FLT_MAX 3.40282347e+38f
#define CLV_DEG2RAD (3.14159265358979323846f / 180.0f)
#define CLV_STACK 64       // traversal stack entries in local memory (deeper trees spill: SpillStack)
#define CLV_MIS_STACK 32   // MIS tree evaluation stack
#define CLV_NEST 6         // wrapper nesting depth handled by the object interpreter
#ifndef CLV_MINB
#define CLV_MINB 8         // resident blocks per SM asked of the wavefront intersect (64 registers)
#endif
#ifndef CLV_MINB_MEDIUM
#define CLV_MINB_MEDIUM CLV_MINB  // the same for its variant with media and object lists
#endif
#ifndef CLV_MINB_CHAIN
#define CLV_MINB_CHAIN 7   // the same for its wrapper-chain variant (72 registers; 6 and 8 slower on the box)
#endif

// Device error flags (bitwise OR into a status word the host reads).
#define CLV_ERR_STACK 1u
#define CLV_ERR_NEST 2u
#define CLV_ERR_MIS 4u

// ------------------------------------------------------------------ vec3 --
struct V {
  float x, y, z;
};
__device__ __forceinline__ V mk(float x, float y, float z) { return V{x, y, z}; }
__device__ __forceinline__ V add(V a, V b) { return mk(a.x + b.x, a.y + b.y, a.z + b.z); }
__device__ __forceinline__ V sub(V a, V b) { return mk(a.x - b.x, a.y - b.y, a.z - b.z); }
__device__ __forceinline__ V neg(V a) { return mk(-a.x, -a.y, -a.z); }
__device__ __forceinline__ V scl(float s, V a) { return mk(s * a.x, s * a.y, s * a.z); }
// a / d for the slab divisions of AABB::distance, given inv = RN(1/d).
// q0 = RN(a*inv); the residual a - q0*d is exact with an FMA and one
// correction step q0 + residual*inv rounds to the correctly rounded quotient
// (Markstein's theorem; Muller et al., Handbook of Floating-Point Arithmetic,
// ch. 8) provided nothing overflows or underflows.  The traversal uses the
// unguarded form only when that is guaranteed for every box of the scene and
// the ray (see RayPre::fast); otherwise it divides.
__device__ __forceinline__ float div_fast(float a, float d, float inv) {
  const float q0 = a * inv;
  const float r = __fmaf_rn(-q0, d, a);
  return __fmaf_rn(r, inv, q0);
}
// the guarded form, valid for any operands (used by the self-test)
__device__ __forceinline__ float div_rn(float a, float d, float inv) {
  const float q0 = a * inv;
  const float aq = fabsf(q0);
  if (aq >= 8.67361738e-19f && aq <= 1.15292150e18f) {  // 2^-60 .. 2^60
    const float r = __fmaf_rn(-q0, d, a);
    return __fmaf_rn(r, inv, q0);
  }
  return a / d;
}

__device__ __forceinline__ V dvs(V a, float s) { return mk(a.x / s, a.y / s, a.z / s); }
__device__ __forceinline__ float dot(V a, V b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
__device__ __forceinline__ V cross(V a, V b) {
  return mk(a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x);
}
__device__ __forceinline__ float nsq(V a) { return dot(a, a); }
__device__ __forceinline__ float len(V a) { return sqrtf(nsq(a)); }
__device__ __forceinline__ V unit(V a) { return dvs(a, len(a)); }
__device__ __forceinline__ float comp(V a, int i) { return i == 0 ? a.x : (i == 1 ? a.y : a.z); }
__device__ __forceinline__ V ld3(const float* p) { return mk(p[0], p[1], p[2]); }
__device__ __forceinline__ float rclamp(float x, float lo, float hi) { return x < lo ? lo : (x > hi ? hi : x); }

struct Ray {
  V o, d;
  float time;
  int lambda;
};
__device__ __forceinline__ V at(const Ray& r, float t) { return add(r.o, scl(t, r.d)); }

// ------------------------------------------------------------------- rng --
// mix64 and Rng: rng.cuh
#define CLV_REJECT 64
// Marsaglia 1972 point on the sphere (rand_distr UnitSphere)
__device__ V random_unit_vector(Rng& r) {
  for (int i = 0; i < CLV_REJECT; ++i) {
    float x1 = r.sym(), x2 = r.sym();
    float s = x1 * x1 + x2 * x2;
    if (s >= 1.0f) continue;
    float f = 2.0f * sqrtf(1.0f - s);
    return unit(mk(x1 * f, x2 * f, 1.0f - 2.0f * s));
  }
  return mk(0.0f, 0.0f, 1.0f);
}
// rejection sampling in the unit disc (rand_distr UnitDisc)
__device__ void random_in_unit_disk(Rng& r, float& ox, float& oy) {
  for (int i = 0; i < CLV_REJECT; ++i) {
    float x1 = r.sym(), x2 = r.sym();
    if (x1 * x1 + x2 * x2 <= 1.0f) { ox = x1; oy = x2; return; }
  }
  ox = 0.0f; oy = 0.0f;
}
__device__ V random_cosine_direction(Rng& r) {  // clovers/src/random.rs:25-36
  float r1 = r.f32();
  float r2 = r.f32();
  float z = sqrtf(1.0f - r2);
  float phi = 2.0f * CLV_PI * r1;
  float x = cosf(phi) * sqrtf(r2);
  float y = sinf(phi) * sqrtf(r2);
  return mk(x, y, z);
}
__device__ __forceinline__ int random_wavelength(Rng& r) {  // uniform integer in [380, 780)
  return 380 + (int)(((uint64_t)r.u32() * 400ull) >> 32);
}

// ------------------------------------------------------------------ boxes --
// Slab interval of AABB::hit for one box: the ray is inside for t in (N, F).
__device__ __forceinline__ void slab(const float* b, V o, V inv, float& N, float& F) {
  float n = -CLV_FLT_MAX * 2.0f, f = CLV_FLT_MAX * 2.0f;  // -inf / +inf
#pragma unroll
  for (int a = 0; a < 3; ++a) {
    float t0 = (b[2 * a] - comp(o, a)) * comp(inv, a);
    float t1 = (b[2 * a + 1] - comp(o, a)) * comp(inv, a);
    float nn, ff;
    if (t0 < t1) { nn = t0; ff = t1; } else { nn = t1; ff = t0; }
    n = fmaxf(n, nn);  // NaN entries are skipped, as the reference's comparisons do
    f = fminf(f, ff);
  }
  N = n;
  F = f;
}
__device__ __forceinline__ bool slab_pass(float N, float F, float tmin, float tmax) {
  return fminf(tmax, F) > fmaxf(tmin, N);
}
// AABB::distance: entry distance or false (None)
__device__ __forceinline__ bool box_distance(const float* b, V o, V d, float& out) {
  float tx1 = (b[0] - o.x) / d.x, tx2 = (b[1] - o.x) / d.x;
  float tmin = fminf(tx1, tx2), tmax = fmaxf(tx1, tx2);
  float ty1 = (b[2] - o.y) / d.y, ty2 = (b[3] - o.y) / d.y;
  tmin = fmaxf(tmin, fminf(ty1, ty2));
  tmax = fminf(tmax, fmaxf(ty1, ty2));
  float tz1 = (b[4] - o.z) / d.z, tz2 = (b[5] - o.z) / d.z;
  tmin = fmaxf(tmin, fminf(tz1, tz2));
  tmax = fminf(tmax, fmaxf(tz1, tz2));
  out = tmin;
  return tmax >= tmin && tmax > 0.0f;
}

// ------------------------------------------------------------- primitives --
// Full hit record (clovers/src/hitrecord.rs:7-33) plus the material id.
struct Rec {
  float t, u, v;
  V p, n;
  bool front;
  uint32_t mat;
};

__device__ __forceinline__ void load_planar(const ClvPlanar* arr, uint32_t i, float f[16]) {
  const float4* p = reinterpret_cast<const float4*>(arr + i);
  float4 a = __ldg(p), b = __ldg(p + 1), c = __ldg(p + 2), e = __ldg(p + 3);
  f[0] = a.x; f[1] = a.y; f[2] = a.z; f[3] = a.w;
  f[4] = b.x; f[5] = b.y; f[6] = b.z; f[7] = b.w;
  f[8] = c.x; f[9] = c.y; f[10] = c.z; f[11] = c.w;
  f[12] = e.x; f[13] = e.y; f[14] = e.z; f[15] = e.w;
}
// Quad::hit / Triangle::hit up to the inside test: distance t and plane coordinates.
__device__ __forceinline__ bool planar_test(const float f[16], bool tri, const Ray& r, float tmin, float tmax,
                                            float& t, float& alpha, float& beta) {
  V q = mk(f[0], f[1], f[2]), u = mk(f[3], f[4], f[5]), v = mk(f[6], f[7], f[8]);
  V n = mk(f[9], f[10], f[11]), w = mk(f[13], f[14], f[15]);
  float d = f[12];
  float denom = dot(n, r.d);
  if (fabsf(denom) < CLV_EPS_RECT) return false;
  t = (-d - dot(n, r.o)) / denom;
  if (t < tmin || t > tmax) return false;
  V ph = sub(at(r, t), q);
  alpha = dot(w, cross(ph, v));
  beta = dot(w, cross(u, ph));
  bool in = (alpha >= 0.0f && alpha <= 1.0f) && (beta >= 0.0f && beta <= 1.0f);
  if (tri) in = in && (alpha + beta <= 1.0f);
  return in;
}
// Watertight ray/triangle test (Woop, Benthin & Wald 2013, "Watertight
// Ray/Triangle Intersection", JCGT 2(1)): edge functions in a ray-aligned
// shear frame, redone in double when one is exactly 0, so a ray through a
// shared edge or vertex hits at least one of the triangles that share it.
// Two-sided like Triangle::hit, t in [tmin, tmax]; alpha / beta are the
// barycentric weights of the second and third vertex (Triangle::hit's plane
// coordinates along u and v).  Not the reference's test: used only in scenes
// loaded with CLV_OPT_WATERTIGHT.
__device__ __forceinline__ bool tri_watertight(const float4* vtx, const Ray& r, float tmin, float tmax, float& t,
                                               float& alpha, float& beta) {
  const float4 p0 = __ldg(vtx), p1 = __ldg(vtx + 1), p2 = __ldg(vtx + 2);
  const float ax = fabsf(r.d.x), ay = fabsf(r.d.y), az = fabsf(r.d.z);
  const int kz = ax > ay ? (ax > az ? 0 : 2) : (ay > az ? 1 : 2);
  int kx = kz == 2 ? 0 : kz + 1, ky = kx == 2 ? 0 : kx + 1;
  const float dz = comp(r.d, kz);
  if (dz < 0.0f) {  // keep the winding
    const int tmp = kx;
    kx = ky;
    ky = tmp;
  }
  const float sx = comp(r.d, kx) / dz, sy = comp(r.d, ky) / dz, sz = 1.0f / dz;
  const V A = sub(mk(p0.x, p0.y, p0.z), r.o), B = sub(mk(p1.x, p1.y, p1.z), r.o), C = sub(mk(p2.x, p2.y, p2.z), r.o);
  const float Ax = comp(A, kx) - sx * comp(A, kz), Ay = comp(A, ky) - sy * comp(A, kz);
  const float Bx = comp(B, kx) - sx * comp(B, kz), By = comp(B, ky) - sy * comp(B, kz);
  const float Cx = comp(C, kx) - sx * comp(C, kz), Cy = comp(C, ky) - sy * comp(C, kz);
  float U = Cx * By - Cy * Bx, W1 = Ax * Cy - Ay * Cx, W2 = Bx * Ay - By * Ax;
  if (U == 0.0f || W1 == 0.0f || W2 == 0.0f) {
    U = (float)((double)Cx * (double)By - (double)Cy * (double)Bx);
    W1 = (float)((double)Ax * (double)Cy - (double)Ay * (double)Cx);
    W2 = (float)((double)Bx * (double)Ay - (double)By * (double)Ax);
  }
  if ((U < 0.0f || W1 < 0.0f || W2 < 0.0f) && (U > 0.0f || W1 > 0.0f || W2 > 0.0f)) return false;
  const float det = U + W1 + W2;
  if (det == 0.0f) return false;
  const float T = U * (sz * comp(A, kz)) + W1 * (sz * comp(B, kz)) + W2 * (sz * comp(C, kz));
  t = T / det;
  if (!(t >= tmin && t <= tmax)) return false;
  alpha = W1 / det;
  beta = W2 / det;
  return true;
}
// Watertight mode of a traversal: CLV_WT_OFF / CLV_WT_ON fixed at compile
// time (the ray-cast and single-scene intersect kernels), CLV_WT_SCENE read
// from the scene (batches, the megakernel, the object interpreter, MIS pdfs).
#define CLV_WT_OFF 0
#define CLV_WT_ON 1
#define CLV_WT_SCENE 2
template <int WT>
__device__ __forceinline__ bool wt_on(const ClvDeviceScene& S) {
  return WT == CLV_WT_SCENE ? S.watertight != 0 : WT == CLV_WT_ON;
}
// A triangle or quad of the scene: its plane record in f and the hit test of
// the scene's triangle mode.
template <int WT = CLV_WT_SCENE>
__device__ __forceinline__ bool planar_hit(const ClvDeviceScene& S, bool tri, uint32_t idx, float f[16], const Ray& r,
                                           float tmin, float tmax, float& t, float& alpha, float& beta) {
  load_planar(tri ? S.tris : S.quads, idx, f);
  if (tri && wt_on<WT>(S))
    return tri_watertight(reinterpret_cast<const float4*>(S.tri_verts) + 3 * (size_t)idx, r, tmin, tmax, t, alpha, beta);
  return planar_test(f, tri, r, tmin, tmax, t, alpha, beta);
}
__device__ __forceinline__ void face(Rec& rec, const Ray& r, V outward) {
  rec.front = dot(r.d, outward) < 0.0f;
  rec.n = rec.front ? outward : neg(outward);
}
__device__ __forceinline__ void planar_record(const float f[16], const Ray& r, float t, float alpha, float beta,
                                              Rec& rec) {
  rec.t = t;
  rec.p = at(r, t);
  rec.u = alpha;
  rec.v = beta;
  face(rec, r, mk(f[9], f[10], f[11]));
}
// Sphere::hit: roots strictly inside (tmin, tmax)
__device__ __forceinline__ bool sphere_test(float4 s, const Ray& r, float tmin, float tmax, float& t) {
  V c = mk(s.x, s.y, s.z);
  V oc = sub(r.o, c);
  float a = nsq(r.d);
  float hb = dot(oc, r.d);
  float cc = nsq(oc) - s.w * s.w;
  float disc = hb * hb - a * cc;
  if (!(disc > 0.0f)) return false;
  float root = sqrtf(disc);
  float d0 = (-hb - root) / a;
  if (d0 < tmax && d0 > tmin) { t = d0; return true; }
  float d1 = (-hb + root) / a;
  if (d1 < tmax && d1 > tmin) { t = d1; return true; }
  return false;
}
__device__ __forceinline__ void sphere_record(V c, float radius, const Ray& r, float t, Rec& rec) {
  rec.t = t;
  rec.p = at(r, t);
  V outward = unit(dvs(sub(rec.p, c), radius));
  V tr = dvs(sub(rec.p, c), radius);  // get_uv, sphere.rs:58-65
  float phi = atan2f(tr.z, tr.x);
  float theta = asinf(tr.y);
  rec.u = 1.0f - (phi + CLV_PI) / (2.0f * CLV_PI);
  rec.v = (theta + CLV_PI / 2.0f) / CLV_PI;
  face(rec, r, outward);
}
__device__ __forceinline__ float4 load_sphere(const ClvDeviceScene& S, uint32_t i) {
  return __ldg(reinterpret_cast<const float4*>(S.spheres) + i);
}

// ----------------------------------------------- compound object interpreter --
// Evaluates any ref (primitive or ClvObj) into a full record, recursing
// through wrappers up to CLV_NEST levels (host validates the nesting).
struct Counters {
  uint32_t nodes, prims;
};

template <int LEVEL>
struct ObjEval {
  static __device__ bool hit(const ClvDeviceScene& S, uint32_t ref, const Ray& r, float tmin, float tmax, Rng* rng,
                             Rec& rec, Counters* cnt, uint32_t* err);
  static __device__ float pdf(const ClvDeviceScene& S, uint32_t ref, V origin, V dir, int lambda, float time);
};
template <>
struct ObjEval<CLV_NEST> {
  static __device__ bool hit(const ClvDeviceScene&, uint32_t, const Ray&, float, float, Rng*, Rec&, Counters*,
                             uint32_t* err) {
    if (err) atomicOr(err, CLV_ERR_NEST);
    return false;
  }
  static __device__ float pdf(const ClvDeviceScene&, uint32_t, V, V, int, float) { return 0.0f; }
};

template <int LEVEL>
__device__ __noinline__ bool ObjEval<LEVEL>::hit(const ClvDeviceScene& S, uint32_t ref, const Ray& r, float tmin, float tmax,
                                    Rng* rng, Rec& rec, Counters* cnt, uint32_t* err) {
  const uint32_t kind = CLV_REF_KIND(ref), idx = CLV_REF_INDEX(ref);
  if (kind == CLV_REF_TRI || kind == CLV_REF_QUAD) {
    if (cnt) cnt->prims++;
    float f[16], t, a, b;
    if (!planar_hit(S, kind == CLV_REF_TRI, idx, f, r, tmin, tmax, t, a, b)) return false;
    planar_record(f, r, t, a, b, rec);
    rec.mat = kind == CLV_REF_TRI ? S.tri_mat[idx] : S.quad_mat[idx];
    return true;
  }
  if (kind == CLV_REF_SPHERE) {
    if (cnt) cnt->prims++;
    float4 s = load_sphere(S, idx);
    float t;
    if (!sphere_test(s, r, tmin, tmax, t)) return false;
    sphere_record(mk(s.x, s.y, s.z), s.w, r, t, rec);
    rec.mat = S.sphere_mat[idx];
    return true;
  }
  if (kind != CLV_REF_OBJ) return false;
  const ClvObj& o = S.objs[idx];
  switch (o.kind) {
    case CLV_OBJ_BOXY: {  // boxy.rs:76-94: closest of 6 quads, tmax narrowing
      bool any = false;
      float closest = tmax;
      for (int k = 0; k < 6; ++k) {
        Rec h;
        if (ObjEval<LEVEL + 1>::hit(S, CLV_MAKE_REF(CLV_REF_QUAD, o.a + k), r, tmin, closest, rng, h, cnt, err)) {
          closest = h.t;
          rec = h;
          any = true;
        }
      }
      return any;
    }
    case CLV_OBJ_LIST: {  // hitable.rs:148-166: None as soon as one member misses
      float best = CLV_FLT_MAX * 2.0f;
      bool any = false;
      for (uint32_t k = 0; k < o.b; ++k) {
        Rec h;
        if (!ObjEval<LEVEL + 1>::hit(S, S.obj_children[o.a + k], r, tmin, tmax, rng, h, cnt, err)) return false;
        if (h.t < best) {
          best = h.t;
          rec = h;
          any = true;
        }
      }
      return any;
    }
    case CLV_OBJ_TRANSLATE: {  // translate.rs:41-78
      V off = mk(o.p[0], o.p[1], o.p[2]);
      Ray moved{sub(r.o, off), r.d, r.time, r.lambda};
      Rec h;
      if (!ObjEval<LEVEL + 1>::hit(S, o.a, moved, tmin, tmax, rng, h, cnt, err)) return false;
      rec = h;
      rec.p = add(h.p, off);
      face(rec, moved, h.n);
      return true;
    }
    case CLV_OBJ_ROTATEY: {  // rotate.rs:82-159
      float s = o.p[0], c = o.p[1];
      V ro = r.o, rd = r.d;
      ro.x = c * r.o.x - s * r.o.z;
      ro.z = s * r.o.x + c * r.o.z;
      rd.x = c * r.d.x - s * r.d.z;
      rd.z = s * r.d.x + c * r.d.z;
      Ray rr{ro, unit(rd), r.time, r.lambda};
      Rec h;
      if (!ObjEval<LEVEL + 1>::hit(S, o.a, rr, tmin, tmax, rng, h, cnt, err)) return false;
      V p = h.p, n = h.n;
      p.x = c * h.p.x + s * h.p.z;
      p.z = -s * h.p.x + c * h.p.z;
      n.x = c * h.n.x + s * h.n.z;
      n.z = -s * h.n.x + c * h.n.z;
      rec = h;
      rec.p = p;
      face(rec, rr, unit(n));
      return true;
    }
    case CLV_OBJ_MEDIUM: {  // constant_medium.rs:65-126
      Rec r1, r2;
      const float inf = CLV_FLT_MAX * 2.0f;
      if (!ObjEval<LEVEL + 1>::hit(S, o.a, r, -inf, inf, rng, r1, cnt, err)) return false;
      if (!ObjEval<LEVEL + 1>::hit(S, o.a, r, r1.t + CLV_EPS_MEDIUM, inf, rng, r2, cnt, err)) return false;
      if (r1.t < tmin) r1.t = tmin;
      if (r2.t > tmax) r2.t = tmax;
      if (r1.t >= r2.t) return false;
      if (r1.t < 0.0f) r1.t = 0.0f;
      float rl = len(r.d);
      float inside = (r2.t - r1.t) * rl;
      // the project's own f32 log: the same bits as the CPU oracle's (clv_log.h)
      float hd = o.p[0] * clv_math::log_f32(rng->f32());
      if (hd > inside) return false;
      rec.t = r1.t + hd / rl;
      rec.p = at(r, rec.t);
      rec.n = random_unit_vector(*rng);
      rec.front = true;
      rec.u = r1.u;
      rec.v = r1.v;
      rec.mat = o.b;
      return true;
    }
    case CLV_OBJ_MOVING: {  // moving_sphere.rs:104-160
      if (cnt) cnt->prims++;
      V c0 = mk(o.p[0], o.p[1], o.p[2]), c1 = mk(o.p[3], o.p[4], o.p[5]);
      float t0 = o.p[6], t1 = o.p[7], radius = o.p[8];
      V c = add(c0, scl((r.time - t0) / (t1 - t0), sub(c1, c0)));
      float t;
      if (!sphere_test(make_float4(c.x, c.y, c.z, radius), r, tmin, tmax, t)) return false;
      sphere_record(c, radius, r, t, rec);
      rec.mat = o.b;
      return true;
    }
  }
  return false;
}

// Flat evaluator for the common compound shape: a chain of Translate /
// RotateY wrappers (up to CLV_CHAIN levels) over a Boxy, quad, triangle,
// sphere or moving sphere.  It walks down transforming the ray exactly as the
// wrappers' hit() do (translate.rs:41-78, rotate.rs:82-159), tests the
// terminal, then walks back up applying each wrapper's record transform and
// set_face_normal with that level's ray direction (recomputed from the top,
// which keeps the loop's state small).  Returns 0 miss, 1 hit, 2 not handled
// here (media, lists, deeper chains).
#define CLV_CHAIN 4
#define CLV_PRAGMA_S(x) _Pragma(#x)
#define CLV_PRAGMA(x) CLV_PRAGMA_S(x)
#ifndef CLV_BOXY_UNROLL
#define CLV_BOXY_UNROLL 1  // unroll factor of a Boxy leaf's loop over its quads
#endif
__device__ __forceinline__ V chain_dir(const ClvDeviceScene& S, uint32_t ref, V d, int upto) {
  // direction of the ray as seen below level `upto` (inclusive)
  for (int j = 0; j <= upto; ++j) {
    const ClvObj& o = S.objs[CLV_REF_INDEX(ref)];
    if (o.kind == CLV_OBJ_ROTATEY) {
      const float sn = o.p[0], cs = o.p[1];
      V rd = d;
      rd.x = cs * d.x - sn * d.z;
      rd.z = sn * d.x + cs * d.z;
      d = unit(rd);
    }
    ref = o.a;
  }
  return d;
}
// The ray below a chain's wrappers: Translate moves the origin, RotateY
// rotates origin and direction and renormalises the direction (rotate.rs:104-
// 126).  Returns false for chains the inline form does not take (too deep, or
// ending in a list or a medium); otherwise r, the terminal ref and the number
// of wrappers n.
__device__ __forceinline__ bool chain_walk(const ClvDeviceScene& S, uint32_t top, const Ray& r0, Ray& r,
                                           uint32_t& ref, int& n) {
  n = 0;
  r = r0;
  ref = top;
  while (CLV_REF_KIND(ref) == CLV_REF_OBJ) {
    const ClvObj& o = S.objs[CLV_REF_INDEX(ref)];
    if (o.kind == CLV_OBJ_TRANSLATE) {
      if (n == CLV_CHAIN) return false;
      r.o = sub(r.o, mk(o.p[0], o.p[1], o.p[2]));
    } else if (o.kind == CLV_OBJ_ROTATEY) {
      if (n == CLV_CHAIN) return false;
      const float sn = o.p[0], cs = o.p[1];
      V ro = r.o, rd = r.d;
      ro.x = cs * r.o.x - sn * r.o.z;
      ro.z = sn * r.o.x + cs * r.o.z;
      rd.x = cs * r.d.x - sn * r.d.z;
      rd.z = sn * r.d.x + cs * r.d.z;
      r.o = ro;
      r.d = unit(rd);
    } else if (o.kind == CLV_OBJ_BOXY || o.kind == CLV_OBJ_MOVING) {
      break;
    } else {
      return false;
    }
    ++n;
    ref = o.a;
  }
  return true;
}
// The record of a hit below n wrappers brought back to the frame of `top`:
// the wrappers' inverse transforms from the innermost out, each setting the
// face against the ray direction as seen at its level.
__device__ __forceinline__ void chain_unwind(const ClvDeviceScene& S, uint32_t top, const Ray& r0, int n, Rec& rec);
template <int WT = CLV_WT_SCENE>
__device__ __forceinline__ int chain_hit(const ClvDeviceScene& S, uint32_t top, const Ray& r0, float tmin, float tmax,
                                         Rec& rec, Counters* cnt) {
  int n;
  Ray r;
  uint32_t ref;
  if (!chain_walk(S, top, r0, r, ref, n)) return 2;
  // terminal
  const uint32_t kind = CLV_REF_KIND(ref), idx = CLV_REF_INDEX(ref);
  bool any = false;
  if (kind == CLV_REF_OBJ) {
    const ClvObj& o = S.objs[idx];
    if (o.kind == CLV_OBJ_BOXY) {  // closest of its 6 quads (boxy.rs:76-94)
      float closest = tmax;
      CLV_PRAGMA(unroll CLV_BOXY_UNROLL)
      for (int k = 0; k < 6; ++k) {
        if (cnt) cnt->prims++;
        float f[16], t, a, b;
        load_planar(S.quads, o.a + k, f);
        if (planar_test(f, false, r, tmin, closest, t, a, b)) {
          planar_record(f, r, t, a, b, rec);
          rec.mat = S.quad_mat[o.a + k];
          closest = t;
          any = true;
        }
      }
    } else {  // MovingSphere (moving_sphere.rs:104-160)
      if (cnt) cnt->prims++;
      const V c0 = mk(o.p[0], o.p[1], o.p[2]), c1 = mk(o.p[3], o.p[4], o.p[5]);
      const V c = add(c0, scl((r.time - o.p[6]) / (o.p[7] - o.p[6]), sub(c1, c0)));
      float t;
      if (sphere_test(make_float4(c.x, c.y, c.z, o.p[8]), r, tmin, tmax, t)) {
        sphere_record(c, o.p[8], r, t, rec);
        rec.mat = o.b;
        any = true;
      }
    }
  } else if (kind == CLV_REF_TRI || kind == CLV_REF_QUAD) {
    if (cnt) cnt->prims++;
    float f[16], t, a, b;
    if (planar_hit<WT>(S, kind == CLV_REF_TRI, idx, f, r, tmin, tmax, t, a, b)) {
      planar_record(f, r, t, a, b, rec);
      rec.mat = kind == CLV_REF_TRI ? S.tri_mat[idx] : S.quad_mat[idx];
      any = true;
    }
  } else if (kind == CLV_REF_SPHERE) {
    if (cnt) cnt->prims++;
    const float4 sp = load_sphere(S, idx);
    float t;
    if (sphere_test(sp, r, tmin, tmax, t)) {
      sphere_record(mk(sp.x, sp.y, sp.z), sp.w, r, t, rec);
      rec.mat = S.sphere_mat[idx];
      any = true;
    }
  } else {
    return 2;
  }
  if (!any) return 0;
  chain_unwind(S, top, r0, n, rec);
  return 1;
}
__device__ __forceinline__ void chain_unwind(const ClvDeviceScene& S, uint32_t top, const Ray& r0, int n, Rec& rec) {
  for (int l = n - 1; l >= 0; --l) {
    uint32_t wr = top;
    for (int j = 0; j < l; ++j) wr = S.objs[CLV_REF_INDEX(wr)].a;
    const ClvObj& o = S.objs[CLV_REF_INDEX(wr)];
    if (o.kind == CLV_OBJ_TRANSLATE) {
      rec.p = add(rec.p, mk(o.p[0], o.p[1], o.p[2]));
      const V d = l == 0 ? r0.d : chain_dir(S, top, r0.d, l - 1);
      const V nn = rec.n;
      rec.front = dot(d, nn) < 0.0f;
      rec.n = rec.front ? nn : neg(nn);
    } else {
      const float sn = o.p[0], cs = o.p[1];
      V p = rec.p, nn = rec.n;
      p.x = cs * rec.p.x + sn * rec.p.z;
      p.z = -sn * rec.p.x + cs * rec.p.z;
      nn.x = cs * rec.n.x + sn * rec.n.z;
      nn.z = -sn * rec.n.x + cs * rec.n.z;
      rec.p = p;
      const V un = unit(nn);
      const V d = chain_dir(S, top, r0.d, l);
      rec.front = dot(d, un) < 0.0f;
      rec.n = rec.front ? un : neg(un);
    }
  }
}

// A compound BVH leaf, out of line so the traversal loop stays small.
__device__ __noinline__ bool compound_leaf(const ClvDeviceScene& S, uint32_t ref, const Ray& r, float tmin,
                                           float tmax, Rng* rng, Rec& rec, Counters* cnt, uint32_t* err) {
  const int c = chain_hit(S, ref, r, tmin, tmax, rec, cnt);
  if (c != 2) return c == 1;
  return ObjEval<0>::hit(S, ref, r, tmin, tmax, rng, rec, cnt, err);
}

// pdf_value of one MIS leaf object (HitableTrait::pdf_value of each type).
__device__ __forceinline__ float planar_pdf(const ClvDeviceScene& S, bool tri, uint32_t idx, V origin, V dir) {
  float f[16], t, a, b;
  Ray r{origin, dir, 0.0f, 0};
  if (!planar_hit(S, tri, idx, f, r, CLV_EPS_ACNE, CLV_FLT_MAX * 2.0f, t, a, b)) return 0.0f;
  Rec rec;
  planar_record(f, r, t, a, b, rec);
  float dist2 = t * t * nsq(dir);
  float cosine = fabsf(dot(dir, rec.n)) / len(dir);
  return dist2 / (cosine * (tri ? S.tri_area[idx] : S.quad_area[idx]));
}
__device__ __forceinline__ float sphere_pdf(float4 s, V origin, V dir) {
  Ray r{origin, dir, 0.0f, 0};
  float t;
  if (!sphere_test(s, r, CLV_EPS_ACNE, CLV_FLT_MAX * 2.0f, t)) return 0.0f;
  V c = mk(s.x, s.y, s.z);
  float ctm = sqrtf(1.0f - s.w * s.w / nsq(sub(c, origin)));
  float sa = 2.0f * CLV_PI * (1.0f - ctm);
  return 1.0f / sa;
}
template <int LEVEL>
__device__ __noinline__ float ObjEval<LEVEL>::pdf(const ClvDeviceScene& S, uint32_t ref, V origin, V dir, int lambda, float time) {
  const uint32_t kind = CLV_REF_KIND(ref), idx = CLV_REF_INDEX(ref);
  if (kind == CLV_REF_TRI || kind == CLV_REF_QUAD) return planar_pdf(S, kind == CLV_REF_TRI, idx, origin, dir);
  if (kind == CLV_REF_SPHERE) return sphere_pdf(load_sphere(S, idx), origin, dir);
  if (kind != CLV_REF_OBJ) return 0.0f;
  const ClvObj& o = S.objs[idx];
  switch (o.kind) {
    case CLV_OBJ_BOXY: {  // boxy.rs:113-128
      float sum = 0.0f;
      for (int k = 0; k < 6; ++k) sum += planar_pdf(S, false, o.a + k, origin, dir) / 6.0f;
      return sum;
    }
    case CLV_OBJ_TRANSLATE:  // translate.rs:81-98 (adds the offset)
      return ObjEval<LEVEL + 1>::pdf(S, o.a, add(origin, mk(o.p[0], o.p[1], o.p[2])), dir, lambda, time);
    case CLV_OBJ_MEDIUM:
      return ObjEval<LEVEL + 1>::pdf(S, o.a, origin, dir, lambda, time);
    default:  // RotateY, MovingSphere, HitableList: 0
      return 0.0f;
  }
}

// ------------------------------------------------------------- traversal --
// Closest-hit state.  For triangles/quads/spheres only (t, ref, u, v) are kept
// and the full record is rebuilt afterwards (deterministic); compound objects
// write their full record to `full` since media consume randomness.
struct Hit {
  float t;
  uint32_t ref;  // leaf ref that produced the hit, CLV_REF_EMPTY if none
  float a, b;    // plane coordinates (triangle / quad)
};

// Per-ray constants of the traversal.  `fast` holds when the scene's box
// coordinates and the ray origin are each 0 or of magnitude in [2^-70, 2^59]
// and the direction components have magnitude in [2^-60, 2]: then every
// a = box - origin is 0 or of magnitude in [2^-93, 2^60], every quotient a/d
// is 0 or normal and finite, and div_fast equals a / d exactly.
struct RayPre {
  V o, d, inv;
  bool fast;
};
__device__ __forceinline__ bool coord_ok(float x) {
  const float a = fabsf(x);
  return x == 0.0f || (a >= 8.47032947e-22f && a <= 5.76460752e17f);  // 2^-70 .. 2^59
}
__device__ __forceinline__ bool dir_ok(float x) {
  const float a = fabsf(x);
  return a >= 8.67361738e-19f && a <= 2.0f;  // 2^-60 .. 2
}
__device__ __forceinline__ float divc(const RayPre& R, float a, int axis) {
  const float d = comp(R.d, axis), inv = comp(R.inv, axis);
  return R.fast ? div_fast(a, d, inv) : a / d;
}
// Exit distance of a box widened by 4 gamma_3 (gamma_n = n u / (1 - n u),
// u = 2^-24) toward +infinity, the conservative box test of Ize 2013
// ("Robust BVH Ray Traversal", JCGT 2(2)) that keeps watertight triangles
// from being culled with their boxes.  Watertight scenes only.
__device__ __forceinline__ float widen_exit(float f) { return fmaxf(f, f + fabsf(f) * 7.1525574e-7f); }
// The box tests of watertight scenes: the exit distance widened, and a zero
// direction component constraining nothing while the origin lies within that
// slab (inclusive) and missing otherwise, where the reference's forms compute
// 0 * inf = NaN and reject a ray that runs along a box face.
__device__ __forceinline__ void slab_wide(const float* b, const RayPre& R, float& N, float& F) {
  float n = -CLV_FLT_MAX * 2.0f, f = CLV_FLT_MAX * 2.0f;
#pragma unroll
  for (int a = 0; a < 3; ++a) {
    const float o = comp(R.o, a);
    if (comp(R.d, a) == 0.0f) {
      if (o < b[2 * a] || o > b[2 * a + 1]) f = -CLV_FLT_MAX * 2.0f;
      continue;
    }
    const float t0 = (b[2 * a] - o) * comp(R.inv, a), t1 = (b[2 * a + 1] - o) * comp(R.inv, a);
    n = fmaxf(n, fminf(t0, t1));
    f = fminf(f, fmaxf(t0, t1));
  }
  N = n;
  F = widen_exit(f);
}
__device__ __forceinline__ bool box_distance_wide(const float* b, const RayPre& R, float& out) {
  float tmin = -CLV_FLT_MAX * 2.0f, tmax = CLV_FLT_MAX * 2.0f;
#pragma unroll
  for (int a = 0; a < 3; ++a) {
    const float o = comp(R.o, a);
    if (comp(R.d, a) == 0.0f) {
      if (o < b[2 * a] || o > b[2 * a + 1]) return false;
      continue;
    }
    const float t1 = divc(R, b[2 * a] - o, a), t2 = divc(R, b[2 * a + 1] - o, a);
    tmin = fmaxf(tmin, fminf(t1, t2));
    tmax = fminf(tmax, fmaxf(t1, t2));
  }
  out = tmin;
  tmax = widen_exit(tmax);
  return tmax >= tmin && tmax > 0.0f;
}
// AABB::distance with div_rn
__device__ __forceinline__ bool box_distance_pre(const float* b, const RayPre& R, float& out) {
  float tx1 = divc(R, b[0] - R.o.x, 0), tx2 = divc(R, b[1] - R.o.x, 0);
  float tmin = fminf(tx1, tx2), tmax = fmaxf(tx1, tx2);
  float ty1 = divc(R, b[2] - R.o.y, 1), ty2 = divc(R, b[3] - R.o.y, 1);
  tmin = fmaxf(tmin, fminf(ty1, ty2));
  tmax = fminf(tmax, fmaxf(ty1, ty2));
  float tz1 = divc(R, b[4] - R.o.z, 2), tz2 = divc(R, b[5] - R.o.z, 2);
  tmin = fmaxf(tmin, fminf(tz1, tz2));
  tmax = fminf(tmax, fmaxf(tz1, tz2));
  out = tmin;
  return tmax >= tmin && tmax > 0.0f;
}

// Tests one BVH leaf with the current tmax.  CPLX: 0 primitives only,
// 1 + wrapper chains (inline), 2 + media and lists (out-of-line interpreter).
template <int CPLX, int WT>
__device__ __forceinline__ bool leaf_test(const ClvDeviceScene& S, uint32_t ref, const Ray& r, float tmin,
                                          float tmax, Rng* rng, Hit& hit, Rec* full, Counters* cnt, uint32_t* err) {
  const uint32_t kind = CLV_REF_KIND(ref), idx = CLV_REF_INDEX(ref);
  if (kind == CLV_REF_TRI || kind == CLV_REF_QUAD) {
    if (cnt) cnt->prims++;
    float f[16], t, a, b;
    if (!planar_hit<WT>(S, kind == CLV_REF_TRI, idx, f, r, tmin, tmax, t, a, b)) return false;
    hit.t = t;
    hit.ref = ref;
    hit.a = a;
    hit.b = b;
    return true;
  }
  if (kind == CLV_REF_SPHERE) {
    if (cnt) cnt->prims++;
    float t;
    if (!sphere_test(load_sphere(S, idx), r, tmin, tmax, t)) return false;
    hit.t = t;
    hit.ref = ref;
    return true;
  }
  if (CPLX == 1) {
    Rec rec;
    const int c = chain_hit<WT>(S, ref, r, tmin, tmax, rec, cnt);
    if (c == 2 && err) atomicOr(err, CLV_ERR_NEST);  // host routes such scenes to CPLX 2
    if (c != 1) return false;
    hit.t = rec.t;
    hit.ref = ref;
    if (full) *full = rec;
    return true;
  }
  if (CPLX == 2) {
    Rec rec;
    if (!compound_leaf(S, ref, r, tmin, tmax, rng, rec, cnt, err)) return false;
    hit.t = rec.t;
    hit.ref = ref;
    if (full) *full = rec;
    return true;
  }
  return false;
}

// BVHNode::hit over the flattened tree, one "call" (node or leaf) per step so
// that warps reconverge every step.
//
// Stack entries are the deferred far children of the nodes on the current
// path (ref, entry distance, slab interval).  Whether a node's near subtree
// produced a hit is tracked without per-entry counters: every entry on the
// stack belongs to an ancestor whose near subtree is being traversed, so when
// a hit is accepted all current entries are marked, which keeps the marked
// entries a prefix [0, marked) of the stack.
// Traversal stacks.  A plain per-thread array (local memory, L1-cached), or a
// hybrid whose first SH entries sit in shared memory (one column per thread
// of a 128-thread block) and whose deeper entries spill to local memory.
__device__ __forceinline__ void st_put(float4* s, int i, float4 v) { s[i] = v; }
__device__ __forceinline__ float4 st_get(float4* s, int i) { return s[i]; }
template <int SH>
struct HybridStack {
  float4* sh;   // this thread's column: entry k at sh[k * 128]
  float4* loc;  // entries SH.. in local memory
};
template <int SH>
__device__ __forceinline__ void st_put(HybridStack<SH>& s, int i, float4 v) {
  if (i < SH) s.sh[i * 128] = v;
  else s.loc[i - SH] = v;
}
template <int SH>
__device__ __forceinline__ float4 st_get(HybridStack<SH>& s, int i) {
  return i < SH ? s.sh[i * 128] : s.loc[i - SH];
}
// Stack for trees deeper than CLV_STACK levels: the first CLV_STACK entries in
// local memory, the rest in a global spill region where entry k of thread t
// sits at region[(k - CLV_STACK) * stride + t] (the threads of a warp side by
// side).  cap = entries available (the scene's tree depth needs at most
// depth - 1: one deferred far child per level of the current path).
struct SpillStack {
  float4* loc;
  float4* glob;     // region + t
  uint32_t stride;  // threads that share the region
  int cap;
};
__device__ __forceinline__ void st_put(SpillStack& s, int i, float4 v) {
  if (i < CLV_STACK) s.loc[i] = v;
  else s.glob[(size_t)(i - CLV_STACK) * s.stride] = v;
}
__device__ __forceinline__ float4 st_get(SpillStack& s, int i) {
  return i < CLV_STACK ? s.loc[i] : s.glob[(size_t)(i - CLV_STACK) * s.stride];
}
// Entries a stack holds.
__device__ __forceinline__ int st_cap(float4*) { return CLV_STACK; }
template <int SH>
__device__ __forceinline__ int st_cap(HybridStack<SH>&) { return CLV_STACK; }
__device__ __forceinline__ int st_cap(SpillStack& s) { return s.cap; }

// Three-input f32 max / min (NaN inputs ignored, as fmaxf / fminf do).
__device__ __forceinline__ float max3f(float a, float b, float c) {
  float d;
  asm("max.f32 %0, %1, %2, %3;" : "=f"(d) : "f"(a), "f"(b), "f"(c));
  return d;
}
__device__ __forceinline__ float min3f(float a, float b, float c) {
  float d;
  asm("min.f32 %0, %1, %2, %3;" : "=f"(d) : "f"(a), "f"(b), "f"(c));
  return d;
}
// Both tests the traversal makes of one child box, from one set of
// differences d = bound - origin (the same f32 values that AABB::distance and
// AABB::hit each compute): the slab interval (N, F) of the child's own
// AABB::hit, made when the child is visited, and its entry distance
// (AABB::distance, the quotients d / direction).  FAST: RayPre::fast holds
// (quotients by div_fast), else IEEE division.
template <bool FAST>
__device__ __forceinline__ bool child_tests(const float* b, const RayPre& R, float& dist, float& N, float& F) {
  float d[6];
#pragma unroll
  for (int a = 0; a < 3; ++a) {
    d[2 * a] = b[2 * a] - comp(R.o, a);
    d[2 * a + 1] = b[2 * a + 1] - comp(R.o, a);
  }
  if (FAST) {
    // Under RayPre::fast every difference is finite and every reciprocal finite
    // and non-zero, so no slab value or quotient is NaN: the reference's
    // compare-and-swap ordering and its chained fmin/fmax reduce to plain
    // min / max (equal up to the sign of a zero, and the results feed only
    // comparisons).
    float t[6], q[6];
#pragma unroll
    for (int k = 0; k < 6; ++k) {
      const int a = k >> 1;
      t[k] = d[k] * comp(R.inv, a);
      q[k] = div_fast(d[k], comp(R.d, a), comp(R.inv, a));
    }
    N = max3f(fminf(t[0], t[1]), fminf(t[2], t[3]), fminf(t[4], t[5]));
    F = min3f(fmaxf(t[0], t[1]), fmaxf(t[2], t[3]), fmaxf(t[4], t[5]));
    const float tmin = max3f(fminf(q[0], q[1]), fminf(q[2], q[3]), fminf(q[4], q[5]));
    const float tmax = min3f(fmaxf(q[0], q[1]), fmaxf(q[2], q[3]), fmaxf(q[4], q[5]));
    dist = tmin;
    return tmax >= tmin && tmax > 0.0f;
  }
  float n = -CLV_FLT_MAX * 2.0f, f = CLV_FLT_MAX * 2.0f;
#pragma unroll
  for (int a = 0; a < 3; ++a) {
    const float t0 = d[2 * a] * comp(R.inv, a), t1 = d[2 * a + 1] * comp(R.inv, a);
    float nn, ff;
    if (t0 < t1) { nn = t0; ff = t1; } else { nn = t1; ff = t0; }
    n = fmaxf(n, nn);
    f = fminf(f, ff);
  }
  N = n;
  F = f;
  float q[6];
#pragma unroll
  for (int k = 0; k < 6; ++k) {
    const int a = k >> 1;
    q[k] = d[k] / comp(R.d, a);
  }
  const float tx1 = q[0], tx2 = q[1];
  float tmin = fminf(tx1, tx2), tmax = fmaxf(tx1, tx2);
  const float ty1 = q[2], ty2 = q[3];
  tmin = fmaxf(tmin, fminf(ty1, ty2));
  tmax = fminf(tmax, fmaxf(ty1, ty2));
  const float tz1 = q[4], tz2 = q[5];
  tmin = fmaxf(tmin, fminf(tz1, tz2));
  tmax = fminf(tmax, fmaxf(tz1, tz2));
  dist = tmin;
  return tmax >= tmin && tmax > 0.0f;
}

// The scalar state (kept in registers); the stack array lives apart from it
// because an indexed array forces its enclosing object into local memory.
struct Trav {
  RayPre R;
  float tmin, tmax;
  int sp, marked;
  uint32_t ref;
  float N, F;
  bool found;
};
template <int WT>
__device__ __forceinline__ void trav_begin(const ClvDeviceScene& S, const Ray& r, float tmin, float tmax, Trav& T,
                                           Hit& hit) {
  hit.ref = CLV_REF_EMPTY;
  hit.t = 0.0f;
  T.R.o = r.o;
  T.R.d = r.d;
  T.R.inv = mk(1.0f / r.d.x, 1.0f / r.d.y, 1.0f / r.d.z);
  T.R.fast = S.boxes_div_safe && dir_ok(r.d.x) && dir_ok(r.d.y) && dir_ok(r.d.z) && coord_ok(r.o.x) &&
             coord_ok(r.o.y) && coord_ok(r.o.z);
  T.tmin = tmin;
  T.tmax = tmax;
  T.sp = 0;
  T.marked = 0;
  T.ref = S.root;
  if (wt_on<WT>(S)) slab_wide(S.root_box, T.R, T.N, T.F);
  else slab(S.root_box, r.o, T.R.inv, T.N, T.F);
  T.found = false;
}
// One node visit or leaf test, then the next reference (descend, or pop the
// next deferred far child whose visit the reference would make).  Returns
// false when the traversal is over (result in hit / T.found).
template <int CPLX, int WT, class STK>
__device__ __forceinline__ bool trav_step(const ClvDeviceScene& S, const Ray& r, Trav& T, STK& stack, Rng* rng,
                                          Hit& hit, Rec* full, Counters* cnt, uint32_t* err) {
  const RayPre& R = T.R;
  uint32_t ref = T.ref;
  if (CLV_REF_KIND(ref) == CLV_REF_NODE) {
    if (cnt) cnt->nodes++;
    if (slab_pass(T.N, T.F, T.tmin, T.tmax)) {
      const float4* p4 = reinterpret_cast<const float4*>(S.nodes + CLV_REF_INDEX(ref));
      const float4 q0 = __ldg(p4), q1 = __ldg(p4 + 1), q2 = __ldg(p4 + 2), q3 = __ldg(p4 + 3);
      const float lb[6] = {q0.x, q0.y, q0.z, q0.w, q1.x, q1.y};
      const float rb[6] = {q1.z, q1.w, q2.x, q2.y, q2.z, q2.w};
      const uint32_t L = __float_as_uint(q3.x), Rr = __float_as_uint(q3.y);
      uint32_t next = CLV_REF_EMPTY;
      bool left_next = true;
      if (!wt_on<WT>(S)) {
        float ld, rd, NL, FL, NR, FR;
        bool lh, rh;
        if (R.fast) {  // one branch per node on the division form
          lh = child_tests<true>(lb, R, ld, NL, FL);
          rh = child_tests<true>(rb, R, rd, NR, FR);
        } else {
          lh = child_tests<false>(lb, R, ld, NL, FL);
          rh = child_tests<false>(rb, R, rd, NR, FR);
        }
        const bool both = L != CLV_REF_EMPTY && Rr != CLV_REF_EMPTY;
        if (both && lh && rh) {
          left_next = ld < rd;
          next = left_next ? L : Rr;
          if (T.sp < st_cap(stack)) {
            st_put(stack, T.sp++, make_float4(__uint_as_float(left_next ? Rr : L), fmaxf(ld, rd), left_next ? NR : NL,
                                              left_next ? FR : FL));
          } else if (err) {
            atomicOr(err, CLV_ERR_STACK);
          }
        } else if (both ? lh : L != CLV_REF_EMPTY) {
          next = L;
        } else if (both ? rh : Rr != CLV_REF_EMPTY) {
          next = Rr;
          left_next = false;
        }
        if (next != CLV_REF_EMPTY) {
          T.N = left_next ? NL : NR;
          T.F = left_next ? FL : FR;
          T.ref = next;
          return true;
        }
      } else if (L != CLV_REF_EMPTY && Rr != CLV_REF_EMPTY) {
        float ld, rd;
        const bool wide = wt_on<WT>(S);
        const bool lh = wide ? box_distance_wide(lb, R, ld) : box_distance_pre(lb, R, ld);
        const bool rh = wide ? box_distance_wide(rb, R, rd) : box_distance_pre(rb, R, rd);
        if (lh && rh) {
          left_next = ld < rd;
          next = left_next ? L : Rr;
          const uint32_t far = left_next ? Rr : L;
          float fN = 0.0f, fF = 0.0f;
          if (CLV_REF_KIND(far) == CLV_REF_NODE) {
            float fb[6];
#pragma unroll
            for (int k = 0; k < 6; ++k) fb[k] = left_next ? rb[k] : lb[k];
            if (wide) slab_wide(fb, R, fN, fF);
            else slab(fb, r.o, R.inv, fN, fF);
          }
          if (T.sp < st_cap(stack)) {
            st_put(stack, T.sp++, make_float4(__uint_as_float(far), fmaxf(ld, rd), fN, fF));
          } else if (err) {
            atomicOr(err, CLV_ERR_STACK);
          }
        } else if (lh) {
          next = L;
        } else if (rh) {
          next = Rr;
          left_next = false;
        }
      } else if (L != CLV_REF_EMPTY) {
        next = L;
      } else if (Rr != CLV_REF_EMPTY) {
        next = Rr;
        left_next = false;
      }
      if (next != CLV_REF_EMPTY) {
        if (CLV_REF_KIND(next) == CLV_REF_NODE) {
          float nb[6];
#pragma unroll
          for (int k = 0; k < 6; ++k) nb[k] = left_next ? lb[k] : rb[k];
          if (wt_on<WT>(S)) slab_wide(nb, R, T.N, T.F);
          else slab(nb, r.o, R.inv, T.N, T.F);
        }
        T.ref = next;
        return true;
      }
    }
  } else {
    if (leaf_test<CPLX, WT>(S, ref, r, T.tmin, T.tmax, rng, hit, full, cnt, err)) {
      T.tmax = hit.t;
      T.found = true;
      T.marked = T.sp;
    }
  }
  // pop the next deferred far child whose visit the reference would make
  while (T.sp > 0) {
    --T.sp;
    const float4 e = st_get(stack, T.sp);
    const bool near_hit = T.sp < T.marked;
    if (T.marked > T.sp) T.marked = T.sp;
    if (near_hit && hit.t < e.y) continue;  // near subtree's hit is closer than the far box
    T.ref = __float_as_uint(e.x);
    T.N = e.z;
    T.F = e.w;
    return true;
  }
  return false;
}
// closest_hit with a caller-provided stack (a local array or a HybridStack)
template <int CPLX, int WT, class STK>
__device__ __forceinline__ bool closest_hit_stk(const ClvDeviceScene& S, const Ray& r, float tmin, float tmax, Rng* rng,
                                                Hit& hit, Rec* full, Counters* cnt, uint32_t* err, STK& stack) {
  Trav T;
  trav_begin<WT>(S, r, tmin, tmax, T, hit);
  while (trav_step<CPLX, WT>(S, r, T, stack, rng, hit, full, cnt, err)) {
  }
  return T.found;
}
template <int CPLX, int WT = CLV_WT_SCENE>
__device__ bool closest_hit(const ClvDeviceScene& S, const Ray& r, float tmin, float tmax, Rng* rng, Hit& hit,
                            Rec* full, Counters* cnt, uint32_t* err) {
  float4 stack_mem[CLV_STACK];
  float4* stack = stack_mem;
  return closest_hit_stk<CPLX, WT>(S, r, tmin, tmax, rng, hit, full, cnt, err, stack);
}

// closest_hit for the 32 lanes of a warp together (every lane calls it; `go`
// is false for lanes without a ray).  Each turn, the warp chooses which of its
// traversing lanes take their next step; the others wait.  A wrapper-chain
// leaf (CPLX 1 and 2) costs several primitive tests and transforms, so a lane
// whose next step is one waits until every traversing lane of the warp is at
// one, and the leaf then runs once for all of them.  Every lane
// still makes exactly closest_hit's sequence of node visits and leaf tests,
// only later in time, so hits and counts are unchanged.
template <int CPLX, int WT, class STK>
__device__ __forceinline__ bool closest_hit_warp(const ClvDeviceScene& S, const Ray& r, bool go, float tmin, float tmax,
                                                 Rng* rng, Hit& hit, Rec* full, Counters* cnt, uint32_t* err,
                                                 STK& stack) {
  Trav T;
  T.found = false;
  T.ref = CLV_REF_EMPTY;
  bool active = go;
  if (go) trav_begin<WT>(S, r, tmin, tmax, T, hit);
  for (;;) {
    const unsigned act = __ballot_sync(0xFFFFFFFFu, active);
    if (act == 0u) break;
    const bool at_chain = active && CLV_REF_KIND(T.ref) == CLV_REF_OBJ;
    const unsigned chains = __ballot_sync(0xFFFFFFFFu, at_chain);
    if (active && (!at_chain || chains == act)) active = trav_step<CPLX, WT>(S, r, T, stack, rng, hit, full, cnt, err);
  }
  return go && T.found;
}
template <int CPLX, int WT>
__device__ __forceinline__ bool closest_hit_warp(const ClvDeviceScene& S, const Ray& r, bool go, float tmin, float tmax,
                                                 Rng* rng, Hit& hit, Rec* full, Counters* cnt, uint32_t* err) {
  float4 stack_mem[CLV_STACK];
  float4* stack = stack_mem;
  return closest_hit_warp<CPLX, WT>(S, r, go, tmin, tmax, rng, hit, full, cnt, err, stack);
}

// Full record of the closest hit (deterministic rebuild for primitives).
__device__ __forceinline__ void hit_record(const ClvDeviceScene& S, const Ray& r, const Hit& h, const Rec& full,
                                           Rec& rec) {
  const uint32_t kind = CLV_REF_KIND(h.ref), idx = CLV_REF_INDEX(h.ref);
  if (kind == CLV_REF_TRI || kind == CLV_REF_QUAD) {
    float f[16];
    load_planar(kind == CLV_REF_TRI ? S.tris : S.quads, idx, f);
    planar_record(f, r, h.t, h.a, h.b, rec);
    rec.mat = kind == CLV_REF_TRI ? S.tri_mat[idx] : S.quad_mat[idx];
  } else if (kind == CLV_REF_SPHERE) {
    float4 s = load_sphere(S, idx);
    sphere_record(mk(s.x, s.y, s.z), s.w, r, h.t, rec);
    rec.mat = S.sphere_mat[idx];
  } else {
    rec = full;
  }
}
__device__ __forceinline__ uint32_t hit_gid(const ClvDeviceScene& S, uint32_t ref) {
  const uint32_t kind = CLV_REF_KIND(ref), idx = CLV_REF_INDEX(ref);
  switch (kind) {
    case CLV_REF_TRI: return S.tri_gid[idx];
    case CLV_REF_QUAD: return S.quad_gid[idx];
    case CLV_REF_SPHERE: return S.sphere_gid[idx];
    case CLV_REF_OBJ: return S.obj_gid[idx];
  }
  return 0xFFFFFFFFu;
}

// ------------------------------------------------------ MIS (priority) tree --
// BVHNode::pdf_value (bvh/hitable_trait.rs:89-111): midpoint of both children
// (f32::midpoint = f64 sum halved, rounded once), single child passed through.
__device__ float mis_pdf(const ClvDeviceScene& S, V origin, V dir, int lambda, float time, uint32_t* err) {
  struct Frame {
    uint32_t node;
    uint32_t stage;  // 0 start, 1 left evaluated
    float lval;
  };
  Frame st[CLV_MIS_STACK];
  int sp = 0;
  uint32_t ref = S.mis_root;
  float val = 0.0f;
  while (true) {
    // descend from `ref` until a leaf value is produced
    while (CLV_REF_KIND(ref) == CLV_REF_NODE && ref != CLV_REF_EMPTY) {
      const ClvMisNode n = S.mis_nodes[CLV_REF_INDEX(ref)];
      if (n.right == CLV_REF_EMPTY) { ref = n.left; continue; }
      if (n.left == CLV_REF_EMPTY) { ref = n.right; continue; }
      if (sp >= CLV_MIS_STACK) {
        if (err) atomicOr(err, CLV_ERR_MIS);
        return 0.0f;
      }
      st[sp++] = Frame{CLV_REF_INDEX(ref), 0u, 0.0f};
      ref = n.left;
    }
    if (ref == CLV_REF_EMPTY) {
      val = 0.0f;
    } else {
      const uint32_t k = CLV_REF_KIND(ref);
      if (k == CLV_REF_TRI || k == CLV_REF_QUAD) val = planar_pdf(S, k == CLV_REF_TRI, CLV_REF_INDEX(ref), origin, dir);
      else if (k == CLV_REF_SPHERE) val = sphere_pdf(load_sphere(S, CLV_REF_INDEX(ref)), origin, dir);
      else val = ObjEval<0>::pdf(S, ref, origin, dir, lambda, time);
    }
    // ascend: combine finished values
    while (true) {
      if (sp == 0) return val;
      Frame& f = st[sp - 1];
      if (f.stage == 0) {
        f.stage = 1;
        f.lval = val;
        ref = S.mis_nodes[f.node].right;
        break;
      }
      val = (float)(((double)f.lval + (double)val) / 2.0);
      --sp;
    }
  }
}
// leaf random(): Sphere (sphere.rs:160-187), Quad (quad.rs:166-172), Triangle (triangle.rs:203-220)
__device__ V leaf_random(const ClvDeviceScene& S, uint32_t ref, V origin, Rng& rng) {
  const uint32_t kind = CLV_REF_KIND(ref), idx = CLV_REF_INDEX(ref);
  if (kind == CLV_REF_SPHERE) {
    float4 s = load_sphere(S, idx);
    V offset = sub(mk(s.x, s.y, s.z), origin);
    float d2 = nsq(offset);
    V w = unit(offset);
    V a = fabsf(w.x) > 0.9f ? unit(mk(0.0f, 1.0f, 0.0f)) : unit(mk(1.0f, 0.0f, 0.0f));
    V vv = unit(cross(w, a));
    V uu = unit(cross(w, vv));
    float r1 = rng.f32();
    float r2 = rng.f32();
    float z = 1.0f + r2 * (sqrtf(1.0f - s.w * s.w / d2) - 1.0f);
    float phi = 2.0f * CLV_PI * r1;
    float x = cosf(phi) * sqrtf(1.0f - z * z);
    float y = sinf(phi) * sqrtf(1.0f - z * z);
    V l = unit(mk(x, y, z));
    return unit(add(add(scl(l.x, uu), scl(l.y, vv)), scl(l.z, w)));
  }
  float f[16];
  load_planar(kind == CLV_REF_TRI ? S.tris : S.quads, idx, f);
  V q = mk(f[0], f[1], f[2]), u = mk(f[3], f[4], f[5]), v = mk(f[6], f[7], f[8]);
  if (kind == CLV_REF_QUAD) {
    float a = rng.f32();
    V pa = add(q, scl(a, u));
    float b = rng.f32();
    return sub(add(pa, scl(b, v)), origin);
  }
  float a = rng.f32(), b = rng.f32();
  if (a + b > 1.0f) { a = 1.0f - a; b = 1.0f - b; }
  return sub(add(add(q, scl(a, u)), scl(b, v)), origin);
}
// BVHNode::random (hitable_trait.rs:115-127): coin flips down to a leaf
__device__ V mis_random(const ClvDeviceScene& S, V origin, Rng& rng) {
  uint32_t ref = S.mis_root;
  for (int guard = 0; guard < 4096 && CLV_REF_KIND(ref) == CLV_REF_NODE && ref != CLV_REF_EMPTY; ++guard) {
    const ClvMisNode n = S.mis_nodes[CLV_REF_INDEX(ref)];
    if (n.right == CLV_REF_EMPTY) ref = n.left;
    else if (n.left == CLV_REF_EMPTY) ref = n.right;
    else ref = rng.boolean() ? n.left : n.right;
  }
  return leaf_random(S, ref, origin, rng);
}

// -------------------------------------------------------------- materials --
__device__ __forceinline__ float spd_get(const ClvDeviceScene& S, uint32_t table, int lambda) {
  return __ldg(S.spd + (size_t)table * 400 + (lambda - 380));
}
__device__ __forceinline__ float tex_color(const ClvDeviceScene& S, const ClvMaterial& m, int lambda, const Rec& rec) {
  switch (m.tex_kind) {
    case CLV_TEX_SOLID: return spd_get(S, m.spd_even, lambda);
    case CLV_TEX_SPATIAL: {
      float d = m.density * CLV_PI;
      float s = 1.0f * sinf(d * rec.p.x) * sinf(d * rec.p.y) * sinf(d * rec.p.z);
      return spd_get(S, s < 0.0f ? m.spd_odd : m.spd_even, lambda);
    }
    case CLV_TEX_SURFACE: {
      float d = m.density * CLV_PI;
      float s = 1.0f * sinf(d * rec.u) * sinf(d * rec.v);
      return spd_get(S, s < 0.0f ? m.spd_odd : m.spd_even, lambda);
    }
    default:
      return rclamp(__ldg(S.illuminant + (size_t)m.illuminant * 400 + (lambda - 380)) * m.intensity, 0.0f, 1.0f);
  }
}
__device__ __forceinline__ float tex_emit(const ClvDeviceScene& S, const ClvMaterial& m, int lambda, const Rec& rec) {
  if (m.tex_kind == CLV_TEX_ILLUMINANT)
    return __ldg(S.illuminant + (size_t)m.illuminant * 400 + (lambda - 380)) * m.intensity;
  return tex_color(S, m, lambda, rec);  // non-illuminant textures emit their colour, unclamped
}
// Material::emit (diffuse_light.rs:41-53, cone_light.rs:43-66)
__device__ __forceinline__ float mat_emit(const ClvDeviceScene& S, const ClvMaterial& m, const Ray& r, int lambda,
                                          const Rec& rec) {
  if (m.kind == CLV_MAT_DIFFUSELIGHT) {
    if (!rec.front) return 0.0f;
    return tex_emit(S, m, lambda, rec);
  }
  if (m.kind == CLV_MAT_CONELIGHT) {
    if (!rec.front) return 0.0f;
    float spread = m.spread * CLV_DEG2RAD;
    float angle = acosf(-dot(r.d, rec.n) / (len(r.d) * len(rec.n)));
    if (angle > spread) return 0.0f;
    return tex_emit(S, m, lambda, rec);
  }
  return 0.0f;
}
// Material::color with the optional thin-film factor (materials.rs:95-102, thin_film.rs:31-54)
__device__ __forceinline__ float mat_color(const ClvDeviceScene& S, const ClvMaterial& m, const Ray& r, int lambda,
                                           const Rec& rec) {
  float tf = 1.0f;
  if (m.thin_film) {
    float n_ratio = 1.0f / m.tf_ior;
    float c1 = -dot(r.d, rec.n);
    float s1 = sqrtf(1.0f - c1 * c1);
    float s2 = n_ratio * s1;
    float c2 = sqrtf(1.0f - (s2 * s2));
    float opd = 2.0f * m.tf_ior * m.tf_thickness * c2;
    float mm = opd / (float)lambda;
    tf = 1.0f + cosf(mm * 2.0f * CLV_PI);
  }
  float k;
  switch (m.kind) {
    case CLV_MAT_DIELECTRIC: k = spd_get(S, m.spd_even, lambda); break;
    case CLV_MAT_DISPERSIVE: k = 1.0f; break;
    case CLV_MAT_CONELIGHT:
    case CLV_MAT_DIFFUSELIGHT: k = rclamp(tex_color(S, m, lambda, rec), 0.0f, 1.0f); break;
    default: k = tex_color(S, m, lambda, rec); break;
  }
  return k * tf;
}
__device__ __forceinline__ V reflect(V v, V n) { return unit(sub(v, scl(2.0f * dot(v, n), n))); }
__device__ __forceinline__ V refract(V v, V n, float ratio) {
  float ct = fminf(-dot(v, n), 1.0f);
  V par = scl(ratio, add(v, scl(ct, n)));
  V perp = scl(-sqrtf(1.0f - nsq(par)), n);
  return unit(add(par, perp));
}
__device__ __forceinline__ float schlick(float cosine, float ri) {
  float r0 = (1.0f - ri) / (1.0f + ri);
  r0 = r0 * r0;
  return r0 + (1.0f - r0) * powf(1.0f - cosine, 5.0f);
}
__device__ __forceinline__ float dispersive_index(const ClvMaterial& m, int lambda) {
  float wm = (float)lambda / 1000.0f;
  if (!m.sellmeier) return m.cauchy_a + (m.cauchy_b / (wm * wm));
  float l2 = wm * wm;  // Sellmeier: n^2 = 1 + sum B_i l^2 / (l^2 - C_i)
  float s = 1.0f;
  for (int i = 0; i < 3; ++i) s = s + m.sell_b[i] * l2 / (l2 - m.sell_c[i]);
  return sqrtf(s);
}

}  // namespace clvd
