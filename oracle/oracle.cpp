// CPU ORACLE for the clovers render hot path -- TEST INFRASTRUCTURE ONLY.
//
// This file is a plain C++ restatement of the reference renderer's algorithm
// (Walther/clovers, Rust).  It exists to check the GB300 product; the product
// never links, loads or calls it.  Only tests, the smoke check and the CPU
// baseline leg of bench.py use it.
//
// Fidelity rules:
//  * f32 arithmetic in the reference's operation order; build with
//    -ffp-contract=off (no FMA contraction, which GCC does by default on
//    aarch64) and without -ffast-math.
//  * nalgebra order of evaluation: dot = (x*x' + y*y') + z*z', cross is the
//    textbook form, normalize divides each component by the norm.
//  * Rust f32::min/max -> fminf/fmaxf (NaN-ignoring minNum/maxNum).
//  * f32::midpoint -> computed in f64 and rounded once.
//  * The reference draws randomness from OS-seeded SmallRng streams and is
//    therefore not reproducible; this oracle (and the GPU product) draw from a
//    counter-based stream per (pixel, sample) instead: key = mix(mix(seed) ^
//    (pixel << 32 | sample)), draw k = SplitMix64 output of key + (k+1)*gamma.
//    Distributions match the reference's (rand 0.9 / rand_distr 0.5); the
//    individual numbers cannot (parity of the random streams is unpinned).
//
// Parity status: pinned by the reference's own known-answer tests
// (clovers/src/spectrum.rs:74-101, clovers/src/objects/triangle.rs:262-416,
// clovers/src/aabb.rs:185-282, clovers/src/interval.rs:69-99,
// clovers/tests/wavelength.rs, clovers/tests/spectrum.rs), restated in
// tests/test_oracle_kat.py.  The palette crate (sRGB <-> XYZ, Bradford
// adaptation) and rand_distr's samplers are third-party and unpinned.

#include <algorithm>
#include <atomic>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <fstream>
#include <memory>
#include <sstream>
#include <stdexcept>
#include <string>
#include <thread>
#include <vector>

#include "../clovers_gb300/csrc/clv_log.h"
#include "../clovers_gb300/csrc/json.hpp"
#include "../clovers_gb300/csrc/spectral_tables.h"

namespace orc {

#ifdef ORC_DOUBLE
// The quality reference: the same algorithm with Float = f64, the reference's
// own precision switch (clovers/src/lib.rs:97-98).  Scene values still come in
// as f32 (the scene the GPU renders), then every operation runs in double.
typedef double Float;
#define FL(x) x
#else
typedef float Float;
#define FL(x) x##f
#endif
static const Float PI = FL(3.14159265358979323846);                 // core::f32::consts::PI
static const Float EPSILON_SHADOW_ACNE = FL(0.001);                 // clovers/src/lib.rs:114
static const Float EPSILON_RECT_THICKNESS = FL(0.0001);             // clovers/src/lib.rs:116
static const Float EPSILON_CONSTANT_MEDIUM = FL(0.0001);            // clovers/src/lib.rs:119
static const Float RADS_PER_DEG = FL(3.14159265358979323846) / FL(180.0);  // f32::to_radians
static const int MIN_WAVELENGTH = 380, MAX_WAVELENGTH = 780, SPECTRUM_SIZE = 400;  // wavelength.rs:14-20
static const int WAVE_SAMPLE_COUNT = 4;                          // wavelength.rs:25

// ---------------------------------------------------------------- vectors --
struct Vec3 {
  Float x, y, z;
  Vec3() : x(0), y(0), z(0) {}
  Vec3(Float a, Float b, Float c) : x(a), y(b), z(c) {}
  Float operator[](int i) const { return i == 0 ? x : (i == 1 ? y : z); }
  Float& operator[](int i) { return i == 0 ? x : (i == 1 ? y : z); }
};
static inline Vec3 operator+(Vec3 a, Vec3 b) { return Vec3(a.x + b.x, a.y + b.y, a.z + b.z); }
static inline Vec3 operator-(Vec3 a, Vec3 b) { return Vec3(a.x - b.x, a.y - b.y, a.z - b.z); }
static inline Vec3 operator-(Vec3 a) { return Vec3(-a.x, -a.y, -a.z); }
static inline Vec3 operator*(Float s, Vec3 a) { return Vec3(s * a.x, s * a.y, s * a.z); }
static inline Vec3 operator*(Vec3 a, Float s) { return Vec3(a.x * s, a.y * s, a.z * s); }
static inline Vec3 operator/(Vec3 a, Float s) { return Vec3(a.x / s, a.y / s, a.z / s); }
static inline Float dot(Vec3 a, Vec3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
static inline Vec3 cross(Vec3 a, Vec3 b) {
  return Vec3(a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x);
}
static inline Float norm_squared(Vec3 a) { return dot(a, a); }
static inline Float norm(Vec3 a) { return std::sqrt(norm_squared(a)); }
static inline Vec3 normalize(Vec3 a) { return a / norm(a); }
static inline Float rmin(Float a, Float b) { return std::fmin(a, b); }
static inline Float rmax(Float a, Float b) { return std::fmax(a, b); }
static inline Float midpoint(Float a, Float b) { return (Float)(((double)a + (double)b) / 2.0); }
// Rust f32::clamp: NaN passes through
static inline Float rclamp(Float x, Float lo, Float hi) { return x < lo ? lo : (x > hi ? hi : x); }
// Natural log of a uniform draw (the free-flight distance of
// constant_medium.rs:102, Rust's ln).  The f32 build uses the project's own
// logarithm (clv_log.h), whose bits the GPU reproduces exactly; the f64 build
// uses the host libm's double log.
#ifdef ORC_DOUBLE
static inline Float ln(Float x) { return std::log(x); }
#else
static inline Float ln(Float x) { return clv_math::log_f32(x); }
#endif

// -------------------------------------------------------------------- rng --
// Counter-based stream (see header).  SplitMix64: Steele, Lea, Flood 2014.
static inline uint64_t mix64(uint64_t z) {
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
  return z ^ (z >> 31);
}
struct Rng {
  uint64_t key;
  uint32_t counter;
  Rng(uint64_t seed, uint32_t pixel, uint32_t sample)
      : key(mix64(mix64(seed) ^ (((uint64_t)pixel << 32) | (uint64_t)sample))), counter(0) {}
  uint32_t next_u32() {
    ++counter;
    return (uint32_t)(mix64(key + (uint64_t)counter * 0x9E3779B97F4A7C15ull) >> 32);
  }
  // rand: Standard f32 = (u32 >> 8) * 2^-24, uniform in [0,1)
  Float next_f32() { return (Float)(next_u32() >> 8) * FL(5.9604644775390625e-8); }
  // rand: Standard bool = sign bit of a u32 draw
  bool next_bool() { return (int32_t)next_u32() < 0; }
  // uniform in [-1, 1)
  Float next_sym() { return FL(2.0) * next_f32() - FL(1.0); }
};
static const int REJECTION_LIMIT = 64;

// rand_distr UnitSphere (Marsaglia 1972), clovers/src/random.rs:11-14
static Vec3 random_unit_vector(Rng& rng) {
  for (int i = 0; i < REJECTION_LIMIT; ++i) {
    Float x1 = rng.next_sym(), x2 = rng.next_sym();
    Float sum = x1 * x1 + x2 * x2;
    if (sum >= FL(1.0)) continue;
    Float factor = FL(2.0) * std::sqrt(FL(1.0) - sum);
    return normalize(Vec3(x1 * factor, x2 * factor, FL(1.0) - FL(2.0) * sum));
  }
  return Vec3(FL(0.0), FL(0.0), FL(1.0));
}
// rand_distr UnitDisc (rejection), clovers/src/random.rs:18-21
static void random_in_unit_disk(Rng& rng, Float& ox, Float& oy) {
  for (int i = 0; i < REJECTION_LIMIT; ++i) {
    Float x1 = rng.next_sym(), x2 = rng.next_sym();
    if (x1 * x1 + x2 * x2 <= FL(1.0)) { ox = x1; oy = x2; return; }
  }
  ox = FL(0.0); oy = FL(0.0);
}
// clovers/src/random.rs:25-36
static Vec3 random_cosine_direction(Rng& rng) {
  Float r1 = rng.next_f32();
  Float r2 = rng.next_f32();
  Float z = std::sqrt(FL(1.0) - r2);
  Float phi = FL(2.0) * PI * r1;
  Float x = std::cos(phi) * std::sqrt(r2);
  Float y = std::sin(phi) * std::sqrt(r2);
  return Vec3(x, y, z);
}
// clovers/src/wavelength.rs:31-35: uniform integer in [380, 780)
static int random_wavelength(Rng& rng) {
  return MIN_WAVELENGTH + (int)(((uint64_t)rng.next_u32() * (uint64_t)SPECTRUM_SIZE) >> 32);
}

// ------------------------------------------------------------- wavelength --
// clovers/src/wavelength.rs:55-60
static void rotate_wavelength(int hero, int out[4]) {
  for (int j = 0; j < WAVE_SAMPLE_COUNT; ++j) {
    int step = j * SPECTRUM_SIZE / WAVE_SAMPLE_COUNT;
    out[j] = MIN_WAVELENGTH + (hero - MIN_WAVELENGTH + step) % SPECTRUM_SIZE;
  }
}
// clovers/src/wavelength.rs:63-66
static Float gaussian(Float x, Float alpha, Float mu, Float s1, Float s2) {
  Float t = (x - mu) / (x < mu ? s1 : s2);
  return alpha * std::exp(-(t * t) / FL(2.0));
}
// clovers/src/wavelength.rs:71-83
static void wavelength_into_xyz(int lambda, Float out[3]) {
  Float l = (Float)lambda;
  Float x = FL(0.0) + gaussian(l, FL(1.056), FL(599.8), FL(37.9), FL(31.0)) + gaussian(l, FL(0.362), FL(442.0), FL(16.0), FL(26.7)) +
            gaussian(l, -FL(0.065), FL(501.1), FL(20.4), FL(26.2));
  Float y = gaussian(l, FL(0.821), FL(568.8), FL(46.9), FL(40.5)) + gaussian(l, FL(0.286), FL(530.9), FL(16.3), FL(31.1));
  Float z = gaussian(l, FL(1.217), FL(437.0), FL(11.8), FL(36.0)) + gaussian(l, FL(0.681), FL(459.0), FL(26.0), FL(13.8));
  out[0] = x; out[1] = y; out[2] = z;
}

// --------------------------------------------------------------- spectrum --
struct SpectralError : std::runtime_error {
  using std::runtime_error::runtime_error;
};
// clovers/src/spectrum/spectrum_grid.rs:16-153 (Meng et al. 2015)
static double spectrum_xyz_to_p(double lambda, const double xyz[3]) {
  using namespace clv_tables;
  double norm_ = 1.0 / (xyz[0] + xyz[1] + xyz[2]);
  if (!(norm_ < 1.7976931348623157e308)) return 0.0;
  double x = xyz[0] * norm_, y = xyz[1] * norm_;
  double uv[2];
  uv[0] = kXyToUv[0] * x + kXyToUv[1] * y + kXyToUv[2];
  uv[1] = kXyToUv[3] * x + kXyToUv[4] * y + kXyToUv[5];
  if (uv[0] < 0.0 || uv[0] >= 12.0 || uv[1] < 0.0 || uv[1] >= 14.0) return 0.0;
  int uvi0 = (int)uv[0], uvi1 = (int)uv[1];
  const GridCell& cell = kGrid[uvi0 + 12 * uvi1];
  int num = cell.num_points;
  if (num == 0) throw SpectralError("colour maps to an empty cell of the spectral grid");
  double p[6];
  double sb = (lambda - 380.0) / (780.0 - 380.0) * (81.0 - 1.0);
  int sb0 = (int)sb;
  int sb1 = sb0 + 1 < 81 ? sb0 + 1 : 80;
  double sbf = sb - (double)sb0;
  for (int i = 0; i < num; ++i) {
    const double* s = kPoints[cell.idx[i]].spectrum;
    p[i] = s[sb0] * (1.0 - sbf) + s[sb1] * sbf;
  }
  double interpolated = 0.0;
  if (cell.inside == 1) {
    uv[0] -= (double)uvi0;
    uv[1] -= (double)uvi1;
    interpolated = p[0] * (1.0 - uv[0]) * (1.0 - uv[1]) + p[2] * (1.0 - uv[0]) * uv[1] + p[3] * uv[0] * uv[1] +
                   p[1] * uv[0] * (1.0 - uv[1]);
  } else {
    const double* o = kPoints[cell.idx[0]].uv;
    double ex = uv[0] - o[0], ey = uv[1] - o[1];
    double e0x = kPoints[cell.idx[1]].uv[0] - o[0];
    double e0y = kPoints[cell.idx[1]].uv[1] - o[1];
    double uu = e0x * ey - ex * e0y;
    for (int i = 0; i < num - 1; ++i) {
      double e1x, e1y;
      if (i == num - 2) {
        e1x = kPoints[cell.idx[1]].uv[0] - o[0];
        e1y = kPoints[cell.idx[1]].uv[1] - o[1];
      } else {
        e1x = kPoints[cell.idx[i + 2]].uv[0] - o[0];
        e1y = kPoints[cell.idx[i + 2]].uv[1] - o[1];
      }
      double vv = ex * e1y - e1x * ey;
      double area = e0x * e1y - e1x * e0y;
      double u = uu / area, v = vv / area;
      double w = 1.0 - u - v;
      if (u < 0.0 || v < 0.0 || w < 0.0) {
        uu = -vv;
        e0x = e1x;
        e0y = e1y;
        continue;
      }
      interpolated = p[0] * w + p[i + 1] * v + p[i == num - 2 ? 1 : i + 2] * u;
      break;
    }
  }
  return interpolated / norm_;
}
// clovers/src/spectrum.rs:46-56
static Float spectral_power(const Float xyz[3], int lambda) {
  double d[3] = {(double)xyz[0], (double)xyz[1], (double)xyz[2]};
  double p = spectrum_xyz_to_p((double)lambda, d) / clv_tables::kEqualEnergyReflectance;
  return (Float)p;
}
// clovers/src/spectrum.rs:19-42
struct SPD {
  std::vector<Float> table;
  SPD() {}
  explicit SPD(const Float xyz[3]) : table(SPECTRUM_SIZE) {
    for (int i = 0; i < SPECTRUM_SIZE; ++i) table[i] = spectral_power(xyz, MIN_WAVELENGTH + i);
  }
  Float get(int lambda) const { return table[lambda - MIN_WAVELENGTH]; }
};

// ------------------------------------------------------------------ color --
// palette 0.7.6 (third-party, parity unpinned): sRGB transfer per IEC
// 61966-2-1, linear sRGB -> XYZ(D65) from the sRGB primaries, Bradford
// adaptation D65 -> E.  The 3x3 product is formed in f64, applied in f64,
// rounded to f32.
static void mat3_mul(const double a[9], const double b[9], double out[9]) {
  for (int r = 0; r < 3; ++r)
    for (int c = 0; c < 3; ++c) out[r * 3 + c] = a[r * 3] * b[c] + a[r * 3 + 1] * b[3 + c] + a[r * 3 + 2] * b[6 + c];
}
static void mat3_inv(const double m[9], double o[9]) {
  double a = m[0], b = m[1], c = m[2], d = m[3], e = m[4], f = m[5], g = m[6], h = m[7], i = m[8];
  double A = e * i - f * h, B = -(d * i - f * g), C = d * h - e * g;
  double det = a * A + b * B + c * C;
  o[0] = A / det; o[1] = -(b * i - c * h) / det; o[2] = (b * f - c * e) / det;
  o[3] = B / det; o[4] = (a * i - c * g) / det; o[5] = -(a * f - c * d) / det;
  o[6] = C / det; o[7] = -(a * h - b * g) / det; o[8] = (a * e - b * d) / det;
}
static void srgb_to_xyz_d65_matrix(double m[9]) {
  const double xr = 0.64, yr = 0.33, xg = 0.30, yg = 0.60, xb = 0.15, yb = 0.06;
  const double W[3] = {0.95047, 1.0, 1.08883};
  double P[9] = {xr / yr, xg / yg, xb / yb, 1.0, 1.0, 1.0, (1 - xr - yr) / yr, (1 - xg - yg) / yg, (1 - xb - yb) / yb};
  double Pi[9];
  mat3_inv(P, Pi);
  double S[3];
  for (int r = 0; r < 3; ++r) S[r] = Pi[r * 3] * W[0] + Pi[r * 3 + 1] * W[1] + Pi[r * 3 + 2] * W[2];
  for (int r = 0; r < 3; ++r)
    for (int c = 0; c < 3; ++c) m[r * 3 + c] = P[r * 3 + c] * S[c];
}
static void bradford(const double src_w[3], const double dst_w[3], double out[9]) {
  const double M[9] = {0.8951, 0.2664, -0.1614, -0.7502, 1.7135, 0.0367, 0.0389, -0.0685, 1.0296};
  double Mi[9];
  mat3_inv(M, Mi);
  double s[3], d[3];
  for (int r = 0; r < 3; ++r) {
    s[r] = M[r * 3] * src_w[0] + M[r * 3 + 1] * src_w[1] + M[r * 3 + 2] * src_w[2];
    d[r] = M[r * 3] * dst_w[0] + M[r * 3 + 1] * dst_w[1] + M[r * 3 + 2] * dst_w[2];
  }
  double D[9] = {d[0] / s[0], 0, 0, 0, d[1] / s[1], 0, 0, 0, d[2] / s[2]};
  double t[9];
  mat3_mul(D, M, t);
  mat3_mul(Mi, t, out);
}
static const double W_D65[3] = {0.95047, 1.0, 1.08883};
static const double W_E[3] = {1.0, 1.0, 1.0};
static Float srgb_decode(Float c) {
  return c <= FL(0.04045) ? c / FL(12.92) : std::pow((c + FL(0.055)) / FL(1.055), FL(2.4));
}
static Float srgb_encode(Float c) {
  return c <= FL(0.0031308) ? c * FL(12.92) : FL(1.055) * std::pow(c, FL(1.0) / FL(2.4)) - FL(0.055);
}
static void apply3(const double m[9], const Float in[3], Float out[3]) {
  for (int r = 0; r < 3; ++r)
    out[r] = (Float)(m[r * 3] * (double)in[0] + m[r * 3 + 1] * (double)in[1] + m[r * 3 + 2] * (double)in[2]);
}
static void linsrgb_to_xyz_e(const Float lin[3], Float out[3]) {
  double m[9], a[9], t[9];
  srgb_to_xyz_d65_matrix(m);
  bradford(W_D65, W_E, a);
  mat3_mul(a, m, t);
  apply3(t, lin, out);
}
static void srgb_to_xyz_e(const Float rgb[3], Float out[3]) {
  Float lin[3] = {srgb_decode(rgb[0]), srgb_decode(rgb[1]), srgb_decode(rgb[2])};
  linsrgb_to_xyz_e(lin, out);
}
static void xyz_d65_to_xyz_e(const Float in[3], Float out[3]) {
  double a[9];
  bradford(W_D65, W_E, a);
  apply3(a, in, out);
}
// clovers-cli/src/write.rs:39-44: Xyz<E> -> Srgb<f32> -> Srgb<u8>
static void xyz_e_to_srgb8(const Float xyz[3], uint8_t out[3]) {
  double m[9], mi[9], a[9], t[9];
  srgb_to_xyz_d65_matrix(m);
  mat3_inv(m, mi);
  bradford(W_E, W_D65, a);
  mat3_mul(mi, a, t);
  Float lin[3];
  apply3(t, xyz, lin);
  for (int i = 0; i < 3; ++i) {
    Float e = srgb_encode(lin[i]);
    Float v = std::round(e * FL(255.0));
    if (!(v > FL(0.0))) v = FL(0.0);  // NaN and negatives -> 0 (saturating cast)
    if (v > FL(255.0)) v = FL(255.0);
    out[i] = (uint8_t)v;
  }
}

// --------------------------------------------------------------- interval --
// clovers/src/interval.rs:10-62
struct Interval {
  Float min = 0, max = 0;
  Interval() {}
  Interval(Float a, Float b) : min(rmin(a, b)), max(rmax(a, b)) {}
  static Interval combine(const Interval& a, const Interval& b) {
    Interval r;
    r.min = rmin(a.min, b.min);
    r.max = rmax(a.max, b.max);
    return r;
  }
  Interval expand(Float delta) const { return Interval(min - delta, max + delta); }
  Float size() const { return max - min; }
  Float center() const { return min + FL(0.5) * size(); }
};

struct Ray {
  Vec3 origin, direction;
  Float time;
  int wavelength;
  Vec3 evaluate(Float t) const { return origin + t * direction; }
};

// ------------------------------------------------------------------- aabb --
// clovers/src/aabb.rs:10-163
struct AABB {
  Interval x, y, z;
  AABB() {}
  AABB(Interval a, Interval b, Interval c) : x(a), y(b), z(c) {}
  static AABB from_coords(Vec3 a, Vec3 b) {
    return AABB(Interval(a.x, b.x), Interval(a.y, b.y), Interval(a.z, b.z));
  }
  const Interval& axis(int n) const { return n == 0 ? x : (n == 1 ? y : z); }
  // wide: the exit distance widened toward +inf by 4 gamma_3 (Ize 2013),
  // the conservative box test of watertight scenes (not the reference's)
  // and a zero direction component constrains nothing while the origin lies
  // within that slab (inclusive), missing otherwise
  static Float widen_exit(Float f) { return std::fmax(f, f + std::fabs(f) * FL(7.1525574e-7)); }
  bool hit(const Ray& ray, Float tmin, Float tmax, bool wide = false) const {
    if (wide) {
      Float n = -INFINITY, f = INFINITY;
      for (int a = 0; a < 3; ++a) {
        const Interval& ax = axis(a);
        const Float o = ray.origin[a];
        if (ray.direction[a] == FL(0.0)) {
          if (o < ax.min || o > ax.max) return false;
          continue;
        }
        Float adinv = FL(1.0) / ray.direction[a];
        Float t0 = (ax.min - o) * adinv, t1 = (ax.max - o) * adinv;
        n = std::fmax(n, std::fmin(t0, t1));
        f = std::fmin(f, std::fmax(t0, t1));
      }
      return std::fmin(tmax, widen_exit(f)) > std::fmax(tmin, n);
    }
    for (int a = 0; a < 3; ++a) {
      const Interval& ax = axis(a);
      Float adinv = FL(1.0) / ray.direction[a];
      Float t0 = (ax.min - ray.origin[a]) * adinv;
      Float t1 = (ax.max - ray.origin[a]) * adinv;
      if (t0 < t1) {
        if (t0 > tmin) tmin = t0;
        if (t1 < tmax) tmax = t1;
      } else {
        if (t1 > tmin) tmin = t1;
        if (t0 < tmax) tmax = t0;
      }
      if (tmax <= tmin) return false;
    }
    return true;
  }
  static AABB combine(const AABB& a, const AABB& b) {
    return AABB(Interval::combine(a.x, b.x), Interval::combine(a.y, b.y), Interval::combine(a.z, b.z));
  }
  void pad() {
    Float d = EPSILON_RECT_THICKNESS;
    Interval nx = x.size() >= d ? x : x.expand(d);
    Interval ny = y.size() >= d ? y : y.expand(d);
    Interval nz = z.size() >= d ? z : z.expand(d);
    x = nx; y = ny; z = nz;
  }
  // returns false for None
  bool distance(const Ray& ray, Float& out, bool wide = false) const {
    if (wide) {
      Float tmin = -INFINITY, tmax = INFINITY;
      const Interval* ax[3] = {&x, &y, &z};
      for (int a = 0; a < 3; ++a) {
        const Float o = ray.origin[a], d = ray.direction[a];
        if (d == FL(0.0)) {
          if (o < ax[a]->min || o > ax[a]->max) return false;
          continue;
        }
        const Float t1 = (ax[a]->min - o) / d, t2 = (ax[a]->max - o) / d;
        tmin = std::fmax(tmin, std::fmin(t1, t2));
        tmax = std::fmin(tmax, std::fmax(t1, t2));
      }
      tmax = widen_exit(tmax);
      if (tmax >= tmin && tmax > FL(0.0)) { out = tmin; return true; }
      return false;
    }
    Float tx1 = (x.min - ray.origin.x) / ray.direction.x;
    Float tx2 = (x.max - ray.origin.x) / ray.direction.x;
    Float tmin = rmin(tx1, tx2), tmax = rmax(tx1, tx2);
    Float ty1 = (y.min - ray.origin.y) / ray.direction.y;
    Float ty2 = (y.max - ray.origin.y) / ray.direction.y;
    tmin = rmax(tmin, rmin(ty1, ty2));
    tmax = rmin(tmax, rmax(ty1, ty2));
    Float tz1 = (z.min - ray.origin.z) / ray.direction.z;
    Float tz2 = (z.max - ray.origin.z) / ray.direction.z;
    tmin = rmax(tmin, rmin(tz1, tz2));
    tmax = rmin(tmax, rmax(tz1, tz2));
    if (tmax >= tmin && tmax > FL(0.0)) { out = tmin; return true; }
    return false;
  }
  Float area() const {
    Vec3 e = Vec3(x.max, y.max, z.max) - Vec3(x.min, y.min, z.min);
    return FL(2.0) * (e.x * e.y + e.y * e.z + e.x * e.z);
  }
  Vec3 centroid() const { return Vec3(x.center(), y.center(), z.center()); }
  AABB offset(Vec3 o) const {
    return AABB(Interval(x.min + o.x, x.max + o.x), Interval(y.min + o.y, y.max + o.y),
                Interval(z.min + o.z, z.max + o.z));
  }
};

// -------------------------------------------------------------- textures --
struct Material;
struct HitRecord {
  Float distance = 0;
  Vec3 position, normal;
  Float u = 0, v = 0;
  const Material* material = nullptr;
  bool front_face = false;
  int gid = -1;  // index of the top-level (BVH leaf) object that was hit
  // clovers/src/hitrecord.rs:36-43
  void set_face_normal(const Ray& ray, Vec3 outward) {
    front_face = dot(ray.direction, outward) < FL(0.0);
    normal = front_face ? outward : -outward;
  }
};

enum TexKind { TEX_SOLID = 0, TEX_SPATIAL = 1, TEX_SURFACE = 2, TEX_ILLUMINANT = 3 };
// clovers/src/textures.rs:17-121 and textures/*.rs, illuminants via clovers/build.rs:66-111
struct Texture {
  int kind = TEX_SOLID;
  SPD even, odd;  // SolidColor uses `even`
  Float density = 0;
  int illuminant = 0;
  Float intensity = FL(1.0);
  Float color(int lambda, const HitRecord& rec) const {
    switch (kind) {
      case TEX_SOLID: return even.get(lambda);
      case TEX_SPATIAL: {
        Float d = density * PI;
        Float s = FL(1.0) * std::sin(d * rec.position.x) * std::sin(d * rec.position.y) * std::sin(d * rec.position.z);
        return s < FL(0.0) ? odd.get(lambda) : even.get(lambda);
      }
      case TEX_SURFACE: {
        Float d = density * PI;
        Float s = FL(1.0) * std::sin(d * rec.u) * std::sin(d * rec.v);
        return s < FL(0.0) ? odd.get(lambda) : even.get(lambda);
      }
      default: {
        Float c = clv_tables::kIlluminants[illuminant][lambda - MIN_WAVELENGTH] * intensity;
        return rclamp(c, FL(0.0), FL(1.0));
      }
    }
  }
  Float emit(int lambda) const {
    if (kind != TEX_ILLUMINANT) return FL(0.0);
    return clv_tables::kIlluminants[illuminant][lambda - MIN_WAVELENGTH] * intensity;
  }
};

// ------------------------------------------------------------- materials --
enum MatKind { M_DIELECTRIC, M_DISPERSIVE, M_LAMBERTIAN, M_CONELIGHT, M_DIFFUSELIGHT, M_METAL, M_ISOTROPIC };
enum PdfKind { PDF_COSINE, PDF_SPHERE, PDF_ZERO };
struct ScatterRecord {
  bool specular = false;
  Ray specular_ray;
  PdfKind pdf = PDF_ZERO;
  Vec3 pdf_w;  // CosinePDF normal
};
// clovers/src/materials.rs:188-207
static Vec3 reflect(Vec3 v, Vec3 n) { return normalize(v - FL(2.0) * dot(v, n) * n); }
static Vec3 refract(Vec3 v, Vec3 n, Float ratio) {
  Float cos_theta = -dot(v, n);
  cos_theta = rmin(cos_theta, FL(1.0));
  Vec3 par = ratio * (v + cos_theta * n);
  Vec3 perp = -std::sqrt(FL(1.0) - norm_squared(par)) * n;
  return normalize(par + perp);
}
static Float schlick(Float cosine, Float ri) {
  Float r0 = (FL(1.0) - ri) / (FL(1.0) + ri);
  r0 = r0 * r0;
  return r0 + (FL(1.0) - r0) * std::pow(FL(1.0) - cosine, FL(5.0));
}

struct Material {
  int kind = M_LAMBERTIAN;
  Texture tex;                  // albedo / emit
  Float fuzz = 0;               // Metal
  Float refractive_index = FL(1.5);  // Dielectric
  SPD color;                    // Dielectric colour
  Float cauchy_a = FL(1.5046), cauchy_b = FL(0.0042);  // Dispersive
  bool sellmeier = false;       // Dispersive, Sellmeier form (extension)
  Float sell_b[3] = {0, 0, 0}, sell_c[3] = {0, 0, 0};
  Float spread = FL(10.0);         // ConeLight
  bool thin_film = false;
  Float tf_ior = FL(1.5), tf_thickness = FL(500.0);

  bool is_wavelength_dependent() const { return thin_film || kind == M_DISPERSIVE; }  // materials.rs:90-92

  // clovers/src/materials/dispersive.rs:80-83 (Cauchy); Sellmeier is this build's extension
  Float dispersive_index(int lambda) const {
    Float wave_micros = (Float)lambda / FL(1000.0);
    if (!sellmeier) return cauchy_a + (cauchy_b / (wave_micros * wave_micros));
    Float l2 = wave_micros * wave_micros;
    Float s = FL(1.0);
    for (int i = 0; i < 3; ++i) s = s + sell_b[i] * l2 / (l2 - sell_c[i]);
    return std::sqrt(s);
  }

  bool scatter(const Ray& ray, const HitRecord& rec, Rng& rng, ScatterRecord& out) const {
    switch (kind) {
      case M_LAMBERTIAN:  // lambertian.rs:23-50
        out.specular = false;
        out.pdf = PDF_COSINE;
        out.pdf_w = rec.normal;
        return true;
      case M_ISOTROPIC:  // isotropic.rs:23-43
        out.specular = false;
        out.pdf = PDF_SPHERE;
        return true;
      case M_METAL: {  // metal.rs:27-51
        Vec3 reflected = reflect(ray.direction, rec.normal);
        Vec3 dir = normalize(reflected + fuzz * random_unit_vector(rng));
        out.specular = true;
        out.specular_ray = Ray{rec.position, dir, ray.time, ray.wavelength};
        out.pdf = PDF_ZERO;
        return true;
      }
      case M_DIELECTRIC:
      case M_DISPERSIVE: {  // dielectric.rs:37-81, dispersive.rs:58-123
        Float ri = kind == M_DIELECTRIC ? refractive_index : dispersive_index(ray.wavelength);
        Float ratio = rec.front_face ? FL(1.0) / ri : ri;
        Vec3 d = ray.direction;
        Float cos_theta = rmin(-dot(d, rec.normal), FL(1.0));
        Float sin_theta = std::sqrt(FL(1.0) - cos_theta * cos_theta);
        Vec3 sdir;
        if (ratio * sin_theta > FL(1.0)) {
          sdir = reflect(d, rec.normal);
        } else {
          Float rp = schlick(cos_theta, ratio);
          if (rng.next_f32() < rp) sdir = reflect(d, rec.normal);
          else sdir = refract(d, rec.normal, ratio);
        }
        out.specular = true;
        out.specular_ray = Ray{rec.position, sdir, ray.time, ray.wavelength};
        out.pdf = PDF_ZERO;
        return true;
      }
      default:  // lights
        return false;
    }
  }
  // returns false for None
  bool scattering_pdf(const HitRecord& rec, const Ray& scattered, Float& out) const {
    if (kind == M_LAMBERTIAN) {
      Float c = dot(rec.normal, normalize(scattered.direction));
      if (c < FL(0.0)) return false;
      out = c / PI;
      return true;
    }
    if (kind == M_ISOTROPIC) { out = FL(1.0) / (FL(4.0) * PI); return true; }
    return false;
  }
  Float emit(const Ray& ray, int lambda, const HitRecord& rec) const {
    if (kind == M_DIFFUSELIGHT) {  // diffuse_light.rs:41-53
      if (!rec.front_face) return FL(0.0);
      return tex.kind == TEX_ILLUMINANT ? tex.emit(lambda) : tex.color(lambda, rec);
    }
    if (kind == M_CONELIGHT) {  // cone_light.rs:43-66
      if (!rec.front_face) return FL(0.0);
      Float spread_radians = spread * RADS_PER_DEG;
      Float angle = std::acos(-dot(ray.direction, rec.normal) / (norm(ray.direction) * norm(rec.normal)));
      if (angle > spread_radians) return FL(0.0);
      return tex.kind == TEX_ILLUMINANT ? tex.emit(lambda) : tex.color(lambda, rec);
    }
    return FL(0.0);
  }
  Float kind_color(const Ray& ray, int lambda, const HitRecord& rec) const {
    (void)ray;
    switch (kind) {
      case M_DIELECTRIC: return color.get(lambda);
      case M_DISPERSIVE: return FL(1.0);
      case M_CONELIGHT:
      case M_DIFFUSELIGHT: return rclamp(tex.color(lambda, rec), FL(0.0), FL(1.0));
      default: return tex.color(lambda, rec);
    }
  }
  // clovers/src/materials.rs:95-102, thin_film.rs:31-54
  Float color_of(const Ray& ray, int lambda, const HitRecord& rec) const {
    Float tf = FL(1.0);
    if (thin_film) {
      Float n1 = FL(1.0), n2 = tf_ior;
      Float n_ratio = n1 / n2;
      Float cos1 = -dot(ray.direction, rec.normal);
      Float sin1 = std::sqrt(FL(1.0) - cos1 * cos1);
      Float sin2 = n_ratio * sin1;
      Float cos2 = std::sqrt(FL(1.0) - (sin2 * sin2));
      Float opd = FL(2.0) * tf_ior * tf_thickness * cos2;
      Float m = opd / (Float)lambda;
      tf = FL(1.0) + std::cos(m * FL(2.0) * PI);
    }
    return kind_color(ray, lambda, rec) * tf;
  }
};

// ------------------------------------------------------------- hitables --
struct Hitable;
typedef std::unique_ptr<Hitable> HPtr;

struct Counters {
  uint64_t nodes = 0, prims = 0;
};

struct Hitable {
  virtual ~Hitable() {}
  virtual bool hit(const Ray& ray, Float dmin, Float dmax, Rng* rng, HitRecord& out, Counters* c) const = 0;
  virtual const AABB* aabb() const = 0;
  virtual Float pdf_value(Vec3 origin, Vec3 direction, int lambda, Float time, Rng* rng) const = 0;
  virtual Vec3 random(Vec3 origin, Rng& rng) const {
    (void)origin; (void)rng;
    throw std::runtime_error("HitableTrait::random called for a Hitable that has no implementation for it");
  }
  virtual bool has_random() const { return false; }
  virtual Vec3 centroid() const = 0;
  virtual bool is_empty() const { return false; }
  virtual bool is_bvh() const { return false; }
  virtual bool is_list() const { return false; }
  // the optional watertight triangle test (no counterpart in the reference)
  virtual void set_watertight(bool) {}
  int gid = -1;  // top-level object index (set on BVH leaves)
};

struct Empty : Hitable {  // clovers/src/hitable.rs:38-72
  bool hit(const Ray&, Float, Float, Rng*, HitRecord&, Counters*) const override { return false; }
  const AABB* aabb() const override { return nullptr; }
  Float pdf_value(Vec3, Vec3, int, Float, Rng*) const override { return FL(0.0); }
  Vec3 centroid() const override { return Vec3(0, 0, 0); }
  bool is_empty() const override { return true; }
};

static int tag_gid(HitRecord& rec, int gid) {
  if (gid >= 0) rec.gid = gid;
  return 0;
}

struct Sphere : Hitable {  // clovers/src/objects/sphere.rs
  Vec3 center;
  Float radius;
  const Material* material;
  AABB box;
  Sphere(Vec3 c, Float r, const Material* m) : center(c), radius(r), material(m) {
    box = AABB::from_coords(c - Vec3(r, r, r), c + Vec3(r, r, r));
  }
  void get_uv(Vec3 p, Float& u, Float& v) const {
    Vec3 t = (p - center) / radius;
    Float phi = std::atan2(t.z, t.x);
    Float theta = std::asin(t.y);
    u = FL(1.0) - (phi + PI) / (FL(2.0) * PI);
    v = (theta + PI / FL(2.0)) / PI;
  }
  bool hit(const Ray& ray, Float dmin, Float dmax, Rng*, HitRecord& out, Counters* c) const override {
    if (c) c->prims++;
    Vec3 oc = ray.origin - center;
    Float a = norm_squared(ray.direction);
    Float half_b = dot(oc, ray.direction);
    Float cc = norm_squared(oc) - radius * radius;
    Float disc = half_b * half_b - a * cc;
    if (disc > FL(0.0)) {
      Float root = std::sqrt(disc);
      for (int k = 0; k < 2; ++k) {
        Float d = k == 0 ? (-half_b - root) / a : (-half_b + root) / a;
        if (d < dmax && d > dmin) {
          out.distance = d;
          out.position = ray.evaluate(d);
          Vec3 outward = normalize((out.position - center) / radius);
          get_uv(out.position, out.u, out.v);
          out.material = material;
          out.set_face_normal(ray, outward);
          tag_gid(out, gid);
          return true;
        }
      }
    }
    return false;
  }
  const AABB* aabb() const override { return &box; }
  Float pdf_value(Vec3 origin, Vec3 direction, int lambda, Float time, Rng* rng) const override {
    Ray r{origin, direction, time, lambda};
    HitRecord rec;
    if (!hit(r, EPSILON_SHADOW_ACNE, INFINITY, rng, rec, nullptr)) return FL(0.0);
    Float cos_theta_max = std::sqrt(FL(1.0) - radius * radius / norm_squared(center - origin));
    Float solid_angle = FL(2.0) * PI * (FL(1.0) - cos_theta_max);
    return FL(1.0) / solid_angle;
  }
  Vec3 random(Vec3 origin, Rng& rng) const override;
  bool has_random() const override { return true; }
  Vec3 centroid() const override { return center; }
};

struct MovingSphere : Hitable {  // clovers/src/objects/moving_sphere.rs
  Vec3 c0, c1;
  Float t0, t1, radius;
  const Material* material;
  AABB box;
  MovingSphere(Vec3 a, Vec3 b, Float ta, Float tb, Float r, const Material* m)
      : c0(a), c1(b), t0(ta), t1(tb), radius(r), material(m) {
    AABB b0 = AABB::from_coords(a - Vec3(r, r, r), a + Vec3(r, r, r));
    AABB b1 = AABB::from_coords(b - Vec3(r, r, r), b + Vec3(r, r, r));
    box = AABB::combine(b0, b1);
  }
  Vec3 center(Float time) const { return c0 + ((time - t0) / (t1 - t0)) * (c1 - c0); }
  bool hit(const Ray& ray, Float dmin, Float dmax, Rng*, HitRecord& out, Counters* c) const override {
    if (c) c->prims++;
    Vec3 oc = ray.origin - center(ray.time);
    Float a = norm_squared(ray.direction);
    Float half_b = dot(oc, ray.direction);
    Float cc = norm_squared(oc) - radius * radius;
    Float disc = half_b * half_b - a * cc;
    if (disc > FL(0.0)) {
      Float root = std::sqrt(disc);
      for (int k = 0; k < 2; ++k) {
        Float d = k == 0 ? (-half_b - root) / a : (-half_b + root) / a;
        if (d < dmax && d > dmin) {
          out.distance = d;
          out.position = ray.evaluate(d);
          Vec3 outward = normalize((out.position - center(ray.time)) / radius);
          Vec3 t = (out.position - center(ray.time)) / radius;
          Float phi = std::atan2(t.z, t.x);
          Float theta = std::asin(t.y);
          out.u = FL(1.0) - (phi + PI) / (FL(2.0) * PI);
          out.v = (theta + PI / FL(2.0)) / PI;
          out.material = material;
          out.set_face_normal(ray, outward);
          tag_gid(out, gid);
          return true;
        }
      }
    }
    return false;
  }
  const AABB* aabb() const override { return &box; }
  Float pdf_value(Vec3, Vec3, int, Float, Rng*) const override { return FL(0.0); }
  Vec3 centroid() const override { return center(FL(0.5)); }
};

// Shared plane-primitive state for Quad and Triangle (quad.rs:61-83, triangle.rs:61-101)
struct Planar : Hitable {
  Vec3 q, u, v, normal, w;
  Float d, area;
  const Material* material;
  AABB box;
  bool triangle;
  Vec3 corner[3];           // the vertices as given (watertight test)
  bool watertight = false;
  void set_watertight(bool on) override { watertight = on && triangle; }
  // Woop, Benthin & Wald 2013: edge functions in the ray's shear frame, in
  // double when one of them is 0; two-sided; t in [dmin, dmax].
  bool hit_watertight(const Ray& ray, Float dmin, Float dmax, Float& t, Float& alpha, Float& beta) const {
    const Vec3 dd = ray.direction;
    const Float ad[3] = {std::fabs(dd.x), std::fabs(dd.y), std::fabs(dd.z)};
    const int kz = ad[0] > ad[1] ? (ad[0] > ad[2] ? 0 : 2) : (ad[1] > ad[2] ? 1 : 2);
    int kx = (kz + 1) % 3, ky = (kx + 1) % 3;
    auto cmp = [](const Vec3& a, int i) { return i == 0 ? a.x : (i == 1 ? a.y : a.z); };
    if (cmp(dd, kz) < FL(0.0)) std::swap(kx, ky);
    const Float sx = cmp(dd, kx) / cmp(dd, kz), sy = cmp(dd, ky) / cmp(dd, kz), sz = FL(1.0) / cmp(dd, kz);
    const Vec3 A = corner[0] - ray.origin, B = corner[1] - ray.origin, C = corner[2] - ray.origin;
    const Float Ax = cmp(A, kx) - sx * cmp(A, kz), Ay = cmp(A, ky) - sy * cmp(A, kz);
    const Float Bx = cmp(B, kx) - sx * cmp(B, kz), By = cmp(B, ky) - sy * cmp(B, kz);
    const Float Cx = cmp(C, kx) - sx * cmp(C, kz), Cy = cmp(C, ky) - sy * cmp(C, kz);
    Float U = Cx * By - Cy * Bx, V = Ax * Cy - Ay * Cx, W = Bx * Ay - By * Ax;
    if (U == FL(0.0) || V == FL(0.0) || W == FL(0.0)) {
      U = (Float)((double)Cx * By - (double)Cy * Bx);
      V = (Float)((double)Ax * Cy - (double)Ay * Cx);
      W = (Float)((double)Bx * Ay - (double)By * Ax);
    }
    if ((U < FL(0.0) || V < FL(0.0) || W < FL(0.0)) && (U > FL(0.0) || V > FL(0.0) || W > FL(0.0))) return false;
    const Float det = U + V + W;
    if (det == FL(0.0)) return false;
    const Float T = U * (sz * cmp(A, kz)) + V * (sz * cmp(B, kz)) + W * (sz * cmp(C, kz));
    t = T / det;
    if (!(t >= dmin && t <= dmax)) return false;
    alpha = V / det;
    beta = W / det;
    return true;
  }
  Planar(Vec3 q_, Vec3 u_, Vec3 v_, const Material* m, bool tri, const Vec3* corners = nullptr)
      : q(q_), u(u_), v(v_), material(m), triangle(tri) {
    corner[0] = corners ? corners[0] : q;
    corner[1] = corners ? corners[1] : q + u;
    corner[2] = corners ? corners[2] : q + v;
    Vec3 n = cross(u, v);
    normal = normalize(n);
    d = -(dot(normal, q));
    w = n / dot(n, n);
    if (tri) {
      area = norm(n) / FL(2.0);
      Vec3 c1 = q, c2 = q + u, c3 = q + v;
      box = AABB(Interval(rmin(rmin(c1.x, c2.x), c3.x), rmax(rmax(c1.x, c2.x), c3.x)),
                 Interval(rmin(rmin(c1.y, c2.y), c3.y), rmax(rmax(c1.y, c2.y), c3.y)),
                 Interval(rmin(rmin(c1.z, c2.z), c3.z), rmax(rmax(c1.z, c2.z), c3.z)));
    } else {
      area = norm(n);
      box = AABB::from_coords(q, q + u + v);
    }
    box.pad();
  }
  bool hit(const Ray& ray, Float dmin, Float dmax, Rng*, HitRecord& out, Counters* c) const override {
    if (c) c->prims++;
    Float t, alpha, beta;
    Vec3 p;
    if (watertight) {
      if (!hit_watertight(ray, dmin, dmax, t, alpha, beta)) return false;
      p = ray.evaluate(t);
    } else {
      Float denom = dot(normal, ray.direction);
      if (std::fabs(denom) < EPSILON_RECT_THICKNESS) return false;
      t = (-d - dot(normal, ray.origin)) / denom;
      if (t < dmin || t > dmax) return false;
      p = ray.evaluate(t);
      Vec3 ph = p - q;
      alpha = dot(w, cross(ph, v));
      beta = dot(w, cross(u, ph));
      bool inside = (alpha >= FL(0.0) && alpha <= FL(1.0)) && (beta >= FL(0.0) && beta <= FL(1.0));
      if (triangle) inside = inside && (alpha + beta <= FL(1.0));
      if (!inside) return false;
    }
    out.distance = t;
    out.position = p;
    out.u = alpha;
    out.v = beta;
    out.material = material;
    out.set_face_normal(ray, normal);
    tag_gid(out, gid);
    return true;
  }
  const AABB* aabb() const override { return &box; }
  Float pdf_value(Vec3 origin, Vec3 direction, int lambda, Float time, Rng* rng) const override {
    Ray r{origin, direction, time, lambda};
    HitRecord rec;
    if (!hit(r, EPSILON_SHADOW_ACNE, INFINITY, rng, rec, nullptr)) return FL(0.0);
    Float dist2 = rec.distance * rec.distance * norm_squared(direction);
    Float cosine = std::fabs(dot(direction, rec.normal)) / norm(direction);
    return dist2 / (cosine * area);
  }
  Vec3 random(Vec3 origin, Rng& rng) const override {
    if (!triangle) {
      Float a = rng.next_f32();
      Vec3 pa = q + (a * u);
      Float b = rng.next_f32();
      return (pa + (b * v)) - origin;
    }
    Float a = rng.next_f32(), b = rng.next_f32();
    if (a + b > FL(1.0)) { a = FL(1.0) - a; b = FL(1.0) - b; }
    return (q + (a * u) + (b * v)) - origin;
  }
  bool has_random() const override { return true; }
  Vec3 centroid() const override {
    return triangle ? q + (u / FL(4.0)) + (v / FL(4.0)) : q + (u / FL(2.0)) + (v / FL(2.0));
  }
};

// Sphere::random, sphere.rs:160-187 (uses ONB, onb.rs:23-40)
struct ONB {
  Vec3 u, v, w;
  explicit ONB(Vec3 w_) : w(w_) {
    Vec3 a = std::fabs(w.x) > FL(0.9) ? normalize(Vec3(0, 1, 0)) : normalize(Vec3(1, 0, 0));
    v = normalize(cross(w, a));
    u = normalize(cross(w, v));
  }
  Vec3 local(Vec3 a) const { return normalize(a.x * u + a.y * v + a.z * w); }
};
Vec3 Sphere::random(Vec3 origin, Rng& rng) const {
  Vec3 offset = center - origin;
  Float dist2 = norm_squared(offset);
  ONB uvw(normalize(offset));
  Float r1 = rng.next_f32();
  Float r2 = rng.next_f32();
  Float z = FL(1.0) + r2 * (std::sqrt(FL(1.0) - radius * radius / dist2) - FL(1.0));
  Float phi = FL(2.0) * PI * r1;
  Float x = std::cos(phi) * std::sqrt(FL(1.0) - z * z);
  Float y = std::sin(phi) * std::sqrt(FL(1.0) - z * z);
  return uvw.local(normalize(Vec3(x, y, z)));
}

struct Boxy : Hitable {  // clovers/src/objects/boxy.rs
  std::vector<HPtr> sides;
  void set_watertight(bool on) override {
    for (auto& h : sides) h->set_watertight(on);
  }
  AABB box;
  Boxy(Vec3 c0, Vec3 c1, const Material* m) {
    Vec3 mn(rmin(c0.x, c1.x), rmin(c0.y, c1.y), rmin(c0.z, c1.z));
    Vec3 mx(rmax(c0.x, c1.x), rmax(c0.y, c1.y), rmax(c0.z, c1.z));
    Vec3 dx(mx.x - mn.x, 0, 0), dy(0, mx.y - mn.y, 0), dz(0, 0, mx.z - mn.z);
    sides.emplace_back(new Planar(Vec3(mn.x, mn.y, mx.z), dx, dy, m, false));
    sides.emplace_back(new Planar(Vec3(mx.x, mn.y, mx.z), -dz, dy, m, false));
    sides.emplace_back(new Planar(Vec3(mx.x, mn.y, mn.z), -dx, dy, m, false));
    sides.emplace_back(new Planar(Vec3(mn.x, mn.y, mn.z), dz, dy, m, false));
    sides.emplace_back(new Planar(Vec3(mn.x, mx.y, mx.z), dx, -dz, m, false));
    sides.emplace_back(new Planar(Vec3(mn.x, mn.y, mn.z), dx, dz, m, false));
    box = AABB::from_coords(c0, c1);
  }
  bool hit(const Ray& ray, Float dmin, Float dmax, Rng* rng, HitRecord& out, Counters* c) const override {
    bool any = false;
    Float closest = dmax;
    HitRecord rec;
    for (auto& s : sides) {
      if (s->hit(ray, dmin, closest, rng, rec, c)) {
        closest = rec.distance;
        out = rec;
        any = true;
      }
    }
    if (any) tag_gid(out, gid);
    return any;
  }
  const AABB* aabb() const override { return &box; }
  Float pdf_value(Vec3 o, Vec3 d, int l, Float t, Rng* rng) const override {
    Float sum = FL(0.0);
    for (auto& s : sides) sum += s->pdf_value(o, d, l, t, rng) / FL(6.0);
    return sum;
  }
  Vec3 centroid() const override { return box.centroid(); }
};

struct HitableList : Hitable {  // clovers/src/hitable.rs:123-195
  std::vector<HPtr> items;
  void set_watertight(bool on) override {
    for (auto& h : items) h->set_watertight(on);
  }
  AABB box;
  bool hit(const Ray& ray, Float dmin, Float dmax, Rng* rng, HitRecord& out, Counters* c) const override {
    Float distance = INFINITY;
    bool any = false;
    for (auto& h : items) {
      HitRecord rec;
      if (!h->hit(ray, dmin, dmax, rng, rec, c)) return false;  // `?` returns None on any miss
      if (rec.distance < distance) {
        distance = rec.distance;
        out = rec;
        any = true;
      }
    }
    if (any) tag_gid(out, gid);
    return any;
  }
  const AABB* aabb() const override { return &box; }
  Float pdf_value(Vec3, Vec3, int, Float, Rng*) const override { return FL(0.0); }
  Vec3 centroid() const override { return box.centroid(); }
  bool is_list() const override { return true; }
};

struct RotateY : Hitable {  // clovers/src/objects/rotate.rs
  HPtr object;
  void set_watertight(bool on) override { object->set_watertight(on); }
  Float sin_t, cos_t;
  bool has_box = false;
  AABB box;
  RotateY(HPtr obj, Float angle) : object(std::move(obj)) {
    Float radians = angle * RADS_PER_DEG;
    sin_t = std::sin(radians);
    cos_t = std::cos(radians);
    const AABB* b = object->aabb();
    if (!b) return;
    Vec3 mn(INFINITY, INFINITY, INFINITY), mx(-INFINITY, -INFINITY, -INFINITY);
    for (int i = 0; i < 2; ++i)
      for (int j = 0; j < 2; ++j)
        for (int k = 0; k < 2; ++k) {
          Float fi = (Float)i, fj = (Float)j, fk = (Float)k;
          Float x = fi * b->x.max + (FL(1.0) - fi) * b->x.min;
          Float y = fj * b->y.max + (FL(1.0) - fj) * b->y.min;
          Float z = fk * b->z.max + (FL(1.0) - fk) * b->z.min;
          Float nx = cos_t * x + sin_t * z;
          Float nz = -sin_t * x + cos_t * z;
          Vec3 t(nx, y, nz);
          for (int a = 0; a < 3; ++a) {
            mn[a] = rmin(mn[a], t[a]);
            mx[a] = rmax(mx[a], t[a]);
          }
        }
    box = AABB::from_coords(mn, mx);
    has_box = true;
  }
  bool hit(const Ray& ray, Float dmin, Float dmax, Rng* rng, HitRecord& out, Counters* c) const override {
    Vec3 o = ray.origin, d = ray.direction;
    o.x = cos_t * ray.origin.x - sin_t * ray.origin.z;
    o.z = sin_t * ray.origin.x + cos_t * ray.origin.z;
    d.x = cos_t * ray.direction.x - sin_t * ray.direction.z;
    d.z = sin_t * ray.direction.x + cos_t * ray.direction.z;
    Ray rr{o, normalize(d), ray.time, ray.wavelength};
    HitRecord h;
    if (!object->hit(rr, dmin, dmax, rng, h, c)) return false;
    Vec3 p = h.position, n = h.normal;
    p.x = cos_t * h.position.x + sin_t * h.position.z;
    p.z = -sin_t * h.position.x + cos_t * h.position.z;
    n.x = cos_t * h.normal.x + sin_t * h.normal.z;
    n.z = -sin_t * h.normal.x + cos_t * h.normal.z;
    n = normalize(n);
    out = h;
    out.position = p;
    out.set_face_normal(rr, n);
    tag_gid(out, gid);
    return true;
  }
  const AABB* aabb() const override { return has_box ? &box : nullptr; }
  Float pdf_value(Vec3, Vec3, int, Float, Rng*) const override { return FL(0.0); }
  Vec3 centroid() const override { return object->centroid(); }
};

struct Translate : Hitable {  // clovers/src/objects/translate.rs
  HPtr object;
  void set_watertight(bool on) override { object->set_watertight(on); }
  Vec3 offset;
  AABB box;
  Translate(HPtr obj, Vec3 off) : object(std::move(obj)), offset(off) {
    const AABB* b = object->aabb();
    if (!b) throw std::runtime_error("Translate of an object without a bounding box");
    box = b->offset(off);
  }
  bool hit(const Ray& ray, Float dmin, Float dmax, Rng* rng, HitRecord& out, Counters* c) const override {
    Ray moved{ray.origin - offset, ray.direction, ray.time, ray.wavelength};
    HitRecord h;
    if (!object->hit(moved, dmin, dmax, rng, h, c)) return false;
    out = h;
    out.position = h.position + offset;
    out.set_face_normal(moved, h.normal);
    tag_gid(out, gid);
    return true;
  }
  const AABB* aabb() const override { return &box; }
  Float pdf_value(Vec3 o, Vec3 d, int l, Float t, Rng* rng) const override {
    return object->pdf_value(o + offset, d, l, t, rng);
  }
  Vec3 centroid() const override { return object->centroid() + offset; }
};

struct ConstantMedium : Hitable {  // clovers/src/objects/constant_medium.rs
  HPtr boundary;
  void set_watertight(bool on) override { boundary->set_watertight(on); }
  Material phase;  // Isotropic(texture)
  Float neg_inv_density;
  ConstantMedium(HPtr b, Float density, const Texture& tex) : boundary(std::move(b)) {
    phase.kind = M_ISOTROPIC;
    phase.tex = tex;
    neg_inv_density = -FL(1.0) / density;
  }
  bool hit(const Ray& ray, Float dmin, Float dmax, Rng* rng, HitRecord& out, Counters* c) const override {
    HitRecord r1, r2;
    if (!boundary->hit(ray, -INFINITY, INFINITY, rng, r1, c)) return false;
    if (!boundary->hit(ray, r1.distance + EPSILON_CONSTANT_MEDIUM, INFINITY, rng, r2, c)) return false;
    if (r1.distance < dmin) r1.distance = dmin;
    if (r2.distance > dmax) r2.distance = dmax;
    if (r1.distance >= r2.distance) return false;
    if (r1.distance < FL(0.0)) r1.distance = FL(0.0);
    Float ray_length = norm(ray.direction);
    Float inside = (r2.distance - r1.distance) * ray_length;
    if (!rng) throw std::runtime_error("ConstantMedium needs randomness");
    Float hit_distance = neg_inv_density * ln(rng->next_f32());
    if (hit_distance > inside) return false;
    out.distance = r1.distance + hit_distance / ray_length;
    out.position = ray.evaluate(out.distance);
    out.normal = random_unit_vector(*rng);
    out.front_face = true;
    out.u = r1.u;
    out.v = r1.v;
    out.material = &phase;
    tag_gid(out, gid);
    return true;
  }
  const AABB* aabb() const override { return boundary->aabb(); }
  Float pdf_value(Vec3 o, Vec3 d, int l, Float t, Rng* rng) const override {
    return boundary->pdf_value(o, d, l, t, rng);
  }
  Vec3 centroid() const override { return boundary->centroid(); }
};

// ------------------------------------------------------------------- bvh --
struct BVHNode : Hitable {  // clovers/src/bvh.rs:21-28, bvh/hitable_trait.rs
  HPtr left, right;
  bool wide = false;  // conservative box tests of watertight scenes
  void set_watertight(bool on) override {
    wide = on;
    left->set_watertight(on);
    right->set_watertight(on);
  }
  AABB box;
  bool hit(const Ray& ray, Float dmin, Float dmax, Rng* rng, HitRecord& out, Counters* c) const override {
    if (c) c->nodes++;
    if (!box.hit(ray, dmin, dmax, wide)) return false;
    const AABB* la = left->aabb();
    const AABB* ra = right->aabb();
    if (!la && !ra) return false;
    if (la && !ra) return left->hit(ray, dmin, dmax, rng, out, c);
    if (!la && ra) return right->hit(ray, dmin, dmax, rng, out, c);
    Float ld = 0, rd = 0;
    bool lh = la->distance(ray, ld, wide), rh = ra->distance(ray, rd, wide);
    if (!lh && !rh) return false;
    if (lh && !rh) return left->hit(ray, dmin, dmax, rng, out, c);
    if (!lh && rh) return right->hit(ray, dmin, dmax, rng, out, c);
    Float far_d = rmax(ld, rd);
    const Hitable* closest = ld < rd ? left.get() : right.get();
    const Hitable* furthest = ld < rd ? right.get() : left.get();
    HitRecord ch;
    bool chit = closest->hit(ray, dmin, dmax, rng, ch, c);
    if (chit) {
      dmax = ch.distance;
      if (ch.distance < far_d) { out = ch; return true; }
    }
    HitRecord fh;
    bool fhit = furthest->hit(ray, dmin, dmax, rng, fh, c);
    if (!chit && !fhit) return false;
    if (!chit) { out = fh; return true; }
    if (!fhit) { out = ch; return true; }
    out = (ch.distance < fh.distance) ? ch : fh;
    return true;
  }
  const AABB* aabb() const override { return &box; }
  Float pdf_value(Vec3 o, Vec3 d, int l, Float t, Rng* rng) const override {
    if (right->is_empty()) return left->pdf_value(o, d, l, t, rng);
    if (left->is_empty()) return right->pdf_value(o, d, l, t, rng);
    Float a = left->pdf_value(o, d, l, t, rng);
    Float b = right->pdf_value(o, d, l, t, rng);
    return midpoint(a, b);
  }
  Vec3 random(Vec3 o, Rng& rng) const override {
    if (right->is_empty()) return left->random(o, rng);
    if (left->is_empty()) return right->random(o, rng);
    if (rng.next_bool()) return left->random(o, rng);
    return right->random(o, rng);
  }
  bool has_random() const override { return true; }
  Vec3 centroid() const override { return box.centroid(); }
  bool is_bvh() const override { return true; }
};

// clovers/src/bvh/build/utils.rs:42-74
static bool vec_bounding_box(const std::vector<HPtr>& v, AABB& out) {
  if (v.empty()) return false;
  bool have = false;
  for (auto& h : v) {
    const AABB* b = h->aabb();
    if (!b) return false;
    if (have) out = AABB::combine(out, *b);
    else { out = *b; have = true; }
  }
  return true;
}

// clovers/src/bvh/build/surface_area_heuristic.rs:134-156
static Float evaluate_sah(const std::vector<HPtr>& hs, int axis, Float pos) {
  AABB lb, rb;
  uint64_t lc = 0, rc = 0;
  for (auto& h : hs) {
    if (h->centroid()[axis] <= pos) {
      lc++;
      lb = AABB::combine(lb, *h->aabb());
    } else {
      rc++;
      rb = AABB::combine(rb, *h->aabb());
    }
  }
  return (Float)lc * lb.area() + (Float)rc * rb.area();
}
// surface_area_heuristic.rs:81-132
static void find_best_split(const std::vector<HPtr>& hs, int& best_axis, Float& best_pos) {
  best_axis = 0;
  best_pos = FL(0.0);
  Float best_cost = INFINITY;
  for (int axis = 0; axis < 3; ++axis) {
    Float bmin = INFINITY, bmax = -INFINITY;
    for (auto& h : hs) {
      Float cv = h->centroid()[axis];
      bmin = rmin(bmin, cv);
      bmax = rmax(bmax, cv);
    }
    if (bmin == bmax) continue;
    Float scale = (bmax - bmin) / FL(8.0);
    for (int i = 0; i < 8; ++i) {
      Float cand = bmin + (Float)i * scale;
      Float cost = evaluate_sah(hs, axis, cand);
      if (cost < best_cost) {
        best_pos = cand;
        best_axis = axis;
        best_cost = cost;
      }
    }
  }
}
// surface_area_heuristic.rs:18-79
static std::unique_ptr<BVHNode> build_sah(std::vector<HPtr> hs) {
  std::unique_ptr<BVHNode> node(new BVHNode());
  if (!vec_bounding_box(hs, node->box)) throw std::runtime_error("BVH build over an empty or unbounded list");
  size_t count = hs.size();
  if (count == 1) {
    node->left = std::move(hs[0]);
    node->right.reset(new Empty());
    return node;
  }
  if (count == 2) {
    node->left = std::move(hs[0]);
    node->right = std::move(hs[1]);
    return node;
  }
  int axis;
  Float pos;
  find_best_split(hs, axis, pos);
  std::vector<HPtr> L, R;
  for (auto& h : hs) {
    if (h->centroid()[axis] <= pos) L.push_back(std::move(h));
    else R.push_back(std::move(h));
  }
  if (L.empty()) {
    node->left = std::move(R[0]);
    R.erase(R.begin());
    node->right = build_sah(std::move(R));
    return node;
  }
  if (R.empty()) {
    HPtr h = std::move(L[0]);
    L.erase(L.begin());
    node->left = build_sah(std::move(L));
    node->right = std::move(h);
    return node;
  }
  node->left = build_sah(std::move(L));
  node->right = build_sah(std::move(R));
  return node;
}
// longest_axis_midpoint.rs:12-93: split at the middle of the list sorted by
// box minimum along the axis of largest span.  The comparator
// (bvh/build/utils.rs:7-21) answers Less only for a strictly smaller minimum,
// so a stable sort keeps ties in list order, while the two-object case, which
// compares the pair directly, puts the second object first on a tie.
static std::unique_ptr<BVHNode> build_lam(std::vector<HPtr> hs) {
  std::unique_ptr<BVHNode> node(new BVHNode());
  if (!vec_bounding_box(hs, node->box)) throw std::runtime_error("No bounding box for objects");
  const Float sx = node->box.x.size(), sy = node->box.y.size(), sz = node->box.z.size();
  const Float largest = rmax(rmax(sx, sy), sz);
  int axis;
  if (sx == largest) axis = 0;
  else if (sy == largest) axis = 1;
  else if (sz == largest) axis = 2;
  else throw std::runtime_error("no axis of largest span (NaN box)");
  auto key = [axis](const HPtr& h) { return h->aabb()->axis(axis).min; };
  const size_t n = hs.size();
  if (n == 1) {
    node->left = std::move(hs[0]);
    node->right.reset(new Empty());
    return node;
  }
  if (n == 2) {
    if (key(hs[0]) < key(hs[1])) {
      node->left = std::move(hs[0]);
      node->right = std::move(hs[1]);
    } else {
      node->left = std::move(hs[1]);
      node->right = std::move(hs[0]);
    }
    return node;
  }
  std::stable_sort(hs.begin(), hs.end(), [&](const HPtr& a, const HPtr& b) { return key(a) < key(b); });
  if (n == 3) {
    node->left = std::move(hs[0]);
    std::unique_ptr<BVHNode> r(new BVHNode());
    r->box = AABB::combine(*hs[1]->aabb(), *hs[2]->aabb());
    r->left = std::move(hs[1]);
    r->right = std::move(hs[2]);
    node->right = std::move(r);
    return node;
  }
  const size_t mid = n / 2;
  std::vector<HPtr> R;
  for (size_t i = mid; i < n; ++i) R.push_back(std::move(hs[i]));
  hs.resize(mid);
  node->left = build_lam(std::move(hs));
  node->right = build_lam(std::move(R));
  return node;
}
static std::unique_ptr<BVHNode> build_bvh(std::vector<HPtr> hs, bool lam) {
  return lam ? build_lam(std::move(hs)) : build_sah(std::move(hs));
}

// ----------------------------------------------------------------- camera --
struct Camera {  // clovers/src/camera.rs:59-126
  Vec3 llc, horizontal, vertical, origin, u, v, w;
  Float lens_radius = 0;
  void init(Vec3 look_from, Vec3 look_at, Vec3 up, Float vfov, Float aspect, Float aperture, Float focus) {
    lens_radius = aperture / FL(2.0);
    Float theta = vfov * PI / FL(180.0);
    Float half_height = std::tan(theta / FL(2.0));
    Float half_width = aspect * half_height;
    origin = look_from;
    w = normalize(look_from - look_at);
    u = normalize(cross(up, w));
    v = normalize(cross(w, u));
    llc = origin - (half_width * focus) * u - (half_height * focus) * v - focus * w;
    horizontal = (FL(2.0) * half_width * focus) * u;
    vertical = (FL(2.0) * half_height * focus) * v;
  }
  Ray get_ray(Float pu, Float pv, Float lx, Float ly, Float time, int lambda) const {
    lx *= lens_radius;
    ly *= lens_radius;
    Vec3 offset = u * lx + v * ly;
    Vec3 dir = llc + pu * horizontal + pv * vertical - origin - offset;
    return Ray{origin + offset, normalize(dir), time, lambda};
  }
};

// ----------------------------------------------------------------- scene --
struct Scene {
  Camera camera;
  Float background[3] = {0, 0, 0};
  SPD background_spd;
  std::vector<std::unique_ptr<Material>> materials;
  std::unique_ptr<BVHNode> bvh_root;
  HPtr mis_root;  // BVHNode or Empty-free tree over priority objects
  size_t object_count = 0;
};

// ------------------------------------------------------------ scene load --
using clv_json::Value;

static Vec3 json_vec3(const Value& v, const char* what) {
  if (v.is_array() && v.arr.size() == 3)
    return Vec3(v.arr[0].as_f32(what), v.arr[1].as_f32(what), v.arr[2].as_f32(what));
  if (v.is_object() && v.has("x")) return Vec3(v.at("x").as_f32(), v.at("y").as_f32(), v.at("z").as_f32());
  throw std::runtime_error(std::string("expected a 3-vector for ") + what);
}
static void json_rgb(const Value& v, Float out[3], const char* what) {
  if (v.is_array() && v.arr.size() == 3) {
    for (int i = 0; i < 3; ++i) out[i] = v.arr[i].as_f32(what);
    return;
  }
  if (v.is_object() && v.has("red")) {
    out[0] = v.at("red").as_f32(); out[1] = v.at("green").as_f32(); out[2] = v.at("blue").as_f32();
    return;
  }
  throw std::runtime_error(std::string("expected an RGB triple for ") + what);
}
static int hexval(char c) {
  if (c >= '0' && c <= '9') return c - '0';
  if (c >= 'a' && c <= 'f') return c - 'a' + 10;
  if (c >= 'A' && c <= 'F') return c - 'A' + 10;
  throw std::runtime_error("bad hex colour");
}
// clovers/src/colorinit.rs:45-60 -> Xyz<E>
static void color_init(const Value& v, Float out[3]) {
  if (v.is_array()) {
    Float rgb[3];
    json_rgb(v, rgb, "color");
    srgb_to_xyz_e(rgb, out);
    return;
  }
  if (!v.is_object() || v.obj.size() != 1) throw std::runtime_error("unsupported colour form");
  const std::string& k = v.obj[0].first;
  const Value& c = v.obj[0].second;
  Float t[3];
  if (k == "hex") {
    std::string s = c.as_string("hex");
    if (!s.empty() && s[0] == '#') s = s.substr(1);
    if (s.size() == 3) s = std::string{s[0], s[0], s[1], s[1], s[2], s[2]};
    if (s.size() != 6) throw std::runtime_error("bad hex colour");
    for (int i = 0; i < 3; ++i) t[i] = (Float)(hexval(s[2 * i]) * 16 + hexval(s[2 * i + 1])) / FL(255.0);
    srgb_to_xyz_e(t, out);
  } else if (k == "srgb") {
    json_rgb(c, t, "srgb");
    srgb_to_xyz_e(t, out);
  } else if (k == "lin_srgb") {
    json_rgb(c, t, "lin_srgb");
    linsrgb_to_xyz_e(t, out);
  } else if (k == "xyz_e") {
    Vec3 x = json_vec3(c, "xyz_e");
    out[0] = x.x; out[1] = x.y; out[2] = x.z;
  } else if (k == "xyz_d65") {
    Vec3 x = json_vec3(c, "xyz_d65");
    Float in[3] = {x.x, x.y, x.z};
    xyz_d65_to_xyz_e(in, out);
  } else {
    throw std::runtime_error("unsupported colour kind: " + k);
  }
}
static const char* const kIllumPrefix = "Illuminant";
static int illuminant_index(const std::string& kind) {
  // texture kinds IlluminantD50, IlluminantLedB1 ... IlluminantFL3_15 (textures.rs:57-108)
  std::string suffix = kind.substr(strlen(kIllumPrefix));
  std::string norm;
  if (suffix.rfind("Led", 0) == 0) norm = "LED_" + suffix.substr(3);
  else norm = suffix;
  for (int i = 0; i < clv_tables::kNumIlluminants; ++i)
    if (norm == clv_tables::kIlluminantNames[i]) return i;
  throw std::runtime_error("unknown texture kind: " + kind);
}
static Texture texture_default() {
  Texture t;
  Float g[3] = {FL(0.5), FL(0.5), FL(0.5)};
  t.kind = TEX_SOLID;
  t.even = SPD(g);
  return t;
}
static Texture texture_init(const Value& v) {
  Texture t;
  const std::string& kind = v.at("kind").as_string("texture kind");
  if (kind == "SolidColor") {
    Float xyz[3];
    color_init(v.at("color"), xyz);
    t.kind = TEX_SOLID;
    t.even = SPD(xyz);
  } else if (kind == "SpatialChecker" || kind == "SurfaceChecker") {
    Float ev[3] = {FL(0.8), FL(0.8), FL(0.8)}, od[3] = {FL(0.5), FL(0.5), FL(0.5)};
    if (v.has("even")) color_init(v.at("even"), ev);
    if (v.has("odd")) color_init(v.at("odd"), od);
    t.kind = kind == "SpatialChecker" ? TEX_SPATIAL : TEX_SURFACE;
    t.even = SPD(ev);
    t.odd = SPD(od);
    t.density = v.has("density") ? v.at("density").as_f32() : (kind == "SpatialChecker" ? FL(1.0) : FL(10.0));
  } else if (kind.rfind(kIllumPrefix, 0) == 0) {
    t.kind = TEX_ILLUMINANT;
    t.illuminant = illuminant_index(kind);
    t.intensity = v.has("intensity") ? v.at("intensity").as_f32() : FL(1.0);
  } else {
    throw std::runtime_error("unknown texture kind: " + kind);
  }
  return t;
}
static Material material_init(const Value& v) {
  Material m;
  const std::string& kind = v.at("kind").as_string("material kind");
  if (kind == "Lambertian" || kind == "Isotropic") {
    m.kind = kind == "Lambertian" ? M_LAMBERTIAN : M_ISOTROPIC;
    m.tex = v.has("albedo") ? texture_init(v.at("albedo")) : texture_default();
  } else if (kind == "Metal") {
    m.kind = M_METAL;
    m.tex = v.has("albedo") ? texture_init(v.at("albedo")) : texture_default();
    m.fuzz = v.has("fuzz") ? v.at("fuzz").as_f32() : FL(0.0);
  } else if (kind == "Dielectric") {
    m.kind = M_DIELECTRIC;
    m.refractive_index = v.has("refractive_index") ? v.at("refractive_index").as_f32() : FL(1.5);
    Float c[3] = {FL(1.0), FL(1.0), FL(1.0)};
    if (v.has("color")) {
      Vec3 x = json_vec3(v.at("color"), "color");
      c[0] = x.x; c[1] = x.y; c[2] = x.z;
    }
    m.color = SPD(c);
  } else if (kind == "Dispersive") {
    m.kind = M_DISPERSIVE;
    if (v.has("cauchy_a")) m.cauchy_a = v.at("cauchy_a").as_f32();
    if (v.has("cauchy_b")) m.cauchy_b = v.at("cauchy_b").as_f32();
    if (v.has("sellmeier_b") || v.has("sellmeier_c")) {
      Vec3 b = json_vec3(v.at("sellmeier_b"), "sellmeier_b"), c = json_vec3(v.at("sellmeier_c"), "sellmeier_c");
      m.sellmeier = true;
      for (int i = 0; i < 3; ++i) { m.sell_b[i] = b[i]; m.sell_c[i] = c[i]; }
    }
  } else if (kind == "DiffuseLight") {
    m.kind = M_DIFFUSELIGHT;
    m.tex = texture_init(v.at("emit"));
  } else if (kind == "ConeLight") {
    m.kind = M_CONELIGHT;
    m.spread = v.at("spread").as_f32();
    m.tex = texture_init(v.at("emit"));
  } else {
    throw std::runtime_error("unknown material kind: " + kind);
  }
  if (v.has("thin_film") && !v.at("thin_film").is_null()) {
    const Value& tf = v.at("thin_film");
    m.thin_film = true;
    m.tf_ior = tf.has("refractive_index") ? tf.at("refractive_index").as_f32() : FL(1.5);
    m.tf_thickness = tf.has("thickness") ? tf.at("thickness").as_f32() : FL(500.0);
  }
  return m;
}

struct Loader {
  Scene* scene;
  std::vector<std::pair<std::string, const Material*>> shared;
  const Material* fallback = nullptr;
  std::string base_dir;

  const Material* material_ref(const Value* v) {
    if (!v || v->is_string()) {
      std::string name = v ? v->str : std::string();
      for (auto& kv : shared)
        if (kv.first == name) return kv.second;
      for (auto& kv : shared)
        if (kv.first.empty()) return kv.second;
      return fallback;
    }
    scene->materials.emplace_back(new Material(material_init(*v)));
    return scene->materials.back().get();
  }

  // clovers/src/objects/stl.rs:52-104 (binary STL)
  void load_stl(const Value& o, std::vector<HPtr>& out) {
    std::string path = o.at("path").as_string("path");
    std::ifstream f(path, std::ios::binary);
    if (!f && !base_dir.empty()) f.open(base_dir + "/" + path, std::ios::binary);
    if (!f) throw std::runtime_error("cannot open STL file " + path);
    std::vector<char> data((std::istreambuf_iterator<char>(f)), std::istreambuf_iterator<char>());
    if (data.size() < 84) throw std::runtime_error("STL file too short");
    uint32_t n;
    std::memcpy(&n, data.data() + 80, 4);
    if (data.size() < 84 + (size_t)n * 50) throw std::runtime_error("STL file truncated (only binary STL is read)");
    const Material* mat = material_ref(o.find("material"));
    Float scale = o.at("scale").as_f32();
    Vec3 center = json_vec3(o.at("center"), "center");
    Vec3 rot = json_vec3(o.at("rotation"), "rotation");
    Float sr = std::sin(rot.x * RADS_PER_DEG), cr = std::cos(rot.x * RADS_PER_DEG);
    Float sp = std::sin(rot.y * RADS_PER_DEG), cp = std::cos(rot.y * RADS_PER_DEG);
    Float sy = std::sin(rot.z * RADS_PER_DEG), cy = std::cos(rot.z * RADS_PER_DEG);
    // nalgebra Rotation3::from_euler_angles(roll, pitch, yaw), row-major
    Float R[9] = {cy * cp, cy * sp * sr - sy * cr, cy * sp * cr + sy * sr,
                  sy * cp, sy * sp * sr + cy * cr, sy * sp * cr - cy * sr,
                  -sp,     cp * sr,                cp * cr};
    for (uint32_t i = 0; i < n; ++i) {
      const char* rec = data.data() + 84 + (size_t)i * 50;
      Vec3 p[3];
      for (int k = 0; k < 3; ++k) {
        float c[3];
        std::memcpy(c, rec + 12 + 12 * k, 12);
        Vec3 a(c[0], c[1], c[2]);
        Vec3 r(R[0] * a.x + R[1] * a.y + R[2] * a.z, R[3] * a.x + R[4] * a.y + R[5] * a.z,
               R[6] * a.x + R[7] * a.y + R[8] * a.z);
        p[k] = r * scale + center;
      }
      out.emplace_back(new Planar(p[0], p[1] - p[0], p[2] - p[0], mat, true, p));
    }
  }

  // clovers/src/objects/ply.rs:55-118 with ply-rs's reading of the file:
  // vertex x/y/z (int, uint, float, double -> f32), face vertex_indices (the
  // first three; unsigned lists as read, signed lists by absolute value).
  void load_ply(const Value& o, std::vector<HPtr>& out) {
    std::string path = o.at("path").as_string("path");
    std::ifstream f(path, std::ios::binary);
    if (!f && !base_dir.empty()) f.open(base_dir + "/" + path, std::ios::binary);
    if (!f) throw std::runtime_error("cannot open PLY file " + path);
    std::string blob((std::istreambuf_iterator<char>(f)), std::istreambuf_iterator<char>());
    const size_t hend = blob.find("end_header");
    if (blob.compare(0, 3, "ply") != 0 || hend == std::string::npos) throw std::runtime_error("not a PLY file");
    size_t body = blob.find('\n', hend);
    body = body == std::string::npos ? blob.size() : body + 1;
    struct P { std::string name, type, count; bool list; };
    struct E { std::string name; unsigned long long n; std::vector<P> props; };
    std::vector<E> elems;
    std::string fmt;
    std::istringstream hs(blob.substr(0, hend));
    std::string ln;
    while (std::getline(hs, ln)) {
      if (!ln.empty() && ln.back() == '\r') ln.pop_back();
      std::istringstream ls(ln);
      std::string w;
      ls >> w;
      if (w == "format") ls >> fmt;
      else if (w == "element") { E e; ls >> e.name >> e.n; elems.push_back(e); }
      else if (w == "property") {
        P p;
        std::string t;
        ls >> t;
        p.list = t == "list";
        if (p.list) ls >> p.count >> p.type >> p.name;
        else { p.type = t; ls >> p.name; }
        elems.back().props.push_back(p);
      }
    }
    auto width = [](const std::string& t) -> int {
      if (t == "char" || t == "int8" || t == "uchar" || t == "uint8") return 1;
      if (t == "short" || t == "int16" || t == "ushort" || t == "uint16") return 2;
      if (t == "double" || t == "float64") return 8;
      return 4;
    };
    const bool ascii = fmt == "ascii", big = fmt == "binary_big_endian";
    std::istringstream as(ascii ? blob.substr(body) : std::string());
    size_t pos = body;
    // one value as (double, is floating type); integers exactly as int64
    auto next = [&](const std::string& t, long long& iv) -> double {
      const bool fl = t == "float" || t == "float32" || t == "double" || t == "float64";
      if (ascii) {
        std::string tok;
        if (!(as >> tok)) throw std::runtime_error("PLY body ends early");
        if (t == "float" || t == "float32") return (double)std::strtof(tok.c_str(), nullptr);
        if (fl) return std::strtod(tok.c_str(), nullptr);
        iv = std::strtoll(tok.c_str(), nullptr, 10);
        return (double)iv;
      }
      const int n = width(t);
      if (pos + n > blob.size()) throw std::runtime_error("PLY body ends early");
      unsigned char b[8];
      for (int k = 0; k < n; ++k) b[k] = (unsigned char)blob[pos + (big ? n - 1 - k : k)];  // little-endian host
      pos += n;
      if (t == "float" || t == "float32") { float v; std::memcpy(&v, b, 4); return v; }
      if (fl) { double v; std::memcpy(&v, b, 8); return v; }
      const bool sg = t == "char" || t == "int8" || t == "short" || t == "int16" || t == "int" || t == "int32";
      unsigned long long u = 0;
      std::memcpy(&u, b, n);
      if (sg && n < 8 && (u >> (8 * n - 1)) & 1ull) u |= ~0ull << (8 * n);
      iv = (long long)u;
      return (double)iv;
    };
    std::vector<Vec3> verts;
    std::vector<unsigned long long> idx;
    for (const E& e : elems)
      for (unsigned long long r = 0; r < e.n; ++r) {
        Float xyz[3] = {0, 0, 0};
        for (const P& p : e.props) {
          long long iv = 0;
          if (p.list) {
            next(p.count, iv);
            const long long cnt = iv;
            for (long long j = 0; j < cnt; ++j) {
              const double v = next(p.type, iv);
              (void)v;
              if (e.name == "face" && p.name == "vertex_indices" && j < 3) idx.push_back(iv < 0 ? -iv : iv);
            }
          } else {
            const double v = next(p.type, iv);
            if (e.name == "vertex" && (p.name == "x" || p.name == "y" || p.name == "z")) {
              const bool is_f32 = p.type == "float" || p.type == "float32";
              xyz[p.name[0] - 'x'] = is_f32 ? (Float)v : (Float)v;  // f64 and ints: one rounding to f32
            }
          }
        }
        if (e.name == "vertex") verts.emplace_back(xyz[0], xyz[1], xyz[2]);
      }
    const Material* mat = material_ref(o.find("material"));
    Float scale = o.at("scale").as_f32();
    Vec3 center = json_vec3(o.at("center"), "center");
    Vec3 rot = json_vec3(o.at("rotation"), "rotation");
    Float sr = std::sin(rot.x * RADS_PER_DEG), cr = std::cos(rot.x * RADS_PER_DEG);
    Float sp = std::sin(rot.y * RADS_PER_DEG), cp = std::cos(rot.y * RADS_PER_DEG);
    Float sy = std::sin(rot.z * RADS_PER_DEG), cy = std::cos(rot.z * RADS_PER_DEG);
    Float R[9] = {cy * cp, cy * sp * sr - sy * cr, cy * sp * cr + sy * sr,
                  sy * cp, sy * sp * sr + cy * cr, sy * sp * cr - cy * sr,
                  -sp,     cp * sr,                cp * cr};
    for (size_t i = 0; i + 2 < idx.size(); i += 3) {
      Vec3 p[3];
      for (int k = 0; k < 3; ++k) {
        const Vec3 a = verts.at(idx[i + k]);
        Vec3 r(R[0] * a.x + R[1] * a.y + R[2] * a.z, R[3] * a.x + R[4] * a.y + R[5] * a.z,
               R[6] * a.x + R[7] * a.y + R[8] * a.z);
        p[k] = r * scale + center;
      }
      out.emplace_back(new Planar(p[0], p[1] - p[0], p[2] - p[0], mat, true, p));
    }
  }

  HPtr object(const Value& o, std::vector<HPtr>* flat_list) {
    const std::string& kind = o.at("kind").as_string("object kind");
    if (kind == "Sphere")
      return HPtr(new Sphere(json_vec3(o.at("center"), "center"), o.at("radius").as_f32(), material_ref(o.find("material"))));
    if (kind == "MovingSphere")
      return HPtr(new MovingSphere(json_vec3(o.at("center_0"), "center_0"), json_vec3(o.at("center_1"), "center_1"), FL(0.0),
                                   FL(1.0), o.at("radius").as_f32(), material_ref(o.find("material"))));
    if (kind == "Quad" || kind == "Triangle")
      return HPtr(new Planar(json_vec3(o.at("q"), "q"), json_vec3(o.at("u"), "u"), json_vec3(o.at("v"), "v"),
                             material_ref(o.find("material")), kind == "Triangle"));
    if (kind == "Boxy")
      return HPtr(new Boxy(json_vec3(o.at("corner_0"), "corner_0"), json_vec3(o.at("corner_1"), "corner_1"),
                           material_ref(o.find("material"))));
    if (kind == "ConstantMedium") {
      HPtr b = object(o.at("boundary"), nullptr);
      Float density = o.has("density") ? o.at("density").as_f32() : FL(0.1);
      Texture t = o.has("texture") ? texture_init(o.at("texture")) : texture_default();
      return HPtr(new ConstantMedium(std::move(b), density, t));
    }
    if (kind == "RotateY") return HPtr(new RotateY(object(o.at("object"), nullptr), o.at("angle").as_f32()));
    if (kind == "Translate")
      return HPtr(new Translate(object(o.at("object"), nullptr), json_vec3(o.at("offset"), "offset")));
    if (kind == "ObjectList" || kind == "STL" || kind == "PLY") {
      std::unique_ptr<HitableList> l(new HitableList());
      if (kind == "STL") load_stl(o, l->items);
      else if (kind == "PLY") load_ply(o, l->items);
      else
        for (auto& c : o.at("objects").arr) l->items.push_back(object(c, nullptr));
      if (!vec_bounding_box(l->items, l->box)) throw std::runtime_error("No bounding box for hitables");
      (void)flat_list;
      return HPtr(l.release());
    }
    throw std::runtime_error("unsupported object kind: " + kind);
  }
};

static HPtr clone_for_priority(const Value& o, Loader& ld) { return ld.object(o, nullptr); }

// clovers-cli/src/scenefile.rs:34-117
static Scene* load_scene(const std::string& text, uint32_t width, uint32_t height, const std::string& base_dir,
                         bool lam = false) {
  Value root = clv_json::parse(text);
  std::unique_ptr<Scene> sc(new Scene());
  Loader ld;
  ld.scene = sc.get();
  ld.base_dir = base_dir;
  Float t0 = root.at("time_0").as_f32(), t1 = root.at("time_1").as_f32();
  (void)t0; (void)t1;
  Float bg_rgb[3];
  json_rgb(root.at("background_color"), bg_rgb, "background_color");
  srgb_to_xyz_e(bg_rgb, sc->background);
  sc->background_spd = SPD(sc->background);
  const Value& cam = root.at("camera");
  sc->camera.init(json_vec3(cam.at("look_from"), "look_from"), json_vec3(cam.at("look_at"), "look_at"),
                  json_vec3(cam.at("up"), "up"), cam.at("vertical_fov").as_f32(), (Float)width / (Float)height,
                  cam.at("aperture").as_f32(), cam.at("focus_distance").as_f32());
  if (root.has("materials")) {
    for (auto& m : root.at("materials").arr) {
      sc->materials.emplace_back(new Material(material_init(m)));
      ld.shared.emplace_back(m.at("name").as_string("name"), sc->materials.back().get());
    }
  }
  sc->materials.emplace_back(new Material());  // SharedMaterial::default(): Lambertian, grey 0.5
  {
    Float g[3] = {FL(0.5), FL(0.5), FL(0.5)};
    sc->materials.back()->tex.even = SPD(g);
  }
  ld.shared.emplace_back(std::string(), sc->materials.back().get());
  ld.fallback = sc->materials.back().get();

  std::vector<HPtr> hitables, priority;
  for (auto& o : root.at("objects").arr) {
    bool prio = o.has("priority") && o.at("priority").as_bool("priority");
    HPtr h = ld.object(o, nullptr);
    if (h->is_list()) {
      HitableList* l = static_cast<HitableList*>(h.get());
      HPtr pl;
      if (prio) pl = clone_for_priority(o, ld);
      HitableList* plist = prio ? static_cast<HitableList*>(pl.get()) : nullptr;
      for (size_t i = 0; i < l->items.size(); ++i) {
        if (l->items[i]->is_list()) throw std::runtime_error("Recursing too hard in scene initialization");
        if (prio) priority.push_back(std::move(plist->items[i]));
        hitables.push_back(std::move(l->items[i]));
      }
    } else {
      if (prio) priority.push_back(clone_for_priority(o, ld));
      hitables.push_back(std::move(h));
    }
  }
  for (size_t i = 0; i < hitables.size(); ++i) hitables[i]->gid = (int)i;
  sc->object_count = hitables.size();
  if (hitables.empty()) throw std::runtime_error("scene has no objects");
  if (priority.empty()) throw std::runtime_error("scene has no priority objects (the reference's MIS BVH build panics)");
  sc->bvh_root = build_bvh(std::move(hitables), lam);  // scenefile.rs:106-108: both trees, one algorithm
  sc->mis_root = build_bvh(std::move(priority), lam);
  return sc.release();
}

static Scene* mesh_scene(const float* verts, uint32_t nverts, const uint32_t* idx, uint32_t ntris) {
  std::unique_ptr<Scene> sc(new Scene());
  sc->materials.emplace_back(new Material());
  Float g[3] = {FL(0.5), FL(0.5), FL(0.5)};
  sc->materials.back()->tex.even = SPD(g);
  const Material* m = sc->materials.back().get();
  std::vector<HPtr> hs;
  hs.reserve(ntris);
  for (uint32_t i = 0; i < ntris; ++i) {
    uint32_t ia = idx[3 * i], ib = idx[3 * i + 1], ic = idx[3 * i + 2];
    if (ia >= nverts || ib >= nverts || ic >= nverts) throw std::runtime_error("vertex index out of range");
    Vec3 a(verts[3 * ia], verts[3 * ia + 1], verts[3 * ia + 2]);
    Vec3 b(verts[3 * ib], verts[3 * ib + 1], verts[3 * ib + 2]);
    Vec3 c(verts[3 * ic], verts[3 * ic + 1], verts[3 * ic + 2]);
    const Vec3 corners[3] = {a, b, c};
    hs.emplace_back(new Planar(a, b - a, c - a, m, true, corners));  // Triangle::from_coordinates
    hs.back()->gid = (int)i;
  }
  sc->object_count = ntris;
  sc->bvh_root = build_sah(std::move(hs));
  return sc.release();
}

// ----------------------------------------------------------------- trace --
// clovers-cli/src/trace.rs:21-122
static void trace(const Ray& ray, const Scene& sc, uint32_t depth, uint32_t max_depth, Rng& rng, Float out[4]) {
  int hero = ray.wavelength;
  int waves[4];
  rotate_wavelength(hero, waves);
  Float bg[4];
  for (int i = 0; i < 4; ++i) bg[i] = sc.background_spd.get(waves[i]);
  if (depth > max_depth) {
    for (int i = 0; i < 4; ++i) out[i] = FL(0.0);
    return;
  }
  HitRecord rec;
  if (!sc.bvh_root->hit(ray, EPSILON_SHADOW_ACNE, FL(3.40282347e+38), &rng, rec, nullptr)) {
    for (int i = 0; i < 4; ++i) out[i] = bg[i];
    return;
  }
  const Material* m = rec.material;
  Float emitted[4];
  for (int i = 0; i < 4; ++i) emitted[i] = m->emit(ray, waves[i], rec);
  ScatterRecord srec;
  if (!m->scatter(ray, rec, rng, srec)) {
    for (int i = 0; i < 4; ++i) out[i] = emitted[i];
    return;
  }
  Float atten[4];
  if (m->is_wavelength_dependent()) {
    atten[0] = m->color_of(ray, hero, rec);
    atten[1] = atten[2] = atten[3] = FL(0.0);
  } else {
    for (int i = 0; i < 4; ++i) atten[i] = m->color_of(ray, waves[i], rec);
  }
  if (srec.specular) {
    Float spec[4];
    trace(srec.specular_ray, sc, depth + 1, max_depth, rng, spec);
    for (int i = 0; i < 4; ++i) out[i] = spec[i] * atten[i];
    return;
  }
  // Diffuse: MixturePDF(HitablePDF(mis root, position), scatter pdf), pdf.rs:122-140
  Vec3 origin = rec.position;
  Vec3 gen;
  if (rng.next_bool()) {
    gen = sc.mis_root->random(origin, rng);
  } else {
    if (srec.pdf == PDF_COSINE) gen = ONB(srec.pdf_w).local(random_cosine_direction(rng));
    else gen = random_unit_vector(rng);  // SpherePDF / ZeroPDF generate
  }
  Vec3 direction = normalize(gen);
  Ray sray{origin, direction, ray.time, ray.wavelength};
  Float light_v = sc.mis_root->pdf_value(origin, direction, hero, ray.time, &rng);
  Float bsdf_v;
  if (srec.pdf == PDF_COSINE) {
    Float cosine = dot(normalize(direction), srec.pdf_w);
    bsdf_v = cosine <= FL(0.0) ? FL(0.0) : cosine / PI;
  } else if (srec.pdf == PDF_SPHERE) {
    bsdf_v = FL(1.0) / (FL(4.0) * PI);
  } else {
    bsdf_v = FL(0.0);
  }
  Float mis = FL(0.5) * light_v + FL(0.5) * bsdf_v;
  Float spdf;
  if (!m->scattering_pdf(rec, sray, spdf)) {
    for (int i = 0; i < 4; ++i) out[i] = emitted[i];
    return;
  }
  Float rec4[4];
  trace(sray, sc, depth + 1, max_depth, rng, rec4);
  for (int i = 0; i < 4; ++i) out[i] = emitted[i] + rec4[i] * atten[i] * spdf / mis;
}

static Float cmf_table[400][3];
static bool cmf_ready = false;
static void ensure_cmf() {
  if (cmf_ready) return;
  for (int i = 0; i < 400; ++i) wavelength_into_xyz(380 + i, cmf_table[i]);
  cmf_ready = true;
}

// One sample's camera ray and wavelengths (clovers-cli/src/draw_cpu.rs:113-128,
// sampler/random.rs:20-32).  (x, r) are buffer coordinates: r = 0 is the top
// row, which the reference renders as camera row y = height-1 (draw_cpu.rs:51);
// the random stream is keyed by the buffer index r*width + x.
static Ray sample_ray(const Scene& sc, uint32_t x, uint32_t r, uint32_t width, uint32_t height, uint32_t sample,
                      uint64_t seed, Rng& rng) {
  rng = Rng(seed, r * width + x, sample);
  Float ox = rng.next_f32(), oy = rng.next_f32();
  Float lx, ly;
  random_in_unit_disk(rng, lx, ly);
  Float time = rng.next_f32();
  int lambda = random_wavelength(rng);
  uint32_t y = height - 1 - r;
  Float pu = ((Float)x + ox) / (Float)width;
  Float pv = ((Float)y + oy) / (Float)height;
  return sc.camera.get_ray(pu, pv, lx, ly, time, lambda);
}

// clovers-cli/src/draw_cpu.rs:101-146 for one pixel: the SUM of film deposits
// over `spp` samples, accumulated in f64 (the reference sums in f32 and then
// divides by spp).
static void render_pixel(const Scene& sc, uint32_t x, uint32_t r, uint32_t width, uint32_t height, uint32_t spp,
                         uint32_t max_depth, uint64_t seed, uint32_t sample_offset, double out[3]) {
  double acc[3] = {0, 0, 0};
  for (uint32_t s = 0; s < spp; ++s) {
    Rng rng(0, 0, 0);
    Ray ray = sample_ray(sc, x, r, width, height, s + sample_offset, seed, rng);
    int waves[4];
    rotate_wavelength(ray.wavelength, waves);
    Float p[4];
    trace(ray, sc, 0, max_depth, rng, p);
    if (p[1] == FL(0.0) && p[2] == FL(0.0) && p[3] == FL(0.0)) {
      const Float* c = cmf_table[waves[0] - 380];
      for (int k = 0; k < 3; ++k) acc[k] += (double)(c[k] * p[0]);
    } else {
      for (int i = 0; i < 4; ++i) {
        if (std::isnormal(p[i]) && p[i] > FL(0.0)) {
          const Float* c = cmf_table[waves[i] - 380];
          for (int k = 0; k < 3; ++k) acc[k] += (double)(c[k] * p[i] / FL(4.0));
        }
      }
    }
  }
  for (int k = 0; k < 3; ++k) out[k] = acc[k];
}

template <class F>
static void parallel_for(uint64_t n, int threads, F fn) {
  if (threads <= 1 || n < 2) {
    for (uint64_t i = 0; i < n; ++i) fn(i);
    return;
  }
  std::atomic<uint64_t> next(0);
  std::vector<std::thread> pool;
  for (int t = 0; t < threads; ++t)
    pool.emplace_back([&]() {
      while (true) {
        uint64_t i = next.fetch_add(1);
        if (i >= n) break;
        fn(i);
      }
    });
  for (auto& th : pool) th.join();
}

}  // namespace orc

// ================================================================ C ABI ===
using namespace orc;

static thread_local std::string g_err;

extern "C" {

const char* orc_last_error() { return g_err.c_str(); }

int orc_spectral_power(float x, float y, float z, int lambda, float* out) {
  try {
    Float xyz[3] = {x, y, z};
    *out = spectral_power(xyz, lambda);
    return 0;
  } catch (std::exception& e) {
    g_err = e.what();
    return -1;
  }
}
void orc_wavelength_into_xyz(int lambda, float out[3]) {
  Float o[3];
  wavelength_into_xyz(lambda, o);
  for (int k = 0; k < 3; ++k) out[k] = (float)o[k];
}
void orc_rotate_wavelength(int hero, int out[4]) { rotate_wavelength(hero, out); }
void orc_srgb_to_xyz_e(const float rgb[3], float out[3]) {
  const Float in[3] = {rgb[0], rgb[1], rgb[2]};
  Float o[3];
  srgb_to_xyz_e(in, o);
  for (int k = 0; k < 3; ++k) out[k] = (float)o[k];
}
void orc_xyz_e_to_srgb8(const float* xyz, uint64_t n, uint8_t* rgb) {
  for (uint64_t i = 0; i < n; ++i) {
    const Float in[3] = {xyz[3 * i], xyz[3 * i + 1], xyz[3 * i + 2]};
    xyz_e_to_srgb8(in, rgb + 3 * i);
  }
}
// Interval / AABB known-answer helpers: box = {xmin,xmax,ymin,ymax,zmin,zmax} (Interval::new order-normalises)
float orc_aabb_area(const float b[6]) {
  AABB a(Interval(b[0], b[1]), Interval(b[2], b[3]), Interval(b[4], b[5]));
  return a.area();
}
void orc_aabb_centroid(const float b[6], float out[3]) {
  AABB a(Interval(b[0], b[1]), Interval(b[2], b[3]), Interval(b[4], b[5]));
  Vec3 c = a.centroid();
  out[0] = c.x; out[1] = c.y; out[2] = c.z;
}
void orc_aabb_combine(const float a[6], const float b[6], float out[6]) {
  AABB x(Interval(a[0], a[1]), Interval(a[2], a[3]), Interval(a[4], a[5]));
  AABB y(Interval(b[0], b[1]), Interval(b[2], b[3]), Interval(b[4], b[5]));
  AABB c = AABB::combine(x, y);
  float r[6] = {c.x.min, c.x.max, c.y.min, c.y.max, c.z.min, c.z.max};
  std::memcpy(out, r, sizeof r);
}
// ray = {ox,oy,oz,tmin,dx,dy,dz,tmax}
int orc_aabb_hit(const float b[6], const float ray[8]) {
  AABB a(Interval(b[0], b[1]), Interval(b[2], b[3]), Interval(b[4], b[5]));
  Ray r{Vec3(ray[0], ray[1], ray[2]), Vec3(ray[4], ray[5], ray[6]), FL(0.0), 600};
  return a.hit(r, ray[3], ray[7]) ? 1 : 0;
}
void orc_interval(float a, float b, float out[4]) {
  Interval i(a, b);
  out[0] = i.min; out[1] = i.max; out[2] = i.size(); out[3] = i.center();
}
// Triangle (kind 1) / Quad (kind 2) / Sphere (kind 3: q=center, u.x=radius) primitive test.
// rec_out = {t, px,py,pz, nx,ny,nz, u,v, front_face}; box_out = padded AABB.
int orc_prim_hit(int kind, const float q[3], const float u[3], const float v[3], const float ray[8], float rec_out[10],
                 float box_out[6]) {
  Material m;
  std::unique_ptr<Hitable> h;
  if (kind == 1 || kind == 2)
    h.reset(new Planar(Vec3(q[0], q[1], q[2]), Vec3(u[0], u[1], u[2]), Vec3(v[0], v[1], v[2]), &m, kind == 1));
  else
    h.reset(new Sphere(Vec3(q[0], q[1], q[2]), u[0], &m));
  const AABB* b = h->aabb();
  float bb[6] = {b->x.min, b->x.max, b->y.min, b->y.max, b->z.min, b->z.max};
  std::memcpy(box_out, bb, sizeof bb);
  Ray r{Vec3(ray[0], ray[1], ray[2]), Vec3(ray[4], ray[5], ray[6]), FL(0.0), 600};
  HitRecord rec;
  if (!h->hit(r, ray[3], ray[7], nullptr, rec, nullptr)) return 0;
  float o[10] = {rec.distance, rec.position.x, rec.position.y, rec.position.z, rec.normal.x, rec.normal.y,
                 rec.normal.z, rec.u, rec.v, rec.front_face ? FL(1.0) : FL(0.0)};
  std::memcpy(rec_out, o, sizeof o);
  return 1;
}

// bvh: 0 longest axis midpoint, 1 surface area heuristic (BvhAlgorithm, bvh.rs:30-39)
void* orc_scene_load_json_bvh(const char* path, uint32_t width, uint32_t height, int bvh) {
  try {
    std::ifstream f(path);
    if (!f) throw std::runtime_error(std::string("cannot open scene file ") + path);
    std::stringstream ss;
    ss << f.rdbuf();
    std::string p(path);
    size_t slash = p.find_last_of('/');
    return load_scene(ss.str(), width, height, slash == std::string::npos ? std::string(".") : p.substr(0, slash),
                      bvh == 0);
  } catch (std::exception& e) {
    g_err = e.what();
    return nullptr;
  }
}
void* orc_scene_load_json(const char* path, uint32_t width, uint32_t height) {
  try {
    std::ifstream f(path);
    if (!f) throw std::runtime_error(std::string("cannot open scene file ") + path);
    std::stringstream ss;
    ss << f.rdbuf();
    std::string p(path);
    size_t slash = p.find_last_of('/');
    return load_scene(ss.str(), width, height, slash == std::string::npos ? std::string(".") : p.substr(0, slash));
  } catch (std::exception& e) {
    g_err = e.what();
    return nullptr;
  }
}
void* orc_scene_from_mesh(const float* verts, uint32_t nverts, const uint32_t* idx, uint32_t ntris) {
  try {
    return mesh_scene(verts, nverts, idx, ntris);
  } catch (std::exception& e) {
    g_err = e.what();
    return nullptr;
  }
}
void orc_scene_free(void* s) { delete static_cast<Scene*>(s); }
// the optional watertight triangle test on every triangle of the scene
void orc_scene_set_watertight(void* s, int on) {
  Scene* sc = static_cast<Scene*>(s);
  if (sc->bvh_root) sc->bvh_root->set_watertight(on != 0);
  if (sc->mis_root) sc->mis_root->set_watertight(on != 0);
}

static void tree_stats(const Hitable* h, uint32_t depth, uint64_t& nodes, uint32_t& max_depth) {
  if (!h->is_bvh()) return;
  const BVHNode* n = static_cast<const BVHNode*>(h);
  nodes++;
  if (depth > max_depth) max_depth = depth;
  tree_stats(n->left.get(), depth + 1, nodes, max_depth);
  tree_stats(n->right.get(), depth + 1, nodes, max_depth);
}
// Shape of the main BVH: BVHNode count and depth (root = 1); MIS tree node count.
void orc_scene_tree_stats(void* s, uint64_t out[3]) {
  Scene* sc = static_cast<Scene*>(s);
  uint64_t n = 0, m = 0;
  uint32_t d = 0, md = 0;
  tree_stats(sc->bvh_root.get(), 1, n, d);
  if (sc->mis_root) tree_stats(sc->mis_root.get(), 1, m, md);
  out[0] = n; out[1] = d; out[2] = m;
}
uint64_t orc_scene_object_count(void* s) { return static_cast<Scene*>(s)->object_count; }

// Camera rays for given sample parameters (parity of the ray generator).
void orc_camera_ray(void* s, float pu, float pv, float lx, float ly, float out[6]) {
  Ray r = static_cast<Scene*>(s)->camera.get_ray(pu, pv, lx, ly, FL(0.0), 600);
  float o[6] = {r.origin.x, r.origin.y, r.origin.z, r.direction.x, r.direction.y, r.direction.z};
  std::memcpy(out, o, sizeof o);
}

// Background and per-wavelength tables, for comparison with the product's uploaded tables.
void orc_scene_background_xyz(void* s, float out[3]) {
  Scene* sc = static_cast<Scene*>(s);
  for (int i = 0; i < 3; ++i) out[i] = sc->background[i];
}


// Closest-hit ray cast, rays = n x {ox,oy,oz,tmin,dx,dy,dz,tmax}.  prim = top-level
// object index or 0xFFFFFFFF; counters (optional) = BVHNode::hit calls and primitive tests.
int orc_raycast(void* s, const float* rays, uint64_t n, uint32_t* prim, float* t, uint32_t* nodes, uint32_t* prims,
                int threads) {
  Scene* sc = static_cast<Scene*>(s);
  std::string err;
  parallel_for((n + 1023) / 1024, threads, [&](uint64_t blk) {
    uint64_t e = std::min<uint64_t>(n, (blk + 1) * 1024);
    for (uint64_t i = blk * 1024; i < e; ++i) {
      const float* r = rays + 8 * i;
      Ray ray{Vec3(r[0], r[1], r[2]), Vec3(r[4], r[5], r[6]), FL(0.0), 600};
      HitRecord rec;
      Counters c;
      Rng rng(0, (uint32_t)i, 0);
      bool h = sc->bvh_root->hit(ray, r[3], r[7], &rng, rec, &c);
      prim[i] = h ? (uint32_t)rec.gid : 0xFFFFFFFFu;
      t[i] = h ? rec.distance : FL(0.0);
      if (nodes) nodes[i] = (uint32_t)c.nodes;
      if (prims) prims[i] = (uint32_t)c.prims;
    }
  });
  return 0;
}

// Path-traced film: xyz_out[(r-r0)*(x1-x0)+(x-x0)] = SUM over spp of the film
// deposits of pixel (x, r) in buffer coordinates (row 0 = top, the reference's
// pixelbuffer order); divide by spp for the reference's mean.  Rows are the
// parallel unit, as in clovers-cli/src/draw_cpu.rs:53-55.
int orc_render(void* s, uint32_t width, uint32_t height, uint32_t spp, uint32_t max_depth, uint64_t seed,
               uint32_t x0, uint32_t r0, uint32_t x1, uint32_t r1, uint32_t sample_offset, double* xyz_out,
               int threads) {
  try {
    Scene* sc = static_cast<Scene*>(s);
    ensure_cmf();
    if (x1 > width || r1 > height || x0 >= x1 || r0 >= r1) throw std::runtime_error("bad crop window");
    uint32_t cw = x1 - x0;
    std::atomic<int> failed(0);
    std::string msg;
    parallel_for(r1 - r0, threads, [&](uint64_t row) {
      uint32_t r = r0 + (uint32_t)row;
      try {
        for (uint32_t x = x0; x < x1; ++x)
          render_pixel(*sc, x, r, width, height, spp, max_depth, seed, sample_offset,
                       xyz_out + 3 * ((uint64_t)row * cw + (x - x0)));
      } catch (std::exception& e) {
        if (!failed.exchange(1)) msg = e.what();
      }
    });
    if (failed) throw std::runtime_error(msg);
    return 0;
  } catch (std::exception& e) {
    g_err = e.what();
    return -1;
  }
}

// The per-pixel sums of film deposits for a list of buffer pixels (index
// r * width + x), e.g. a stratified subset of the image; one work unit per pixel.
int orc_render_pixels(void* s, uint32_t width, uint32_t height, uint32_t spp, uint32_t max_depth, uint64_t seed,
                      const uint32_t* pixels, uint64_t n, uint32_t sample_offset, double* xyz_out, int threads) {
  try {
    Scene* sc = static_cast<Scene*>(s);
    ensure_cmf();
    for (uint64_t i = 0; i < n; ++i)
      if (pixels[i] >= (uint64_t)width * height) throw std::runtime_error("pixel index outside the image");
    std::atomic<int> failed(0);
    std::string msg;
    parallel_for(n, threads, [&](uint64_t i) {
      try {
        render_pixel(*sc, pixels[i] % width, pixels[i] / width, width, height, spp, max_depth, seed, sample_offset,
                     xyz_out + 3 * i);
      } catch (std::exception& e) {
        if (!failed.exchange(1)) msg = e.what();
      }
    });
    if (failed) throw std::runtime_error(msg);
    return 0;
  } catch (std::exception& e) {
    g_err = e.what();
    return -1;
  }
}

// ln of n f32 values through the render path's logarithm (clv_log.h), the
// routine the GPU's media use.
void orc_log_f32(const float* x, uint64_t n, float* y) {
  for (uint64_t i = 0; i < n; ++i) y[i] = clv_math::log_f32(x[i]);
}

// Debug render modes (clovers-cli/src/draw_cpu.rs:148-207): one ray per pixel
// through its corner (x / width, y / height), no lens offset, with a drawn
// wavelength and time.  Mode 1 colours the hit normal (normals.rs:11-37),
// modes 2 and 3 the BVH node and primitive test counts through the ramp of
// debug_visualizations.rs:18-35.  Writes linear sRGB per buffer pixel (row 0
// at the top of the image, like the path tracer's film).
int orc_render_debug(void* s, uint32_t width, uint32_t height, uint32_t mode, uint64_t seed, uint32_t sample_offset,
                     float* rgb_out, int threads) {
  try {
    Scene* sc = static_cast<Scene*>(s);
    if (mode < 1 || mode > 3) throw std::runtime_error("debug mode must be 1, 2 or 3");
    parallel_for(height, threads, [&](uint64_t row) {
      for (uint32_t x = 0; x < width; ++x) {
        const uint64_t pix = row * width + x;
        const uint32_t y = height - 1 - (uint32_t)row;
        Rng rng(seed, (uint32_t)pix, sample_offset);
        const int lambda = random_wavelength(rng);
        const Float time = rng.next_f32();
        const Ray ray = sc->camera.get_ray((Float)x / (Float)width, (Float)y / (Float)height, FL(0.0), FL(0.0), time, lambda);
        HitRecord rec;
        Counters c;
        const bool any = sc->bvh_root->hit(ray, EPSILON_SHADOW_ACNE, FL(3.40282347e+38), &rng, rec, &c);
        float* o = rgb_out + 3 * pix;
        o[0] = o[1] = o[2] = FL(0.0);
        if (mode == 1) {
          if (any) {
            const Vec3 n{-rec.normal.x, rec.normal.y, -rec.normal.z};
            o[0] = FL(0.5) + FL(0.5) * n.x;
            o[1] = FL(0.5) + FL(0.5) * n.y;
            o[2] = n.z < FL(0.0) ? FL(0.0) : n.z;
          }
        } else {
          const uint64_t d = mode == 2 ? c.nodes : c.prims;
          if (d <= 255) {
            o[0] = o[1] = o[2] = (Float)d / FL(255.0);
          } else if (d <= 511) {
            o[0] = FL(1.0);
            o[1] = FL(1.0);
          } else if (d <= 1023) {
            o[0] = FL(1.0);
            o[1] = FL(0.5);
          } else {
            o[0] = FL(1.0);
          }
        }
      }
    });
    return 0;
  } catch (std::exception& e) {
    g_err = e.what();
    return -1;
  }
}

// One path's spectral powers (trace.rs return value) for buffer pixel (x, r), sample index.
int orc_trace_sample(void* s, uint32_t width, uint32_t height, uint32_t x, uint32_t r, uint32_t sample,
                     uint32_t max_depth, uint64_t seed, float p_out[4], int waves_out[4], float ray_out[6]) {
  try {
    Scene* sc = static_cast<Scene*>(s);
    Rng rng(0, 0, 0);
    Ray ray = sample_ray(*sc, x, r, width, height, sample, seed, rng);
    float ro[6] = {ray.origin.x, ray.origin.y, ray.origin.z, ray.direction.x, ray.direction.y, ray.direction.z};
    std::memcpy(ray_out, ro, sizeof ro);
    rotate_wavelength(ray.wavelength, waves_out);
    Float p[4];
    trace(ray, *sc, 0, max_depth, rng, p);
    for (int k = 0; k < 4; ++k) p_out[k] = (float)p[k];
    return 0;
  } catch (std::exception& e) {
    g_err = e.what();
    return -1;
  }
}

}  // extern "C"
