// Host-side spectral and colour conversions used when a scene is flattened:
// every colour of the scene becomes a 400-entry f32 spectral power table
// (one entry per integer wavelength 380..779 nm), so the device never runs the
// f64 grid uplift or the colour-space maths.
//
//  * spectral_power: clovers/src/spectrum.rs:46-56 over the Meng et al. 2015
//    grid, clovers/src/spectrum/spectrum_grid.rs:16-153 (f64).
//  * wavelength_to_xyz: the analytic CIE 1931 fit, clovers/src/wavelength.rs:63-83.
//  * sRGB <-> XYZ(E): what the reference takes from the palette crate
//    (clovers/src/colorinit.rs:45-60, clovers-cli/src/scenefile.rs:43-44,
//    clovers-cli/src/write.rs:39-44): IEC 61966-2-1 transfer curve, the sRGB
//    primaries with the D65 white (0.95047, 1, 1.08883) and Bradford
//    adaptation between D65 and E, composed in f64 and applied in f64.
#pragma once

#include <cmath>
#include <cstdint>
#include <stdexcept>

#include "spectral_tables.h"

namespace clv {

struct SpectralError : std::runtime_error {
  using std::runtime_error::runtime_error;
};

// f64 evaluation of the Meng et al. grid at one wavelength.
inline double grid_power(double lambda, const double xyz[3]) {
  using namespace clv_tables;
  const double sum = xyz[0] + xyz[1] + xyz[2];
  const double inv = 1.0 / sum;
  if (!(inv < 1.7976931348623157e308)) return 0.0;
  const double cx = xyz[0] * inv, cy = xyz[1] * inv;
  double u = kXyToUv[0] * cx + kXyToUv[1] * cy + kXyToUv[2];
  double v = kXyToUv[3] * cx + kXyToUv[4] * cy + kXyToUv[5];
  if (u < 0.0 || u >= 12.0 || v < 0.0 || v >= 14.0) return 0.0;
  const int iu = (int)u, iv = (int)v;
  const GridCell& cell = kGrid[iu + 12 * iv];
  const int n = cell.num_points;
  if (n == 0) throw SpectralError("colour falls in an empty cell of the spectral uplift grid");
  // linear interpolation of each corner spectrum at lambda (81 samples, 5 nm)
  const double pos = (lambda - 380.0) / (780.0 - 380.0) * (81.0 - 1.0);
  const int s0 = (int)pos;
  const int s1 = s0 + 1 < 81 ? s0 + 1 : 80;
  const double fr = pos - (double)s0;
  double p[6];
  for (int i = 0; i < n; ++i) {
    const double* sp = kPoints[cell.idx[i]].spectrum;
    p[i] = sp[s0] * (1.0 - fr) + sp[s1] * fr;
  }
  double r = 0.0;
  if (cell.inside == 1) {
    u -= (double)iu;
    v -= (double)iv;
    // corner layout 2 3 / 0 1
    r = p[0] * (1.0 - u) * (1.0 - v) + p[2] * (1.0 - u) * v + p[3] * u * v + p[1] * u * (1.0 - v);
  } else {
    // triangle fan around corner 0: find the triangle holding (u, v)
    const double* c0 = kPoints[cell.idx[0]].uv;
    const double ex = u - c0[0], ey = v - c0[1];
    double ax = kPoints[cell.idx[1]].uv[0] - c0[0];
    double ay = kPoints[cell.idx[1]].uv[1] - c0[1];
    double bu = ax * ey - ex * ay;
    for (int i = 0; i + 1 < n; ++i) {
      const int nxt = (i == n - 2) ? 1 : i + 2;
      const double bx = kPoints[cell.idx[nxt]].uv[0] - c0[0];
      const double by = kPoints[cell.idx[nxt]].uv[1] - c0[1];
      const double bv = ex * by - bx * ey;
      const double area = ax * by - bx * ay;
      const double wu = bu / area, wv = bv / area;
      const double ww = 1.0 - wu - wv;
      if (wu < 0.0 || wv < 0.0 || ww < 0.0) {
        bu = -bv;
        ax = bx;
        ay = by;
        continue;
      }
      r = p[0] * ww + p[i + 1] * wv + p[nxt] * wu;
      break;
    }
  }
  return r / inv;
}

inline float spectral_power(const float xyz[3], int lambda) {
  const double d[3] = {(double)xyz[0], (double)xyz[1], (double)xyz[2]};
  return (float)(grid_power((double)lambda, d) / clv_tables::kEqualEnergyReflectance);
}

inline void spd_table(const float xyz[3], float out[400]) {
  for (int i = 0; i < 400; ++i) out[i] = spectral_power(xyz, 380 + i);
}

inline float cie_lobe(float x, float alpha, float mu, float s1, float s2) {
  const float t = (x - mu) / (x < mu ? s1 : s2);
  return alpha * std::exp(-(t * t) / 2.0f);
}
inline void wavelength_to_xyz(int lambda, float out[3]) {
  const float l = (float)lambda;
  out[0] = 0.0f + cie_lobe(l, 1.056f, 599.8f, 37.9f, 31.0f) + cie_lobe(l, 0.362f, 442.0f, 16.0f, 26.7f) +
           cie_lobe(l, -0.065f, 501.1f, 20.4f, 26.2f);
  out[1] = cie_lobe(l, 0.821f, 568.8f, 46.9f, 40.5f) + cie_lobe(l, 0.286f, 530.9f, 16.3f, 31.1f);
  out[2] = cie_lobe(l, 1.217f, 437.0f, 11.8f, 36.0f) + cie_lobe(l, 0.681f, 459.0f, 26.0f, 13.8f);
}

// ---- colour spaces (3x3 matrices, row-major, f64)
inline void m3_mul(const double a[9], const double b[9], double o[9]) {
  for (int r = 0; r < 3; ++r)
    for (int c = 0; c < 3; ++c) o[r * 3 + c] = a[r * 3] * b[c] + a[r * 3 + 1] * b[3 + c] + a[r * 3 + 2] * b[6 + c];
}
inline void m3_inv(const double m[9], double o[9]) {
  const double a = m[0], b = m[1], c = m[2], d = m[3], e = m[4], f = m[5], g = m[6], h = m[7], i = m[8];
  const double A = e * i - f * h, B = -(d * i - f * g), C = d * h - e * g;
  const double det = a * A + b * B + c * C;
  o[0] = A / det; o[1] = -(b * i - c * h) / det; o[2] = (b * f - c * e) / det;
  o[3] = B / det; o[4] = (a * i - c * g) / det; o[5] = -(a * f - c * d) / det;
  o[6] = C / det; o[7] = -(a * h - b * g) / det; o[8] = (a * e - b * d) / det;
}
// linear sRGB -> XYZ with the D65 white, from the primaries' chromaticities
inline void m3_linsrgb_to_xyz(double m[9]) {
  const double xr = 0.64, yr = 0.33, xg = 0.30, yg = 0.60, xb = 0.15, yb = 0.06;
  const double W[3] = {0.95047, 1.0, 1.08883};
  const double P[9] = {xr / yr, xg / yg, xb / yb, 1.0, 1.0, 1.0,
                       (1 - xr - yr) / yr, (1 - xg - yg) / yg, (1 - xb - yb) / yb};
  double Pi[9], S[3];
  m3_inv(P, Pi);
  for (int r = 0; r < 3; ++r) S[r] = Pi[r * 3] * W[0] + Pi[r * 3 + 1] * W[1] + Pi[r * 3 + 2] * W[2];
  for (int r = 0; r < 3; ++r)
    for (int c = 0; c < 3; ++c) m[r * 3 + c] = P[r * 3 + c] * S[c];
}
// Bradford von-Kries adaptation between two white points
inline void m3_bradford(const double from[3], const double to[3], double o[9]) {
  const double M[9] = {0.8951, 0.2664, -0.1614, -0.7502, 1.7135, 0.0367, 0.0389, -0.0685, 1.0296};
  double Mi[9], s[3], d[3], t[9];
  m3_inv(M, Mi);
  for (int r = 0; r < 3; ++r) {
    s[r] = M[r * 3] * from[0] + M[r * 3 + 1] * from[1] + M[r * 3 + 2] * from[2];
    d[r] = M[r * 3] * to[0] + M[r * 3 + 1] * to[1] + M[r * 3 + 2] * to[2];
  }
  const double D[9] = {d[0] / s[0], 0, 0, 0, d[1] / s[1], 0, 0, 0, d[2] / s[2]};
  m3_mul(D, M, t);
  m3_mul(Mi, t, o);
}
static const double kWhiteD65[3] = {0.95047, 1.0, 1.08883};
static const double kWhiteE[3] = {1.0, 1.0, 1.0};

inline void m3_apply(const double m[9], const float in[3], float out[3]) {
  for (int r = 0; r < 3; ++r)
    out[r] = (float)(m[r * 3] * (double)in[0] + m[r * 3 + 1] * (double)in[1] + m[r * 3 + 2] * (double)in[2]);
}
inline float srgb_to_linear(float c) { return c <= 0.04045f ? c / 12.92f : std::pow((c + 0.055f) / 1.055f, 2.4f); }
inline float linear_to_srgb(float c) { return c <= 0.0031308f ? c * 12.92f : 1.055f * std::pow(c, 1.0f / 2.4f) - 0.055f; }

inline void linsrgb_to_xyz_e(const float lin[3], float out[3]) {
  double a[9], b[9], t[9];
  m3_linsrgb_to_xyz(a);
  m3_bradford(kWhiteD65, kWhiteE, b);
  m3_mul(b, a, t);
  m3_apply(t, lin, out);
}
inline void srgb_to_xyz_e(const float rgb[3], float out[3]) {
  const float lin[3] = {srgb_to_linear(rgb[0]), srgb_to_linear(rgb[1]), srgb_to_linear(rgb[2])};
  linsrgb_to_xyz_e(lin, out);
}
inline void xyz_d65_to_xyz_e(const float in[3], float out[3]) {
  double b[9];
  m3_bradford(kWhiteD65, kWhiteE, b);
  m3_apply(b, in, out);
}
// XYZ(E) -> linear sRGB (the first half of write.rs:41), as an f64 matrix
inline void m3_xyz_e_to_linsrgb(double o[9]) {
  double a[9], ai[9], b[9];
  m3_linsrgb_to_xyz(a);
  m3_inv(a, ai);
  m3_bradford(kWhiteE, kWhiteD65, b);
  m3_mul(ai, b, o);
}

}  // namespace clv
