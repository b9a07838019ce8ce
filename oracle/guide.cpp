// CPU oracle of the path guide -- TEST INFRASTRUCTURE ONLY.
//
// The reference renderer has no path guiding, so there is no reference code
// to follow here: this file restates the guide's specification (the network,
// the von Mises-Fisher mixture head, its sampling rule and the gradient of
// the training loss -f log q) in double precision, independently of the CUDA
// kernels, so the tests can check the tensor-core forward and backward passes.
// With bf16 = 1 it rounds operands to bfloat16 at the points where the GPU
// kernels store them for the tensor cores (encoded inputs, weights, hidden
// activations, output and hidden-layer gradients); with bf16 = 0 everything
// stays in double, which is what the finite-difference checks use.
//
// Specification:
//   u[7] in [0,1] -> x[176]: x[24j+2k] = sin(2^k pi u_j), x[24j+2k+1] =
//   cos(2^k pi u_j) (k < 12, double-angle recurrence in f32 from sin/cos of
//   pi u_j), x[168+j] = u_j, x[175] = 1;  h1 = relu(W1 x), h2 = relu(W2 h1),
//   h3 = relu(W3 h2) with unit 63 of each forced to 1;  o = W4 h3 (40).
//   Lobe k: mu = o[5k..5k+2] / |.|, kappa = exp(clamp(o[5k+3], -3, 8)),
//   weight = softmax(o[5k+4]);  vMF density kappa / (2 pi (1 - e^{-2 kappa}))
//   * exp(kappa (mu.w - 1)).
#include <cmath>
#include <cstdint>
#include <cstring>
#include <vector>

namespace {

constexpr int IN = 176, H = 64, OUT = 40, LOBES = 8, FREQ = 12;
constexpr int P_W1 = 0, P_W2 = H * IN, P_W3 = P_W2 + H * H, P_W4 = P_W3 + H * H, NPARAM = P_W4 + OUT * H;
constexpr double LOGK_MIN = -3.0, LOGK_MAX = 8.0;
constexpr double TWO_PI = 6.283185307179586476925286766559;

// round-to-nearest-even to bfloat16, returned as float
float bf16(float x) {
  uint32_t u;
  std::memcpy(&u, &x, 4);
  if ((u & 0x7F800000u) == 0x7F800000u) return x;  // inf / nan unchanged
  const uint32_t lsb = (u >> 16) & 1u;
  u += 0x7FFFu + lsb;
  u &= 0xFFFF0000u;
  float r;
  std::memcpy(&r, &u, 4);
  return r;
}
double rnd(double x, int b) { return b ? (double)bf16((float)x) : x; }

void encode(const float* u, int b, double* x) {
  for (int j = 0; j < 7; ++j) {
    float s = (float)std::sin(M_PI * (double)u[j]);
    float c = (float)std::cos(M_PI * (double)u[j]);
    x[24 * j] = s;
    x[24 * j + 1] = c;
    for (int k = 1; k < FREQ; ++k) {
      const float s2 = (2.0f * s) * c;
      const float c2 = std::fma(-2.0f * s, s, 1.0f);
      s = s2;
      c = c2;
      x[24 * j + 2 * k] = s;
      x[24 * j + 2 * k + 1] = c;
    }
  }
  for (int j = 0; j < 7; ++j) x[168 + j] = u[j];
  x[175] = 1.0;
  for (int i = 0; i < IN; ++i) x[i] = rnd(x[i], b);
}

struct Net {
  std::vector<double> w;  // parameters, rounded if bf16
  explicit Net(const float* p, int b) : w(NPARAM) {
    for (int i = 0; i < NPARAM; ++i) w[i] = rnd(p[i], b);
  }
};

// forward pass of one input; keeps the activations for the backward pass
struct Acts {
  double x[IN], h[3][H], o[OUT];
  bool mask[3][H];
};
void forward(const Net& N, const float* u, int b, Acts& A) {
  encode(u, b, A.x);
  const double* in = A.x;
  int nin = IN;
  const int off[3] = {P_W1, P_W2, P_W3};
  for (int l = 0; l < 3; ++l) {
    for (int o = 0; o < H; ++o) {
      double z = 0.0;
      for (int k = 0; k < nin; ++k) z += N.w[off[l] + o * nin + k] * in[k];
      const double zz = b ? (double)(float)z : z;  // the GPU accumulates in f32
      double h = zz > 0.0 ? zz : 0.0;
      if (o == H - 1) h = 1.0;
      A.mask[l][o] = h > 0.0;
      A.h[l][o] = rnd(h, b);
    }
    in = A.h[l];
    nin = H;
  }
  for (int o = 0; o < OUT; ++o) {
    double z = 0.0;
    for (int k = 0; k < H; ++k) z += N.w[P_W4 + o * H + k] * A.h[2][k];
    A.o[o] = b ? (double)(float)z : z;
  }
}

struct Mix {
  double mu[LOBES][3], kap[LOBES], w[LOBES], nrm[LOBES], mlen[LOBES];
  bool clamped[LOBES];
};
void make_mix(const double* o, Mix& m) {
  double mx = -1e300;
  for (int k = 0; k < LOBES; ++k) mx = std::fmax(mx, o[5 * k + 4]);
  double sum = 0.0;
  for (int k = 0; k < LOBES; ++k) {
    const double x = o[5 * k], y = o[5 * k + 1], z = o[5 * k + 2];
    const double l = std::sqrt(x * x + y * y + z * z);
    if (l > 1e-6) {
      m.mu[k][0] = x / l;
      m.mu[k][1] = y / l;
      m.mu[k][2] = z / l;
      m.mlen[k] = l;
    } else {
      m.mu[k][0] = 0.0;
      m.mu[k][1] = 0.0;
      m.mu[k][2] = 1.0;
      m.mlen[k] = 1e-6;
    }
    double lk = o[5 * k + 3];
    m.clamped[k] = !(lk >= LOGK_MIN && lk <= LOGK_MAX);
    if (m.clamped[k]) lk = lk > LOGK_MAX ? LOGK_MAX : LOGK_MIN;
    m.kap[k] = std::exp(lk);
    m.nrm[k] = m.kap[k] / (TWO_PI * -std::expm1(-2.0 * m.kap[k]));
    m.w[k] = std::exp(o[5 * k + 4] - mx);
    sum += m.w[k];
  }
  for (int k = 0; k < LOBES; ++k) m.w[k] /= sum;
}
double mix_pdf(const Mix& m, const double* d, double* v) {
  double q = 0.0;
  for (int k = 0; k < LOBES; ++k) {
    const double c = m.mu[k][0] * d[0] + m.mu[k][1] * d[1] + m.mu[k][2] * d[2];
    v[k] = m.nrm[k] * std::exp(m.kap[k] * (c - 1.0));
    q += m.w[k] * v[k];
  }
  return q;
}
// d(-f log q)/do; returns -f log q
double mix_grad(const Mix& m, const double* d, double f, double* g) {
  double v[LOBES];
  const double q = std::fmax(mix_pdf(m, d, v), 1e-300);
  const double s = -f / q;
  for (int k = 0; k < LOBES; ++k) {
    const double kap = m.kap[k];
    const double c = m.mu[k][0] * d[0] + m.mu[k][1] * d[1] + m.mu[k][2] * d[2];
    const double a = s * m.w[k] * v[k];
    g[5 * k + 4] = a - s * m.w[k] * q;
    g[5 * k + 3] = m.clamped[k] ? 0.0 : a * (1.0 / kap - 2.0 / std::expm1(2.0 * kap) + c - 1.0) * kap;
    const double t = a * kap / m.mlen[k];
    for (int e = 0; e < 3; ++e) g[5 * k + e] = t * (d[e] - m.mu[k][e] * c);
  }
  return f > 0.0 ? -f * std::log(q) : 0.0;
}

}  // namespace

extern "C" {

void orc_guide_forward(const float* params, const float* queries, uint64_t n, int b, float* out) {
  const Net N(params, b);
  Acts A;
  for (uint64_t i = 0; i < n; ++i) {
    forward(N, queries + 8 * i, b, A);
    for (int o = 0; o < OUT; ++o) out[OUT * i + o] = (float)A.o[o];
  }
}

// Gradient sums over the records (12 floats each: u[7], -, w.xyz, f) of the
// loss -f log q(w); returns the loss sum.
double orc_guide_gradient(const float* params, const float* records, uint64_t n, int b, double* grads) {
  const Net N(params, b);
  std::memset(grads, 0, sizeof(double) * NPARAM);
  double loss = 0.0;
  Acts A;
  for (uint64_t r = 0; r < n; ++r) {
    const float* R = records + 12 * r;
    const double f = R[11] > 0.0f && std::isfinite(R[11]) ? R[11] : 0.0;
    if (f == 0.0) continue;
    forward(N, R, b, A);
    Mix m;
    make_mix(A.o, m);
    const double d[3] = {R[8], R[9], R[10]};
    double go[OUT];
    loss += mix_grad(m, d, f, go);
    for (int o = 0; o < OUT; ++o) go[o] = rnd(go[o], b);
    // layer 4
    double dh[H], dz[H];
    for (int k = 0; k < H; ++k) {
      double s = 0.0;
      for (int o = 0; o < OUT; ++o) {
        grads[P_W4 + o * H + k] += go[o] * A.h[2][k];
        s += go[o] * N.w[P_W4 + o * H + k];
      }
      dh[k] = b ? (double)(float)s : s;
    }
    const int off[3] = {P_W1, P_W2, P_W3};
    for (int l = 2; l >= 0; --l) {
      for (int k = 0; k < H; ++k) dz[k] = rnd(k != H - 1 && A.mask[l][k] ? dh[k] : 0.0, b);
      const double* in = l == 0 ? A.x : A.h[l - 1];
      const int nin = l == 0 ? IN : H;
      for (int o = 0; o < H; ++o)
        for (int k = 0; k < nin; ++k) grads[off[l] + o * nin + k] += dz[o] * in[k];
      if (l > 0) {
        for (int k = 0; k < H; ++k) {
          double s = 0.0;
          for (int o = 0; o < H; ++o) s += dz[o] * N.w[off[l] + o * H + k];
          dh[k] = b ? (double)(float)s : s;
        }
      }
    }
  }
  return loss;
}

// Mixture density at unit direction w of one output vector.
double orc_guide_pdf(const float* out40, const float* w) {
  double o[OUT], d[3] = {w[0], w[1], w[2]}, v[LOBES];
  for (int i = 0; i < OUT; ++i) o[i] = out40[i];
  Mix m;
  make_mix(o, m);
  return mix_pdf(m, d, v);
}

// Lobe by u0 (first k whose cumulative weight exceeds u0), then Jakob's vMF
// sample with (u1, u2) in the branchless frame of Duff et al. 2017.
void orc_guide_sample(const float* out40, float u0, float u1, float u2, float* w) {
  double o[OUT];
  for (int i = 0; i < OUT; ++i) o[i] = out40[i];
  Mix m;
  make_mix(o, m);
  int k = LOBES - 1;
  double acc = 0.0;
  for (int j = 0; j < LOBES - 1; ++j) {
    acc += m.w[j];
    if (u0 < acc) {
      k = j;
      break;
    }
  }
  const double kap = m.kap[k];
  double W = 1.0 + std::log(u1 + (1.0 - u1) * std::exp(-2.0 * kap)) / kap;
  W = std::fmin(1.0, std::fmax(-1.0, W));
  const double sw = std::sqrt(std::fmax(0.0, 1.0 - W * W));
  const double ph = TWO_PI * u2, cp = std::cos(ph), sp = std::sin(ph);
  const double mx = m.mu[k][0], my = m.mu[k][1], mz = m.mu[k][2];
  const double sg = std::copysign(1.0, mz), a = -1.0 / (sg + mz), bb = mx * my * a;
  const double t[3] = {1.0 + sg * mx * mx * a, sg * bb, -sg * mx};
  const double bv[3] = {bb, sg + my * my * a, -my};
  double r[3];
  for (int e = 0; e < 3; ++e) r[e] = W * m.mu[k][e] + sw * (cp * t[e] + sp * bv[e]);
  const double l = std::sqrt(r[0] * r[0] + r[1] * r[1] + r[2] * r[2]);
  for (int e = 0; e < 3; ++e) w[e] = (float)(r[e] / l);
}

}  // extern "C"
