// Tensor-core kernels of the path guide (network and training rule: guide.cuh).
//
//   guide_infer_kernel<QUEUE>  per 128 guided vertices: encode -> 4 layers on
//                              tcgen05.mma (BF16 x BF16 -> FP32 in TMEM) -> vMF
//                              head; samples the guided directions and returns
//                              the mixture density of every bounce direction
//   guide_infer_kernel<ARRAY>  same network on an array of inputs (tests)
//   guide_train_kernel         forward + backward of 128-record tiles; the
//                              weight gradients accumulate in TMEM over the
//                              tiles of a CTA and are added to global memory once
//   guide_adam_kernel          Adam step; rewrites the BF16 operand blob
//
// Operands live in shared memory in the no-swizzle K-major canonical layout
// (gd_cofs); the weights arrive by one bulk copy (cp.async.bulk) per CTA.  One
// thread issues the MMAs and commits them to an mbarrier; every wait on an
// mbarrier is bounded by a clock limit, after which the kernel raises
// CLV_ERR_GUIDE, frees its TMEM and returns.
#include <cuda_bf16.h>
#include <cuda_runtime.h>
#include <stdint.h>

#include <cmath>
#include <cstring>
#include <stdexcept>
#include <string>
#include <vector>

#include "clovers_gpu.h"
#include "guide.cuh"
#include "rng.cuh"

namespace gd {

// ------------------------------------------------------------ PTX wrappers --
__device__ __forceinline__ uint32_t smem_u32(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }

// Shared-memory matrix descriptor of tcgen05.mma: start address, leading
// (K-direction) and stride (M/N-direction) byte offsets, all >> 4; bit 46 is
// the descriptor version of this architecture; no swizzle, base offset 0.
__device__ __forceinline__ uint64_t sdesc(uint32_t saddr, uint32_t lbo, uint32_t sbo) {
  return (uint64_t)((saddr & 0x3FFFFu) >> 4) | ((uint64_t)((lbo & 0x3FFFFu) >> 4) << 16) |
         ((uint64_t)((sbo & 0x3FFFFu) >> 4) << 32) | (1ull << 46);
}
// Instruction descriptor of kind::f16: D f32 (bits 4-5 = 1), A and B bf16
// (bits 7-9 and 10-12 = 1), both K-major, N >> 3 at bit 17, M >> 4 at bit 24.
__host__ __device__ constexpr uint32_t idesc_bf16(uint32_t M, uint32_t N) {
  return (1u << 4) | (1u << 7) | (1u << 10) | ((N >> 3) << 17) | ((M >> 4) << 24);
}

__device__ __forceinline__ void mma_bf16(uint32_t d_tmem, uint64_t ad, uint64_t bd, uint32_t id, uint32_t acc) {
  asm volatile(
      "{\n\t.reg .pred p;\n\tsetp.ne.b32 p, %4, 0;\n\t"
      "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}"
      ::"r"(d_tmem), "l"(ad), "l"(bd), "r"(id), "r"(acc)
      : "memory");
}
// Arrives on the mbarrier once every MMA this thread issued has completed.
__device__ __forceinline__ void mma_commit(uint32_t bar) {
  asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(bar) : "memory");
}
__device__ __forceinline__ void tc_fence_before() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void tc_fence_after() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }
// generic-proxy shared-memory writes -> visible to the tensor core (async proxy)
__device__ __forceinline__ void fence_async_smem() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }

__device__ __forceinline__ void tmem_alloc(uint32_t dst_smem, uint32_t ncols) {
  asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(dst_smem), "r"(ncols)
               : "memory");
}
__device__ __forceinline__ void tmem_relinquish() {
  asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
}
__device__ __forceinline__ void tmem_dealloc(uint32_t taddr, uint32_t ncols) {
  asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(taddr), "r"(ncols) : "memory");
}
// 16 consecutive fp32 columns of this thread's TMEM lane (32x32b shape)
__device__ __forceinline__ void tmem_ld16(uint32_t taddr, float* v) {
  uint32_t r[16];
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];\n\t"
      "tcgen05.wait::ld.sync.aligned;"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]), "=r"(r[8]),
        "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
      : "r"(taddr)
      : "memory");
#pragma unroll
  for (int i = 0; i < 16; ++i) v[i] = __uint_as_float(r[i]);
}

__device__ __forceinline__ void mbar_init(uint32_t bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(bar), "r"(count) : "memory");
}
__device__ __forceinline__ void mbar_init_fence() { asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory"); }
__device__ __forceinline__ bool mbar_try(uint32_t bar, uint32_t parity) {
  uint32_t ok;
  asm volatile(
      "{\n\t.reg .pred p;\n\tmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\tselp.u32 %0, 1, 0, p;\n\t}"
      : "=r"(ok)
      : "r"(bar), "r"(parity)
      : "memory");
  return ok != 0;
}
// Waits for phase `parity` of the barrier for at most `limit` SM clocks (by
// default about one second); false when the wait ran out.
#define GD_WAIT_CLOCKS 2000000000ll
__device__ __forceinline__ bool mbar_wait(uint32_t bar, uint32_t parity, long long limit = GD_WAIT_CLOCKS) {
  const long long t0 = clock64();
  while (!mbar_try(bar, parity))
    if (clock64() - t0 > limit) return false;
  return true;
}
__device__ __forceinline__ void mbar_expect_tx(uint32_t bar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(bar), "r"(bytes) : "memory");
}
// One-dimensional bulk copy global -> shared (TMA), completing on `bar`.
__device__ __forceinline__ void bulk_g2s(uint32_t dst, const void* src, uint32_t bytes, uint32_t bar) {
  asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(dst),
               "l"(src), "r"(bytes), "r"(bar)
               : "memory");
}
// Loads `bytes` (a multiple of 16) in chunks of at most 16 KB; thread 0 only.
__device__ __forceinline__ void bulk_load(void* dst, const void* src, uint32_t bytes, uint32_t bar) {
  mbar_expect_tx(bar, bytes);
  for (uint32_t off = 0; off < bytes; off += 16384u) {
    const uint32_t n = bytes - off < 16384u ? bytes - off : 16384u;
    bulk_g2s(smem_u32(dst) + off, static_cast<const unsigned char*>(src) + off, n, bar);
  }
}

// D[128 x N] (+)= A[128 x K] * B[N x K]^T, both operands K-major canonical.
__device__ __forceinline__ void mma_gemm(uint32_t d_tmem, uint32_t a, uint32_t b, uint32_t K, uint32_t N, bool acc) {
  const uint32_t id = idesc_bf16(128, N);
  for (uint32_t k0 = 0; k0 < K; k0 += 16) {
    const uint64_t ad = sdesc(a + k0 * 16u, 128u, K * 16u);
    const uint64_t bd = sdesc(b + k0 * 16u, 128u, K * 16u);
    mma_bf16(d_tmem, ad, bd, id, (k0 > 0 || acc) ? 1u : 0u);
  }
}

__device__ __forceinline__ uint32_t pack_bf16(float a, float b) {
  const __nv_bfloat162 h = __floats2bfloat162_rn(a, b);
  return *reinterpret_cast<const uint32_t*>(&h);
}
__device__ __forceinline__ void st_bf16(unsigned char* p, float a) {
  *reinterpret_cast<__nv_bfloat16*>(p) = __float2bfloat16_rn(a);
}

// ---------------------------------------------------------------- encoding --
// sin/cos of 2^k pi u by the double-angle recurrence from sincospi(u).
__device__ __forceinline__ void freq_row(float u, float* v) {
  float s, c;
  sincospif(u, &s, &c);
  v[0] = s;
  v[1] = c;
#pragma unroll
  for (int k = 1; k < GD_FREQ; ++k) {
    const float s2 = (2.0f * s) * c;
    const float c2 = fmaf(-2.0f * s, s, 1.0f);
    s = s2;
    c = c2;
    v[2 * k] = s;
    v[2 * k + 1] = c;
  }
}
// Row `row` of the encoded-input tile (K = 176), 16-byte stores.
__device__ __forceinline__ void encode_row(unsigned char* tile, uint32_t row, const float u[7]) {
#pragma unroll
  for (int j = 0; j < 7; ++j) {
    float v[24];
    freq_row(u[j], v);
#pragma unroll
    for (int ch = 0; ch < 3; ++ch) {
      const uint4 w = make_uint4(pack_bf16(v[8 * ch], v[8 * ch + 1]), pack_bf16(v[8 * ch + 2], v[8 * ch + 3]),
                                 pack_bf16(v[8 * ch + 4], v[8 * ch + 5]), pack_bf16(v[8 * ch + 6], v[8 * ch + 7]));
      *reinterpret_cast<uint4*>(tile + gd_cofs(row, 24 * j + 8 * ch, GD_IN)) = w;
    }
  }
  const uint4 w = make_uint4(pack_bf16(u[0], u[1]), pack_bf16(u[2], u[3]), pack_bf16(u[4], u[5]),
                             pack_bf16(u[6], 1.0f));
  *reinterpret_cast<uint4*>(tile + gd_cofs(row, 168, GD_IN)) = w;
}
// Column `col` of the transposed tile (N = 176 features x K = 128 records).
__device__ __forceinline__ void encode_col(unsigned char* tile, uint32_t col, const float u[7]) {
#pragma unroll
  for (int j = 0; j < 7; ++j) {
    float v[24];
    freq_row(u[j], v);
#pragma unroll
    for (int e = 0; e < 24; ++e) st_bf16(tile + gd_cofs(24 * j + e, col, GD_TILE), v[e]);
  }
#pragma unroll
  for (int j = 0; j < 7; ++j) st_bf16(tile + gd_cofs(168 + j, col, GD_TILE), u[j]);
  st_bf16(tile + gd_cofs(175, col, GD_TILE), 1.0f);
}

// Half of a row of the encoded-input tile (two threads share a row): half 0
// the features of inputs 0-3, half 1 those of inputs 4-6 and the raw inputs
// with the constant 1 (columns 168..175).  Both halves run the same code.
__device__ __forceinline__ float input_j(const float u[7], int j) {
  return j == 0 ? u[0] : j == 1 ? u[1] : j == 2 ? u[2] : j == 3 ? u[3] : j == 4 ? u[4] : j == 5 ? u[5] : u[6];
}
__device__ __forceinline__ void encode_row_half(unsigned char* tile, uint32_t row, const float u[7], uint32_t half) {
  const int j0 = half ? 4 : 0, j1 = half ? 7 : 4;
#pragma unroll 1
  for (int j = j0; j < j1; ++j) {
    float v[24];
    freq_row(input_j(u, j), v);
#pragma unroll
    for (int ch = 0; ch < 3; ++ch) {
      const uint4 w = make_uint4(pack_bf16(v[8 * ch], v[8 * ch + 1]), pack_bf16(v[8 * ch + 2], v[8 * ch + 3]),
                                 pack_bf16(v[8 * ch + 4], v[8 * ch + 5]), pack_bf16(v[8 * ch + 6], v[8 * ch + 7]));
      *reinterpret_cast<uint4*>(tile + gd_cofs(row, 24 * j + 8 * ch, GD_IN)) = w;
    }
  }
  if (half) {
    const uint4 w = make_uint4(pack_bf16(u[0], u[1]), pack_bf16(u[2], u[3]), pack_bf16(u[4], u[5]),
                               pack_bf16(u[6], 1.0f));
    *reinterpret_cast<uint4*>(tile + gd_cofs(row, 168, GD_IN)) = w;
  }
}
// The same half of column `col` of the transposed tile.
__device__ __forceinline__ void encode_col_half(unsigned char* tile, uint32_t col, const float u[7], uint32_t half) {
  const int j0 = half ? 4 : 0, j1 = half ? 7 : 4;
#pragma unroll 1
  for (int j = j0; j < j1; ++j) {
    float v[24];
    freq_row(input_j(u, j), v);
#pragma unroll
    for (int e = 0; e < 24; ++e) st_bf16(tile + gd_cofs(24 * j + e, col, GD_TILE), v[e]);
  }
  if (half) {
#pragma unroll
    for (int j = 0; j < 7; ++j) st_bf16(tile + gd_cofs(168 + j, col, GD_TILE), u[j]);
    st_bf16(tile + gd_cofs(175, col, GD_TILE), 1.0f);
  }
}

// ---------------------------------------------------------------- vMF head --
struct Mix {
  float mu[GD_LOBES][3];
  float kap[GD_LOBES];
  float w[GD_LOBES];    // mixture weights (softmax)
  float nrm[GD_LOBES];  // kappa / (2 pi (1 - exp(-2 kappa)))
  float mlen[GD_LOBES];
  uint32_t kclamp;      // bit k: concentration clamped (no gradient)
};
__device__ __forceinline__ void make_mix(const float* o, Mix& m) {
  float mx = -3.0e38f;
#pragma unroll
  for (int k = 0; k < GD_LOBES; ++k) mx = fmaxf(mx, o[5 * k + 4]);
  float sum = 0.0f;
  m.kclamp = 0u;
#pragma unroll
  for (int k = 0; k < GD_LOBES; ++k) {
    const float x = o[5 * k], y = o[5 * k + 1], z = o[5 * k + 2];
    const float l = sqrtf(x * x + y * y + z * z);
    if (l > 1e-6f) {
      m.mu[k][0] = x / l;
      m.mu[k][1] = y / l;
      m.mu[k][2] = z / l;
      m.mlen[k] = l;
    } else {
      m.mu[k][0] = 0.0f;
      m.mu[k][1] = 0.0f;
      m.mu[k][2] = 1.0f;
      m.mlen[k] = 1e-6f;
    }
    float lk = o[5 * k + 3];
    if (!(lk >= GD_LOGK_MIN && lk <= GD_LOGK_MAX)) {
      m.kclamp |= 1u << k;
      lk = lk < GD_LOGK_MIN ? GD_LOGK_MIN : (lk > GD_LOGK_MAX ? GD_LOGK_MAX : GD_LOGK_MIN);
    }
    const float kap = expf(lk);
    m.kap[k] = kap;
    m.nrm[k] = kap / (6.283185307179586f * -expm1f(-2.0f * kap));
    const float e = expf(o[5 * k + 4] - mx);
    m.w[k] = e;
    sum += e;
  }
  const float inv = 1.0f / sum;
#pragma unroll
  for (int k = 0; k < GD_LOBES; ++k) m.w[k] *= inv;
}
// Mixture density at unit direction (x, y, z); v[k] receives each lobe's density.
__device__ __forceinline__ float mix_pdf(const Mix& m, float x, float y, float z, float* v) {
  float q = 0.0f;
#pragma unroll
  for (int k = 0; k < GD_LOBES; ++k) {
    const float c = m.mu[k][0] * x + m.mu[k][1] * y + m.mu[k][2] * z;
    v[k] = m.nrm[k] * expf(m.kap[k] * (c - 1.0f));
    q += m.w[k] * v[k];
  }
  return q;
}
__device__ __forceinline__ void vmf_sample(float mx, float my, float mz, float kap, float u1, float u2, float& x,
                                           float& y, float& z);
// Lobe by u0, then the vMF sample of Jakob 2012 ("Numerically stable sampling
// of the von Mises-Fisher distribution on S2") in the frame of Duff et al. 2017.
__device__ __forceinline__ void mix_sample(const Mix& m, float u0, float u1, float u2, float& x, float& y, float& z) {
  float acc = 0.0f, mx = m.mu[GD_LOBES - 1][0], my = m.mu[GD_LOBES - 1][1], mz = m.mu[GD_LOBES - 1][2];
  float kap = m.kap[GD_LOBES - 1];
  bool found = false;
#pragma unroll
  for (int k = 0; k < GD_LOBES - 1; ++k) {
    acc += m.w[k];
    if (!found && u0 < acc) {
      found = true;
      mx = m.mu[k][0];
      my = m.mu[k][1];
      mz = m.mu[k][2];
      kap = m.kap[k];
    }
  }
  vmf_sample(mx, my, mz, kap, u1, u2, x, y, z);
}
// Jakob 2012's vMF sample around unit mean (mx, my, mz), concentration kap.
__device__ __forceinline__ void vmf_sample(float mx, float my, float mz, float kap, float u1, float u2, float& x,
                                           float& y, float& z) {
  float W = 1.0f + logf(u1 + (1.0f - u1) * expf(-2.0f * kap)) / kap;
  W = fminf(1.0f, fmaxf(-1.0f, W));
  const float sw = sqrtf(fmaxf(0.0f, 1.0f - W * W));
  float sp, cp;
  sincospif(2.0f * u2, &sp, &cp);
  const float sg = copysignf(1.0f, mz);
  const float a = -1.0f / (sg + mz);
  const float b = mx * my * a;
  const float tx = 1.0f + sg * mx * mx * a, ty = sg * b, tz = -sg * mx;
  const float bx = b, by = sg + my * my * a, bz = -my;
  x = W * mx + sw * (cp * tx + sp * bx);
  y = W * my + sw * (cp * ty + sp * by);
  z = W * mz + sw * (cp * tz + sp * bz);
  const float l = sqrtf(x * x + y * y + z * z);
  x /= l;
  y /= l;
  z /= l;
}
// d(-f log q(w)) / d o for the 40 outputs; returns -f log q.
__device__ __forceinline__ float mix_grad(const Mix& m, float x, float y, float z, float f, float* d) {
  float v[GD_LOBES];
  const float q = fmaxf(mix_pdf(m, x, y, z, v), 1e-30f);
  const float g = -f / q;
#pragma unroll
  for (int k = 0; k < GD_LOBES; ++k) {
    const float kap = m.kap[k];
    const float c = m.mu[k][0] * x + m.mu[k][1] * y + m.mu[k][2] * z;
    const float a = g * m.w[k] * v[k];
    d[5 * k + 4] = a - g * m.w[k] * q;
    const float dk = a * (1.0f / kap - 2.0f / expm1f(2.0f * kap) + c - 1.0f);
    d[5 * k + 3] = (m.kclamp >> k) & 1u ? 0.0f : dk * kap;
    const float s = a * kap / m.mlen[k];
    d[5 * k + 0] = s * (x - m.mu[k][0] * c);
    d[5 * k + 1] = s * (y - m.mu[k][1] * c);
    d[5 * k + 2] = s * (z - m.mu[k][2] * c);
  }
  return f > 0.0f ? -f * logf(q) : 0.0f;
}

}  // namespace gd

namespace gd {

// ------------------------------------------------------------- inference --
#define GI_XCH (GD_B_FWD + GD_TILE * GD_IN * 2 + GD_TILE * GD_H * 2)  // head exchange: 10 x 128 floats
#define GD_SMEM_INFER (GI_XCH + 10 * GD_TILE * 4 + 64)
enum { SRC_QUEUE = 0, SRC_ARRAY = 1 };
struct ArrayIO {
  const float4* in;  // 2 per query: u0..u3 | u4..u6, -
  float* out;        // GD_OUT raw outputs per query
  uint32_t n;
};

__device__ __forceinline__ float sat(float x) { return fminf(1.0f, fmaxf(0.0f, x)); }

// Every thread: publish its shared-tile writes, thread 0 issues the MMAs, all
// wait for their completion (bounded).  Returns false on a timeout (uniform).
template <class Issue>
__device__ __forceinline__ bool run_mma(uint32_t bar, uint32_t& phase, Issue issue) {
  fence_async_smem();
  tc_fence_before();
  __syncthreads();
  if (threadIdx.x == 0) {
    tc_fence_after();
    issue();
    mma_commit(bar);
  }
  const bool ok = __syncthreads_and(mbar_wait(bar, phase)) != 0;
  phase ^= 1u;
  tc_fence_after();
  return ok;
}

// Hidden layer epilogue of this thread's row: TMEM (64 fp32) -> relu -> unit 63
// set to 1 -> bf16 row of the next layer's A tile; optionally the transposed
// copy (column `row` of a 64 x 128 tile).  Returns the mask of units > 0.
__device__ __forceinline__ uint64_t hidden_epilogue(uint32_t trow, unsigned char* a_tile, unsigned char* t_tile,
                                                    uint32_t row) {
  uint64_t mask = 0;
#pragma unroll
  for (int c = 0; c < 4; ++c) {
    float v[16];
    tmem_ld16(trow + 16u * c, v);
#pragma unroll
    for (int i = 0; i < 16; ++i) {
      float h = fmaxf(v[i], 0.0f);
      if (16 * c + i == GD_H - 1) h = 1.0f;
      v[i] = h;
      if (h > 0.0f) mask |= 1ull << (16 * c + i);
    }
#pragma unroll
    for (int hh = 0; hh < 2; ++hh) {
      const float* p = v + 8 * hh;
      *reinterpret_cast<uint4*>(a_tile + gd_cofs(row, 16 * c + 8 * hh, GD_H)) =
          make_uint4(pack_bf16(p[0], p[1]), pack_bf16(p[2], p[3]), pack_bf16(p[4], p[5]), pack_bf16(p[6], p[7]));
    }
    if (t_tile) {
#pragma unroll
      for (int i = 0; i < 16; ++i) st_bf16(t_tile + gd_cofs(16 * c + i, row, GD_TILE), v[i]);
    }
  }
  return mask;
}

// Half of hidden_epilogue: columns [c0, c0 + 32) of this thread's row (c0 =
// 0 or 32), out of line so that the three layers and both halves share one
// copy of the code; t_tile (optional) receives the transposed copy.  The
// returned mask holds bit u - c0 for each unit u > 0.
__device__ __noinline__ uint32_t hidden_epilogue_half(uint32_t trow, unsigned char* a_tile, unsigned char* t_tile,
                                                      uint32_t row, uint32_t c0) {
  uint32_t mask = 0;
#pragma unroll
  for (uint32_t cc = 0; cc < 2; ++cc) {
    const uint32_t c = c0 / 16 + cc;
    float v[16];
    tmem_ld16(trow + 16u * c, v);
#pragma unroll
    for (int i = 0; i < 16; ++i) {
      float h = fmaxf(v[i], 0.0f);
      if (16 * c + i == GD_H - 1) h = 1.0f;
      v[i] = h;
      if (h > 0.0f) mask |= 1u << (16 * cc + i);
    }
#pragma unroll
    for (int hh = 0; hh < 2; ++hh) {
      const float* p = v + 8 * hh;
      *reinterpret_cast<uint4*>(a_tile + gd_cofs(row, 16 * c + 8 * hh, GD_H)) =
          make_uint4(pack_bf16(p[0], p[1]), pack_bf16(p[2], p[3]), pack_bf16(p[4], p[5]), pack_bf16(p[6], p[7]));
    }
    if (t_tile) {
#pragma unroll
      for (int i = 0; i < 16; ++i) st_bf16(t_tile + gd_cofs(16 * c + i, row, GD_TILE), v[i]);
    }
  }
  return mask;
}
// Half of backward_epilogue over the same columns (mask from hidden_epilogue_half).
__device__ __noinline__ void backward_epilogue_half(uint32_t trow, uint32_t mask, unsigned char* a_tile,
                                                    unsigned char* t_tile, uint32_t row, uint32_t c0) {
#pragma unroll
  for (uint32_t cc = 0; cc < 2; ++cc) {
    const uint32_t c = c0 / 16 + cc;
    float v[16];
    tmem_ld16(trow + 16u * c, v);
#pragma unroll
    for (int i = 0; i < 16; ++i) {
      const uint32_t unit = 16 * c + i;
      v[i] = (unit != GD_H - 1 && ((mask >> (16 * cc + i)) & 1u)) ? v[i] : 0.0f;
    }
    if (a_tile) {
#pragma unroll
      for (int hh = 0; hh < 2; ++hh) {
        const float* p = v + 8 * hh;
        *reinterpret_cast<uint4*>(a_tile + gd_cofs(row, 16 * c + 8 * hh, GD_H)) =
            make_uint4(pack_bf16(p[0], p[1]), pack_bf16(p[2], p[3]), pack_bf16(p[4], p[5]), pack_bf16(p[6], p[7]));
      }
    }
#pragma unroll
    for (int i = 0; i < 16; ++i) st_bf16(t_tile + gd_cofs(16 * c + i, row, GD_TILE), v[i]);
  }
}

// The vMF head split over the two threads of a row: each evaluates four
// lobes (K0 = 0 or 4) and the two exchange the softmax maximum, the softmax
// sum and the mixture density through shared memory (xch: 3 x 2 x 128
// floats; every thread of the CTA calls these, so the barriers are uniform).
struct Mix4 {
  float mu[4][3], kap[4], w[4], nrm[4], mlen[4];
  uint32_t kclamp;  // bit j: the concentration of lobe K0 + j was clamped
};
__device__ __forceinline__ float pair_exchange(float* xch, uint32_t row, uint32_t half, float v, bool take_max) {
  xch[half * GD_TILE + row] = v;
  __syncthreads();
  const float a = xch[row], b = xch[GD_TILE + row];
  return take_max ? fmaxf(a, b) : a + b;
}
// o[j] = output 5 K0 + j (j < 20).  Fills m (weights normalised over all 8 lobes).
__device__ __forceinline__ void make_mix4(const float* o, Mix4& m, float* xch, uint32_t row, uint32_t half) {
  float lmax = -3.0e38f;
#pragma unroll
  for (int k = 0; k < 4; ++k) lmax = fmaxf(lmax, o[5 * k + 4]);
  const float mx = pair_exchange(xch, row, half, lmax, true);
  float sum = 0.0f;
  m.kclamp = 0u;
#pragma unroll
  for (int k = 0; k < 4; ++k) {
    const float x = o[5 * k], y = o[5 * k + 1], z = o[5 * k + 2];
    const float l = sqrtf(x * x + y * y + z * z);
    if (l > 1e-6f) {
      m.mu[k][0] = x / l;
      m.mu[k][1] = y / l;
      m.mu[k][2] = z / l;
      m.mlen[k] = l;
    } else {
      m.mu[k][0] = 0.0f;
      m.mu[k][1] = 0.0f;
      m.mu[k][2] = 1.0f;
      m.mlen[k] = 1e-6f;
    }
    float lk = o[5 * k + 3];
    if (!(lk >= GD_LOGK_MIN && lk <= GD_LOGK_MAX)) {
      m.kclamp |= 1u << k;
      lk = lk < GD_LOGK_MIN ? GD_LOGK_MIN : (lk > GD_LOGK_MAX ? GD_LOGK_MAX : GD_LOGK_MIN);
    }
    const float kap = expf(lk);
    m.kap[k] = kap;
    m.nrm[k] = kap / (6.283185307179586f * -expm1f(-2.0f * kap));
    const float e = expf(o[5 * k + 4] - mx);
    m.w[k] = e;
    sum += e;
  }
  const float inv = 1.0f / pair_exchange(xch + 2 * GD_TILE, row, half, sum, false);
#pragma unroll
  for (int k = 0; k < 4; ++k) m.w[k] *= inv;
}
// d[j] = d(-f log q(w)) / d output 5 K0 + j for the four lobes; returns -f log q
// (the caller counts it once per row).
__device__ __forceinline__ float mix_grad4(const Mix4& m, float x, float y, float z, float f, float* d, float* xch,
                                           uint32_t row, uint32_t half) {
  float v[4], c[4];
  float qh = 0.0f;
#pragma unroll
  for (int k = 0; k < 4; ++k) {
    c[k] = m.mu[k][0] * x + m.mu[k][1] * y + m.mu[k][2] * z;
    v[k] = m.nrm[k] * expf(m.kap[k] * (c[k] - 1.0f));
    qh += m.w[k] * v[k];
  }
  const float q = fmaxf(pair_exchange(xch + 4 * GD_TILE, row, half, qh, false), 1e-30f);
  const float g = -f / q;
#pragma unroll
  for (int k = 0; k < 4; ++k) {
    const float kap = m.kap[k];
    const float a = g * m.w[k] * v[k];
    d[5 * k + 4] = a - g * m.w[k] * q;
    const float dk = a * (1.0f / kap - 2.0f / expm1f(2.0f * kap) + c[k] - 1.0f);
    d[5 * k + 3] = (m.kclamp >> k) & 1u ? 0.0f : dk * kap;
    const float s = a * kap / m.mlen[k];
    d[5 * k + 0] = s * (x - m.mu[k][0] * c[k]);
    d[5 * k + 1] = s * (y - m.mu[k][1] * c[k]);
    d[5 * k + 2] = s * (z - m.mu[k][2] * c[k]);
  }
  return f > 0.0f ? -f * logf(q) : 0.0f;
}

// Eight warps: warps w and w + 4 read the same TMEM lanes, so every query of
// a tile has two threads, which split its encoding and its hidden-layer
// epilogues; the first of the two evaluates the vMF head (and draws from it).
template <int SRC>
__global__ void __launch_bounds__(256) guide_infer_kernel(GuideDev G, GdQueue Q, ArrayIO A) {
  extern __shared__ __align__(1024) unsigned char smem[];
  unsigned char* sw = smem;
  unsigned char* sx = smem + GD_B_FWD;
  unsigned char* sh = sx + GD_TILE * GD_IN * 2;
  float* xch = reinterpret_cast<float*>(smem + GI_XCH);
  uint64_t* bars = reinterpret_cast<uint64_t*>(smem + GI_XCH + 10 * GD_TILE * 4);
  uint32_t* tslot = reinterpret_cast<uint32_t*>(bars + 2);
  const uint32_t tid = threadIdx.x, warp = tid >> 5;
  const uint32_t quad = warp & 3u, half = warp >> 2;
  const uint32_t row = quad * 32u + (tid & 31u);
  const uint32_t n = SRC == SRC_QUEUE ? *Q.count : A.n;
  const uint32_t ntiles = (n + GD_TILE - 1) / GD_TILE;
  if (blockIdx.x >= ntiles) return;  // uniform over the CTA
  const uint32_t bw = smem_u32(&bars[0]), bm = smem_u32(&bars[1]);
  if (warp == 0) {
    tmem_alloc(smem_u32(tslot), 64);
    tmem_relinquish();
  }
  if (tid == 0) {
    mbar_init(bw, 1);
    mbar_init(bm, 1);
    mbar_init_fence();
  }
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tmem = *tslot;
  const uint32_t trow = tmem + ((quad * 32u) << 16);
  if (tid == 0) bulk_load(sw, G.wblob, GD_B_FWD, bw);
  bool ok = __syncthreads_and(mbar_wait(bw, 0)) != 0;
  uint32_t phase = 0;
  const uint32_t a_x = smem_u32(sx), a_h = smem_u32(sh), b_w = smem_u32(sw);
  // The inputs of a tile (and, for queued queries, the slot's direction record, key and
  // random-stream position).  Loading them one tile ahead, during the current tile's MMAs,
  // measured no faster (179.6 vs 178.9 us for the first guided bounce of the caustic prism).
  struct In {
    float u[7];
    uint32_t slot, ctr;
    bool valid;
    float4 hv;
    uint2 key;
  };
  auto load = [&](uint32_t tile, In& x) {
    const uint32_t qi = tile * GD_TILE + row;
    x.valid = tile < ntiles && qi < n;
#pragma unroll
    for (int j = 0; j < 7; ++j) x.u[j] = 0.0f;
    x.slot = 0;
    x.ctr = 0;
    x.hv = make_float4(0.0f, 0.0f, 1.0f, 0.0f);
    x.key = make_uint2(0u, 0u);
    if (!x.valid) return;
    if (SRC == SRC_QUEUE) {
      const uint32_t slot = Q.queue[qi];
      x.slot = slot;
      const float4 f0 = Q.full[3 * slot];
      const float4 dl = Q.d_lambda[slot];
      const uint4 mt = Q.meta[slot];
      x.ctr = mt.z;
      x.hv = Q.hit[slot];
      x.key = Q.key[slot];
      float lo[3], inv[3];
      gd_box(G, mt.w, lo, inv);
      x.u[0] = sat((f0.x - lo[0]) * inv[0]);
      x.u[1] = sat((f0.y - lo[1]) * inv[1]);
      x.u[2] = sat((f0.z - lo[2]) * inv[2]);
      x.u[3] = sat(0.5f - 0.5f * dl.x);  // outgoing direction = -ray direction
      x.u[4] = sat(0.5f - 0.5f * dl.y);
      x.u[5] = sat(0.5f - 0.5f * dl.z);
      x.u[6] = ((float)__float_as_int(dl.w) - 380.0f) * 0.0025f;
    } else {
      const float4 a = A.in[2 * qi], b = A.in[2 * qi + 1];
      x.u[0] = a.x; x.u[1] = a.y; x.u[2] = a.z; x.u[3] = a.w;
      x.u[4] = b.x; x.u[5] = b.y; x.u[6] = b.z;
    }
  };
  In cur;
  for (uint32_t tile = blockIdx.x; ok && tile < ntiles; tile += gridDim.x) {
    load(tile, cur);
    const uint32_t qi = tile * GD_TILE + row;
    const bool valid = cur.valid;
    const uint32_t slot = cur.slot;
    float u[7];
#pragma unroll
    for (int j = 0; j < 7; ++j) u[j] = cur.u[j];
    const float4 hv_cur = cur.hv;
    const uint2 key_cur = cur.key;
    const uint32_t ctr_cur = cur.ctr;
    encode_row_half(sx, row, u, half);
    ok = run_mma(bm, phase, [&] { mma_gemm(tmem, a_x, b_w + GD_B_W1, GD_IN, GD_H, false); });
    if (!ok) break;
    hidden_epilogue_half(trow, sh, nullptr, row, 32u * half);
    ok = run_mma(bm, phase, [&] { mma_gemm(tmem, a_h, b_w + GD_B_W2, GD_H, GD_H, false); });
    if (!ok) break;
    hidden_epilogue_half(trow, sh, nullptr, row, 32u * half);
    ok = run_mma(bm, phase, [&] { mma_gemm(tmem, a_h, b_w + GD_B_W3, GD_H, GD_H, false); });
    if (!ok) break;
    hidden_epilogue_half(trow, sh, nullptr, row, 32u * half);
    ok = run_mma(bm, phase, [&] { mma_gemm(tmem, a_h, b_w + GD_B_W4, GD_H, GD_OUTP, false); });
    if (!ok) break;
    if (SRC == SRC_ARRAY) {
      if (half == 0) {
        float o[GD_OUTP];
        tmem_ld16(trow, o);
        tmem_ld16(trow + 16u, o + 16);
        tmem_ld16(trow + 32u, o + 32);
        if (valid) {
#pragma unroll
          for (int i = 0; i < GD_OUT; ++i) A.out[(size_t)GD_OUT * qi + i] = o[i];
        }
      }
      tc_fence_before();  // the next tile's MMAs overwrite these columns after a barrier
    } else {
      // the head: lobes 0-3 (half 0) or 4-7 (half 1); every thread takes part (uniform barriers)
      float o32[32];
      tmem_ld16(trow + 16u * half, o32);
      tmem_ld16(trow + 16u * half + 16u, o32 + 16);
      tc_fence_before();
      float o[20];  // output 20 half + j (selected, not indexed: o32 stays in registers)
#pragma unroll
      for (int j = 0; j < 20; ++j) o[j] = half ? o32[j + 4] : o32[j];
      Mix4 m;
      make_mix4(o, m, xch, row, half);
      const float4 hv = hv_cur;
      const bool guided = valid && hv.w != 0.0f;  // this bounce samples the guide
      clvd::Rng rng;
      float u0 = 0.0f, u1 = 0.0f, u2 = 0.0f;
      if (guided) {
        rng.key = (uint64_t)key_cur.x | ((uint64_t)key_cur.y << 32);
        rng.counter = ctr_cur;
        u0 = rng.f32();
        u1 = rng.f32();
        u2 = rng.f32();
      }
      // lobe choice by u0 over the cumulative weights in lobe order (as mix_sample): the first
      // half's running sum, or -1 if it already chose, goes to the second half
      float acc = 0.0f;
      int pick = -1;
      float* xs = xch + 4 * GD_TILE;  // [row]: first half's sum or -1
      if (half == 0) {
#pragma unroll
        for (int k = 0; k < 4; ++k) {
          acc += m.w[k];
          if (pick < 0 && u0 < acc) pick = k;
        }
        xs[row] = pick >= 0 ? -1.0f : acc;
      }
      __syncthreads();
      if (half == 1) {
        const float a0 = xs[row];
        if (a0 >= 0.0f) {
          acc = a0;
#pragma unroll
          for (int k = 0; k < 3; ++k) {  // lobes 4..6; lobe 7 takes the rest
            acc += m.w[k];
            if (pick < 0 && u0 < acc) pick = k;
          }
          if (pick < 0) pick = 3;
        }
      }
      float* xd = xch + 5 * GD_TILE;  // [3][row]: the sampled direction from the half that owns the lobe
      if (guided && pick >= 0) {
        float mx = 0.0f, my = 0.0f, mz = 1.0f, kp = 1.0f;  // the picked lobe, selected without indexing
#pragma unroll
        for (int k = 0; k < 4; ++k)
          if (k == pick) {
            mx = m.mu[k][0];
            my = m.mu[k][1];
            mz = m.mu[k][2];
            kp = m.kap[k];
          }
        float x, y, z;
        vmf_sample(mx, my, mz, kp, u1, u2, x, y, z);
        xd[row] = x;
        xd[GD_TILE + row] = y;
        xd[2 * GD_TILE + row] = z;
      }
      __syncthreads();
      float x = hv.x, y = hv.y, z = hv.z;
      if (guided) {
        x = xd[row];
        y = xd[GD_TILE + row];
        z = xd[2 * GD_TILE + row];
      }
      float qh = 0.0f;
#pragma unroll
      for (int k = 0; k < 4; ++k)
        qh += m.w[k] * (m.nrm[k] * expf(m.kap[k] * (m.mu[k][0] * x + m.mu[k][1] * y + m.mu[k][2] * z - 1.0f)));
      const float q = pair_exchange(xch + 8 * GD_TILE, row, half, qh, false);
      if (half == 0 && valid) {
        Q.hit[slot] = make_float4(x, y, z, q);
        if (guided) Q.meta[slot].z = rng.counter;
      }
    }
  }
  __syncthreads();
  if (!ok && tid == 0) {
    atomicOr(G.err, CLV_ERR_GUIDE);
    mbar_wait(bw, 0);  // copies or MMAs still in flight, bounded
    mbar_wait(bm, phase ^ 1u);
  }
  __syncthreads();
  if (warp == 0) {
    tc_fence_after();
    tmem_dealloc(tmem, 64);
  }
}

}  // namespace gd

namespace gd {

// ---------------------------------------------------------------- training --
// Shared memory of the training kernel (bytes).
#define GT_W 0                                   // weights, forward and transposed: GD_B_ALL
#define GT_X (GT_W + GD_B_ALL)                   // X (128 x 176) / X^T (176 x 128)
#define GT_A (GT_X + GD_TILE * GD_IN * 2)        // H (forward A, K = 64) / dZ (backward A, K <= 64)
#define GT_ZT (GT_A + GD_TILE * GD_H * 2)        // dZ^T (64 x 128); as an M = 128 operand its rows
                                                 // 64..127 read on into GT_HT (lanes never read back)
#define GT_HT (GT_ZT + GD_H * GD_TILE * 2)       // H1^T, H2^T, H3^T (64 x 128 each)
#define GT_XCH (GT_HT + 3 * GD_H * GD_TILE * 2)  // head exchange of the two threads of a row: 3 x 256 floats
#define GT_BAR (GT_XCH + 3 * 2 * GD_TILE * 4)    // mbarriers, TMEM address
#define GD_SMEM_TRAIN (GT_BAR + 64)
#define GT_HT_BYTES (GD_H * GD_TILE * 2)
// TMEM columns of the training kernel (512 allocated)
#define GT_DF 0u     // forward accumulator
#define GT_DB 64u    // backward accumulator
#define GT_DW1 128u  // dW1: lanes = out (64), columns = in (176)
#define GT_DW2 320u
#define GT_DW3 384u
#define GT_DW4 448u

// dZ = dH * relu'(z) (unit 63 carries no gradient): row of the next backward
// A tile (optional) and column `row` of the transposed tile.
__device__ __forceinline__ void backward_epilogue(uint32_t trow, uint64_t mask, unsigned char* a_tile,
                                                  unsigned char* t_tile, uint32_t row) {
#pragma unroll
  for (int c = 0; c < 4; ++c) {
    float v[16];
    tmem_ld16(trow + 16u * c, v);
#pragma unroll
    for (int i = 0; i < 16; ++i) {
      const int unit = 16 * c + i;
      v[i] = (unit != GD_H - 1 && ((mask >> unit) & 1ull)) ? v[i] : 0.0f;
    }
    if (a_tile) {
#pragma unroll
      for (int hh = 0; hh < 2; ++hh) {
        const float* p = v + 8 * hh;
        *reinterpret_cast<uint4*>(a_tile + gd_cofs(row, 16 * c + 8 * hh, GD_H)) =
            make_uint4(pack_bf16(p[0], p[1]), pack_bf16(p[2], p[3]), pack_bf16(p[4], p[5]), pack_bf16(p[6], p[7]));
      }
    }
#pragma unroll
    for (int i = 0; i < 16; ++i) st_bf16(t_tile + gd_cofs(16 * c + i, row, GD_TILE), v[i]);
  }
}

// Adds the loss gradient of records [0, n) (GD_REC_F4 float4 each) into
// grad (sums, fp32) and the loss sum into *loss.  Eight warps: warps w and
// w + 4 read the same TMEM lanes (rows 32 (w mod 4) ..), so every row of a
// tile has two threads, which split its encoding (inputs 0-3 | 4-6 and the
// raw inputs), its hidden-layer epilogues (units 0-31 | 32-63) and the vMF
// head and its gradient (lobes 0-3 | 4-7).
__global__ void __launch_bounds__(256, 1) guide_train_kernel(const unsigned char* __restrict__ wblob,
                                                             const float4* __restrict__ rec, uint32_t n,
                                                             float* __restrict__ grad, double* __restrict__ loss,
                                                             uint32_t* err) {
  extern __shared__ __align__(1024) unsigned char smem[];
  unsigned char* sw = smem + GT_W;
  unsigned char* sx = smem + GT_X;
  unsigned char* sa = smem + GT_A;
  unsigned char* szt = smem + GT_ZT;
  unsigned char* sht = smem + GT_HT;
  float* xch = reinterpret_cast<float*>(smem + GT_XCH);
  uint64_t* bars = reinterpret_cast<uint64_t*>(smem + GT_BAR);
  uint32_t* tslot = reinterpret_cast<uint32_t*>(bars + 2);
  const uint32_t tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const uint32_t quad = warp & 3u, half = warp >> 2;
  const uint32_t row = quad * 32u + lane;  // tile row (record) of this thread
  const uint32_t ntiles = (n + GD_TILE - 1) / GD_TILE;
  if (blockIdx.x >= ntiles) return;
  const uint32_t bw = smem_u32(&bars[0]), bm = smem_u32(&bars[1]);
  if (warp == 0) {
    tmem_alloc(smem_u32(tslot), 512);
    tmem_relinquish();
  }
  if (tid == 0) {
    mbar_init(bw, 1);
    mbar_init(bm, 1);
    mbar_init_fence();
  }
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tmem = *tslot;
  const uint32_t trow = tmem + ((quad * 32u) << 16);
  if (tid == 0) bulk_load(sw, wblob, GD_B_ALL, bw);
  bool ok = __syncthreads_and(mbar_wait(bw, 0)) != 0;
  uint32_t phase = 0;
  const uint32_t a_x = smem_u32(sx), a_a = smem_u32(sa), a_zt = smem_u32(szt), a_ht = smem_u32(sht);
  const uint32_t b_w = smem_u32(sw);
  bool first = true;
  double lsum = 0.0;
  for (uint32_t tile = blockIdx.x; ok && tile < ntiles; tile += gridDim.x) {
    const uint32_t r = tile * GD_TILE + row;
    float u[7] = {0.0f, 0.0f, 0.0f, 0.0f, 0.0f, 0.0f, 0.0f};
    float wx = 0.0f, wy = 0.0f, wz = 1.0f, f = 0.0f;
    if (r < n) {
      const float4 a = rec[GD_REC_F4 * (size_t)r], b = rec[GD_REC_F4 * (size_t)r + 1];
      u[0] = a.x; u[1] = a.y; u[2] = a.z; u[3] = a.w;
      u[4] = b.x; u[5] = b.y; u[6] = b.z;
      const float4 c = rec[GD_REC_F4 * (size_t)r + 2];
      wx = c.x; wy = c.y; wz = c.z;
      f = (c.w > 0.0f && c.w < 3.0e38f) ? c.w : 0.0f;
    }
    // forward
    encode_row_half(sx, row, u, half);
    ok = run_mma(bm, phase, [&] { mma_gemm(tmem + GT_DF, a_x, b_w + GD_B_W1, GD_IN, GD_H, false); });
    if (!ok) break;
    uint32_t m1, m2, m3;
    m1 = hidden_epilogue_half(trow + GT_DF, sa, sht, row, 32u * half);
    ok = run_mma(bm, phase, [&] { mma_gemm(tmem + GT_DF, a_a, b_w + GD_B_W2, GD_H, GD_H, false); });
    if (!ok) break;
    m2 = hidden_epilogue_half(trow + GT_DF, sa, sht + GT_HT_BYTES, row, 32u * half);
    ok = run_mma(bm, phase, [&] { mma_gemm(tmem + GT_DF, a_a, b_w + GD_B_W3, GD_H, GD_H, false); });
    if (!ok) break;
    m3 = hidden_epilogue_half(trow + GT_DF, sa, sht + 2 * GT_HT_BYTES, row, 32u * half);
    ok = run_mma(bm, phase, [&] { mma_gemm(tmem + GT_DF, a_a, b_w + GD_B_W4, GD_H, GD_OUTP, false); });
    if (!ok) break;
    {  // the head: lobes 0-3 (half 0) or 4-7 (half 1), outputs 20 half .. 20 half + 19
      float o32[32];
      tmem_ld16(trow + GT_DF + 16u * half, o32);
      tmem_ld16(trow + GT_DF + 16u * half + 16u, o32 + 16);
      float o[20];  // output 20 half + j (selected, not indexed: o32 stays in registers)
#pragma unroll
      for (int j = 0; j < 20; ++j) o[j] = half ? o32[j + 4] : o32[j];
      float d[20];
#pragma unroll
      for (int i = 0; i < 20; ++i) d[i] = 0.0f;
      Mix4 m;
      make_mix4(o, m, xch, row, half);
      const float l = mix_grad4(m, wx, wy, wz, f, d, xch, row, half);
      if (f > 0.0f) {
        if (half == 0) lsum += (double)l;
      } else {
#pragma unroll
        for (int i = 0; i < 20; ++i) d[i] = 0.0f;
      }
      // dO row (K = 48, chunks of 8 outputs) and column `row` of dO^T; outputs 40..47 are zero
      if (half == 0) {
#pragma unroll
        for (int c = 0; c < 2; ++c)
          *reinterpret_cast<uint4*>(sa + gd_cofs(row, 8 * c, GD_OUTP)) =
              make_uint4(pack_bf16(d[8 * c], d[8 * c + 1]), pack_bf16(d[8 * c + 2], d[8 * c + 3]),
                         pack_bf16(d[8 * c + 4], d[8 * c + 5]), pack_bf16(d[8 * c + 6], d[8 * c + 7]));
#pragma unroll
        for (int i = 16; i < 20; ++i) st_bf16(sa + gd_cofs(row, i, GD_OUTP), d[i]);
#pragma unroll
        for (int i = 0; i < 20; ++i) st_bf16(szt + gd_cofs(i, row, GD_TILE), d[i]);
      } else {
        float e[28];  // outputs 20..47
#pragma unroll
        for (int i = 0; i < 28; ++i) e[i] = i < 20 ? d[i] : 0.0f;
#pragma unroll
        for (int i = 0; i < 4; ++i) st_bf16(sa + gd_cofs(row, 20 + i, GD_OUTP), e[i]);
#pragma unroll
        for (int c = 0; c < 3; ++c)
          *reinterpret_cast<uint4*>(sa + gd_cofs(row, 24 + 8 * c, GD_OUTP)) =
              make_uint4(pack_bf16(e[4 + 8 * c], e[5 + 8 * c]), pack_bf16(e[6 + 8 * c], e[7 + 8 * c]),
                         pack_bf16(e[8 + 8 * c], e[9 + 8 * c]), pack_bf16(e[10 + 8 * c], e[11 + 8 * c]));
#pragma unroll
        for (int i = 0; i < 28; ++i) st_bf16(szt + gd_cofs(20 + i, row, GD_TILE), e[i]);
      }
    }
    // dH3 = dO W4 ; dW4 += dO^T H3
    ok = run_mma(bm, phase, [&] {
      mma_gemm(tmem + GT_DB, a_a, b_w + GD_B_W4T, GD_OUTP, GD_H, false);
      mma_gemm(tmem + GT_DW4, a_zt, a_ht + 2 * GT_HT_BYTES, GD_TILE, GD_H, !first);
    });
    if (!ok) break;
    backward_epilogue_half(trow + GT_DB, m3, sa, szt, row, 32u * half);
    // dH2 = dZ3 W3 ; dW3 += dZ3^T H2
    ok = run_mma(bm, phase, [&] {
      mma_gemm(tmem + GT_DB, a_a, b_w + GD_B_W3T, GD_H, GD_H, false);
      mma_gemm(tmem + GT_DW3, a_zt, a_ht + GT_HT_BYTES, GD_TILE, GD_H, !first);
    });
    if (!ok) break;
    backward_epilogue_half(trow + GT_DB, m2, sa, szt, row, 32u * half);
    // dH1 = dZ2 W2 ; dW2 += dZ2^T H1
    ok = run_mma(bm, phase, [&] {
      mma_gemm(tmem + GT_DB, a_a, b_w + GD_B_W2T, GD_H, GD_H, false);
      mma_gemm(tmem + GT_DW2, a_zt, a_ht, GD_TILE, GD_H, !first);
    });
    if (!ok) break;
    backward_epilogue_half(trow + GT_DB, m1, nullptr, szt, row, 32u * half);
    // X^T replaces X, whose last reader has completed
    encode_col_half(sx, row, u, half);
    // dW1 += dZ1^T X
    ok = run_mma(bm, phase, [&] { mma_gemm(tmem + GT_DW1, a_zt, a_x, GD_TILE, GD_IN, !first); });
    if (!ok) break;
    first = false;
  }
  // loss sum
#pragma unroll
  for (int off = 16; off > 0; off >>= 1) lsum += __shfl_down_sync(0xFFFFFFFFu, lsum, off);
  if (lane == 0 && lsum != 0.0) atomicAdd(loss, lsum);
  // weight gradients: TMEM lanes 0..63 (quads 0 and 1) hold rows out = row; the two
  // warps of a quad split the columns; vector (float4) reductions into grad
  if (ok && !first && quad < 2) {
    float v[16];
    auto flush = [&](uint32_t tcol, float* dst) {
      tmem_ld16(trow + tcol, v);
#pragma unroll
      for (int i = 0; i < 16; i += 4)
        atomicAdd(reinterpret_cast<float4*>(dst + i), make_float4(v[i], v[i + 1], v[i + 2], v[i + 3]));
    };
    const uint32_t c1a = half == 0 ? 0u : 6u, c1b = half == 0 ? 6u : GD_IN / 16;  // dW1: chunks 0-5 | 6-10
#pragma unroll 1
    for (uint32_t c = c1a; c < c1b; ++c) flush(GT_DW1 + 16u * c, grad + GD_P_W1 + row * GD_IN + 16u * c);
#pragma unroll 1
    for (uint32_t c = 2u * half; c < 2u * half + 2u; ++c) {
      flush(GT_DW2 + 16u * c, grad + GD_P_W2 + row * GD_H + 16u * c);
      flush(GT_DW3 + 16u * c, grad + GD_P_W3 + row * GD_H + 16u * c);
      tmem_ld16(trow + GT_DW4 + 16u * c, v);  // every lane loads (the load is warp-wide); rows < 40 exist
      if (row < GD_OUT) {
#pragma unroll
        for (int i = 0; i < 16; i += 4)
          atomicAdd(reinterpret_cast<float4*>(grad + GD_P_W4 + row * GD_H + 16u * c + i),
                    make_float4(v[i], v[i + 1], v[i + 2], v[i + 3]));
      }
    }
  }
  __syncthreads();
  if (!ok && tid == 0) {
    atomicOr(err, CLV_ERR_GUIDE);
    mbar_wait(bw, 0);
    mbar_wait(bm, phase ^ 1u);
  }
  tc_fence_before();
  __syncthreads();
  if (warp == 0) {
    tc_fence_after();
    tmem_dealloc(tmem, 512);
  }
}

// Gathers the records that carry light (f > 0); the others add nothing to the
// gradient.  Warp-aggregated append, order not preserved.
// Keeps the records with a positive finite weight.  Record k of the input is
// read at (k * GD_SHUFFLE) mod n, a permutation of [0, n) since the prime
// GD_SHUFFLE exceeds n: the records come out of the renderer roughly in pixel
// order, and the training steps take consecutive batches of the output, which
// this spreads over the whole image.
#ifndef GD_SHUFFLE
#define GD_SHUFFLE 2654435761ull  // prime above the largest record capacity (2^26)
#endif
__global__ void guide_compact_kernel(const float4* __restrict__ rec, uint32_t n, float4* __restrict__ out,
                                     unsigned int* __restrict__ count) {
  const uint32_t k = blockIdx.x * blockDim.x + threadIdx.x;
  const uint32_t i = k < n ? (uint32_t)(((uint64_t)k * GD_SHUFFLE) % n) : 0u;
  bool keep = false;
  float4 c = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
  if (k < n) {
    c = rec[GD_REC_F4 * (size_t)i + 2];
    keep = c.w > 0.0f && c.w < 3.0e38f;
  }
  const unsigned m = __ballot_sync(0xFFFFFFFFu, keep);
  if (!m) return;
  const int lane = threadIdx.x & 31, leader = __ffs(m) - 1;
  unsigned base = 0;
  if (lane == leader) base = atomicAdd(count, (unsigned)__popc(m));
  base = __shfl_sync(0xFFFFFFFFu, base, leader);
  if (keep) {
    float4* o = out + GD_REC_F4 * (size_t)(base + __popc(m & ((1u << lane) - 1u)));
    o[0] = rec[GD_REC_F4 * (size_t)i];
    o[1] = rec[GD_REC_F4 * (size_t)i + 1];
    o[2] = c;
  }
}

// bf16 copies of parameter i in the operand blob (forward and transposed)
__device__ __forceinline__ void blob_store(unsigned char* blob, uint32_t i, float w) {
  const __nv_bfloat16 b = __float2bfloat16_rn(w);
  if (i < GD_P_W2) {
    *reinterpret_cast<__nv_bfloat16*>(blob + GD_B_W1 + gd_cofs(i / GD_IN, i % GD_IN, GD_IN)) = b;
    return;
  }
  uint32_t j, fwd, bwd, kt;
  if (i < GD_P_W3) {
    j = i - GD_P_W2; fwd = GD_B_W2; bwd = GD_B_W2T; kt = GD_H;
  } else if (i < GD_P_W4) {
    j = i - GD_P_W3; fwd = GD_B_W3; bwd = GD_B_W3T; kt = GD_H;
  } else {
    j = i - GD_P_W4; fwd = GD_B_W4; bwd = GD_B_W4T; kt = GD_OUTP;
  }
  const uint32_t o = j / GD_H, k = j % GD_H;
  *reinterpret_cast<__nv_bfloat16*>(blob + fwd + gd_cofs(o, k, GD_H)) = b;
  *reinterpret_cast<__nv_bfloat16*>(blob + bwd + gd_cofs(k, o, kt)) = b;
}

// Adam (Kingma & Ba 2015) on the mean gradient (grad * gscale), then the bf16
// blob; with update == 0 only the blob is rewritten.  Clears grad.
__global__ void guide_adam_kernel(float* __restrict__ p, float* __restrict__ m, float* __restrict__ v,
                                  float* __restrict__ g, unsigned char* __restrict__ blob, float lr, float b1, float b2,
                                  float eps, float bc1, float bc2, float gscale, int update) {
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= GD_NPARAM) return;
  float w = p[i];
  if (update) {
    float gg = g[i] * gscale;
    g[i] = 0.0f;
    if (!isfinite(gg)) gg = 0.0f;
    const float mm = b1 * m[i] + (1.0f - b1) * gg;
    const float vv = b2 * v[i] + (1.0f - b2) * gg * gg;
    m[i] = mm;
    v[i] = vv;
    w -= lr * (mm / bc1) / (sqrtf(vv / bc2) + eps);
    p[i] = w;
  }
  blob_store(blob, i, w);
}

// D = A B^T on hashed bf16 operands (128 x K by N x K) through the same
// descriptors, against a CUDA-core sum of the same bf16 products.  One CTA.
__global__ void __launch_bounds__(128, 1) guide_selftest_kernel(uint32_t N, uint32_t K, uint64_t seed, float* out,
                                                                float* maxerr, uint32_t* err) {
  extern __shared__ __align__(1024) unsigned char smem[];
  unsigned char* sA = smem;
  unsigned char* sB = smem + 128 * K * 2;
  uint64_t* bars = reinterpret_cast<uint64_t*>(sB + N * K * 2);
  uint32_t* tslot = reinterpret_cast<uint32_t*>(bars + 1);
  const uint32_t tid = threadIdx.x, warp = tid >> 5;
  auto val = [&](uint32_t which, uint32_t r, uint32_t k) {
    const uint64_t h = clvd::mix64(seed ^ ((uint64_t)which << 40) ^ ((uint64_t)r << 20) ^ k);
    return __bfloat162float(__float2bfloat16_rn((float)((int)(h & 0xFFu) - 128) / 64.0f));
  };
  for (uint32_t k = 0; k < K; ++k) st_bf16(sA + gd_cofs(tid, k, K), val(0, tid, k));
  for (uint32_t r = tid; r < N; r += 128)
    for (uint32_t k = 0; k < K; ++k) st_bf16(sB + gd_cofs(r, k, K), val(1, r, k));
  const uint32_t bm = smem_u32(&bars[0]);
  if (warp == 0) {
    tmem_alloc(smem_u32(tslot), 256);
    tmem_relinquish();
  }
  if (tid == 0) {
    mbar_init(bm, 1);
    mbar_init_fence();
  }
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tmem = *tslot;
  uint32_t phase = 0;
  const bool ok = run_mma(bm, phase, [&] { mma_gemm(tmem, smem_u32(sA), smem_u32(sB), K, N, false); });
  float worst = 0.0f;
  if (ok) {
    const uint32_t trow = tmem + ((warp * 32u) << 16);
    for (uint32_t c = 0; c < N; c += 16) {
      float v[16];
      tmem_ld16(trow + c, v);
      for (int i = 0; i < 16; ++i) {
        float ref = 0.0f;
        for (uint32_t k = 0; k < K; ++k) ref += val(0, tid, k) * val(1, c + i, k);
        worst = fmaxf(worst, fabsf(v[i] - ref));
        out[(size_t)tid * N + c + i] = v[i];
      }
    }
  } else if (tid == 0) {
    atomicOr(err, CLV_ERR_GUIDE);
  }
  for (int off = 16; off > 0; off >>= 1) worst = fmaxf(worst, __shfl_down_sync(0xFFFFFFFFu, worst, off));
  if ((tid & 31) == 0) atomicMax(reinterpret_cast<int*>(maxerr), __float_as_int(worst));
  tc_fence_before();
  __syncthreads();
  if (warp == 0) {
    tc_fence_after();
    tmem_dealloc(tmem, 256);
  }
}

// Self-test of the bounded-wait error path: the kernel initialises an
// mbarrier for one arrival that never comes -- nothing asynchronous is
// issued, no copy and no MMA -- so mbar_wait runs out after `limit` clocks.
// The kernel then does what the production kernels do on a timeout: raise
// CLV_ERR_GUIDE, free its TMEM, return.  done[0] = 1 once the TMEM is freed.
__global__ void __launch_bounds__(128) guide_wait_selftest_kernel(uint32_t* err, long long limit, uint32_t* done) {
  __shared__ __align__(8) uint64_t bar;
  __shared__ uint32_t tslot;
  const uint32_t tid = threadIdx.x, warp = tid >> 5;
  if (warp == 0) {
    tmem_alloc(smem_u32(&tslot), 32);
    tmem_relinquish();
  }
  if (tid == 0) {
    mbar_init(smem_u32(&bar), 1);
    mbar_init_fence();
  }
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tmem = tslot;
  const bool ok = __syncthreads_and(mbar_wait(smem_u32(&bar), 0, limit)) != 0;
  if (!ok && tid == 0) atomicOr(err, CLV_ERR_GUIDE);
  __syncthreads();
  if (warp == 0) {
    tc_fence_after();
    tmem_dealloc(tmem, 32);
  }
  __syncthreads();
  if (tid == 0) done[0] = 1u;
}

}  // namespace gd

// ------------------------------------------------------------------- host --
using namespace gd;

namespace {

void ckg(cudaError_t e, const char* what) {
  if (e != cudaSuccess) throw std::runtime_error(std::string(what) + ": " + cudaGetErrorString(e));
}
uint64_t hmix(uint64_t z) {
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
  return z ^ (z >> 31);
}
int sms() {  // cached: launches inside a stream capture make no device queries
  static int n = 0;
  if (n == 0) {
    int dev = 0, v = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&v, cudaDevAttrMultiProcessorCount, dev);
    n = v > 0 ? v : 1;
  }
  return n;
}
template <class K>
void smem_attr(K kernel, int bytes) {
  ckg(cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes), "cudaFuncSetAttribute");
}

// He-uniform hidden layers; the output layer starts near zero except its bias
// column (hidden unit 63), which spreads the 8 lobe means over the sphere with
// concentration e^1 and equal weights.
std::vector<float> init_params(uint64_t seed) {
  std::vector<float> p(GD_NPARAM, 0.0f);
  uint64_t ctr = 0;
  auto uni = [&]() { return (float)((hmix(seed + 0x9E3779B97F4A7C15ull * ++ctr) >> 40) * (1.0 / 16777216.0)); };
  auto fill = [&](int off, int rows, int cols, float a) {
    for (int i = 0; i < rows * cols; ++i) p[off + i] = (2.0f * uni() - 1.0f) * a;
  };
  fill(GD_P_W1, GD_H, GD_IN, std::sqrt(6.0f / GD_IN));
  fill(GD_P_W2, GD_H, GD_H, std::sqrt(6.0f / GD_H));
  fill(GD_P_W3, GD_H, GD_H, std::sqrt(6.0f / GD_H));
  fill(GD_P_W4, GD_OUT, GD_H, 0.01f);
  const float gold = 2.39996323f;  // golden-angle spiral
  for (int k = 0; k < GD_LOBES; ++k) {
    const float z = 1.0f - (2.0f * k + 1.0f) / GD_LOBES, r = std::sqrt(1.0f - z * z), ph = gold * k;
    const float dir[3] = {r * std::cos(ph), r * std::sin(ph), z};
    for (int c = 0; c < 3; ++c) p[GD_P_W4 + (5 * k + c) * GD_H + (GD_H - 1)] = dir[c];
    p[GD_P_W4 + (5 * k + 3) * GD_H + (GD_H - 1)] = 1.0f;
    p[GD_P_W4 + (5 * k + 4) * GD_H + (GD_H - 1)] = 0.0f;
  }
  return p;
}

void pack(clv_guide* g, cudaStream_t st) {
  guide_adam_kernel<<<(GD_NPARAM + 255) / 256, 256, 0, st>>>(g->params, g->adam_m, g->adam_v, g->grad, g->wblob, 0.0f,
                                                             0.0f, 0.0f, 0.0f, 1.0f, 1.0f, 0.0f, 0);
  clv_internal_count_launches(1);
}

// Gradient sums of records [0, n) into g->grad, loss sum into g->loss.
void launch_train(clv_guide* g, const float4* rec, uint32_t n, cudaStream_t st) {
  if (n == 0) return;
  const uint32_t tiles = (n + GD_TILE - 1) / GD_TILE;
  const uint32_t grid = std::min<uint32_t>(tiles, (uint32_t)sms());
  smem_attr(guide_train_kernel, GD_SMEM_TRAIN);
  guide_train_kernel<<<grid, 256, GD_SMEM_TRAIN, st>>>(g->wblob, rec, n, g->grad, g->loss, g->err);
  clv_internal_count_launches(1);
}

}  // namespace

clv_guide::~clv_guide() {
  for (void* p : {(void*)params, (void*)adam_m, (void*)adam_v, (void*)grad, (void*)wblob, (void*)rec,
                  (void*)rec_count, (void*)rec_keep, (void*)keep_count, (void*)slot, (void*)err, (void*)loss})
    if (p) cudaFree(p);
}

uint4* clv_guide::ensure_slots(uint32_t q) {
  if (q > slots) {
    if (slot) cudaFree(slot);
    slot = nullptr;
    slots = 0;
    ckg(cudaMalloc(&slot, (size_t)q * sizeof(uint4)), "cudaMalloc guide slots");
    slots = q;
  }
  return slot;
}

void gd_prepare() {
  sms();
  smem_attr(guide_infer_kernel<SRC_QUEUE>, GD_SMEM_INFER);
}

void gd_launch_queue(const GuideDev& G, const GdQueue& Q, uint32_t max_queries, cudaStream_t st) {
  const uint32_t tiles = (max_queries + GD_TILE - 1) / GD_TILE;
  const uint32_t grid = std::max<uint32_t>(1, std::min<uint32_t>(tiles, 2u * (uint32_t)sms()));
  guide_infer_kernel<SRC_QUEUE><<<grid, 256, GD_SMEM_INFER, st>>>(G, Q, ArrayIO{nullptr, nullptr, 0u});
}

void gd_reset_records(clv_guide* g, cudaStream_t st) {
  ckg(cudaMemsetAsync(g->rec_count, 0, sizeof(unsigned int), st), "cudaMemsetAsync");
}

GuideDev gd_view(clv_guide* g, const float root_box[6], float alpha) {
  GuideDev G{};
  G.wblob = g->wblob;
  G.rec = g->rec;
  G.rec_count = g->rec_count;
  G.rec_cap = g->rec_cap;
  G.slot = g->slot;
  for (int a = 0; a < 3; ++a) {
    const float lo = root_box[2 * a], ext = root_box[2 * a + 1] - root_box[2 * a];
    G.bmin[a] = lo;
    G.binv[a] = ext > 0.0f ? 1.0f / ext : 0.0f;
  }
  G.boxes = nullptr;
  G.alpha = alpha;
  G.err = g->err;
  return G;
}

extern "C" {

int clv_guide_create(const clv_guide_opts* o, clv_guide** out) {
  if (!out) return clv_internal_fail(CLV_E_INVALID, "null argument");
  *out = nullptr;
  clv_guide_opts d{};
  if (o) d = *o;
  if (d.record_capacity == 0) d.record_capacity = 1u << 21;
  if (d.record_capacity > (1u << 26)) return clv_internal_fail(CLV_E_INVALID, "record capacity above 2^26");
  clv_guide* g = new clv_guide();
  try {
    g->rec_cap = d.record_capacity;
    g->lr = d.learning_rate > 0.0f ? d.learning_rate : 5e-3f;
    const size_t pb = GD_NPARAM * sizeof(float);
    ckg(cudaMalloc(&g->params, pb), "cudaMalloc");
    ckg(cudaMalloc(&g->adam_m, pb), "cudaMalloc");
    ckg(cudaMalloc(&g->adam_v, pb), "cudaMalloc");
    ckg(cudaMalloc(&g->grad, pb), "cudaMalloc");
    ckg(cudaMalloc(&g->wblob, GD_B_ALL), "cudaMalloc");
    ckg(cudaMalloc(&g->rec, (size_t)g->rec_cap * GD_REC_F4 * sizeof(float4)), "cudaMalloc guide records");
    ckg(cudaMalloc(&g->rec_count, sizeof(unsigned int)), "cudaMalloc");
    ckg(cudaMalloc(&g->rec_keep, (size_t)g->rec_cap * GD_REC_F4 * sizeof(float4)), "cudaMalloc guide records");
    ckg(cudaMalloc(&g->keep_count, sizeof(unsigned int)), "cudaMalloc");
    ckg(cudaMalloc(&g->err, sizeof(uint32_t)), "cudaMalloc");
    ckg(cudaMalloc(&g->loss, sizeof(double)), "cudaMalloc");
    const std::vector<float> p = init_params(d.seed);
    ckg(cudaMemcpy(g->params, p.data(), pb, cudaMemcpyHostToDevice), "cudaMemcpy");
    ckg(cudaMemset(g->adam_m, 0, pb), "cudaMemset");
    ckg(cudaMemset(g->adam_v, 0, pb), "cudaMemset");
    ckg(cudaMemset(g->grad, 0, pb), "cudaMemset");
    ckg(cudaMemset(g->wblob, 0, GD_B_ALL), "cudaMemset");  // padding rows stay zero
    ckg(cudaMemset(g->rec_count, 0, sizeof(unsigned int)), "cudaMemset");
    ckg(cudaMemset(g->err, 0, sizeof(uint32_t)), "cudaMemset");
    ckg(cudaMemset(g->loss, 0, sizeof(double)), "cudaMemset");
    pack(g, 0);
    ckg(cudaDeviceSynchronize(), "guide init");
  } catch (std::exception& e) {
    delete g;
    return clv_internal_fail(CLV_E_CUDA, e.what());
  }
  *out = g;
  return CLV_OK;
}

void clv_guide_free(clv_guide* g) { delete g; }

int clv_guide_get_params(const clv_guide* g, float* params) {
  if (!g || !params) return clv_internal_fail(CLV_E_INVALID, "null argument");
  if (cudaMemcpy(params, g->params, GD_NPARAM * sizeof(float), cudaMemcpyDeviceToHost) != cudaSuccess)
    return clv_internal_fail(CLV_E_CUDA, "cudaMemcpy D2H");
  return CLV_OK;
}

int clv_guide_set_params(clv_guide* g, const float* params) {
  if (!g || !params) return clv_internal_fail(CLV_E_INVALID, "null argument");
  try {
    ckg(cudaMemcpy(g->params, params, GD_NPARAM * sizeof(float), cudaMemcpyHostToDevice), "cudaMemcpy H2D");
    pack(g, 0);
    ckg(cudaDeviceSynchronize(), "guide pack");
  } catch (std::exception& e) {
    return clv_internal_fail(CLV_E_CUDA, e.what());
  }
  return CLV_OK;
}

int clv_guide_forward(clv_guide* g, const float* queries, uint64_t n, float* out) {
  if (!g || (n && (!queries || !out))) return clv_internal_fail(CLV_E_INVALID, "null argument");
  if (n == 0) return CLV_OK;
  if (n > (1ull << 26)) return clv_internal_fail(CLV_E_INVALID, "too many queries");
  void* buf = nullptr;
  try {
    const size_t bi = n * 8 * sizeof(float), bo = n * GD_OUT * sizeof(float);
    ckg(cudaMalloc(&buf, bi + bo), "cudaMalloc");
    ckg(cudaMemcpy(buf, queries, bi, cudaMemcpyHostToDevice), "cudaMemcpy H2D");
    ArrayIO A{static_cast<const float4*>(buf), reinterpret_cast<float*>(static_cast<char*>(buf) + bi), (uint32_t)n};
    GuideDev G{};
    G.wblob = g->wblob;
    G.err = g->err;
    const uint32_t tiles = (uint32_t)((n + GD_TILE - 1) / GD_TILE);
    smem_attr(guide_infer_kernel<SRC_ARRAY>, GD_SMEM_INFER);
    guide_infer_kernel<SRC_ARRAY><<<std::min<uint32_t>(tiles, 2u * sms()), 256, GD_SMEM_INFER>>>(G, GdQueue{}, A);
    clv_internal_count_launches(1);
    ckg(cudaGetLastError(), "guide forward launch");
    ckg(cudaMemcpy(out, A.out, bo, cudaMemcpyDeviceToHost), "cudaMemcpy D2H");
    uint32_t e = 0;
    ckg(cudaMemcpy(&e, g->err, sizeof e, cudaMemcpyDeviceToHost), "cudaMemcpy D2H");
    cudaFree(buf);
    buf = nullptr;
    if (e) {
      cudaMemset(g->err, 0, sizeof e);
      return clv_internal_fail(CLV_E_DEVICE, "guide kernel timed out waiting for the tensor cores");
    }
  } catch (std::exception& ex) {
    if (buf) cudaFree(buf);
    return clv_internal_fail(CLV_E_CUDA, ex.what());
  }
  return CLV_OK;
}

int clv_guide_gradient(clv_guide* g, const float* records, uint64_t n, float* grads, double* loss) {
  if (!g || !grads || (n && !records)) return clv_internal_fail(CLV_E_INVALID, "null argument");
  if (n > (1ull << 26)) return clv_internal_fail(CLV_E_INVALID, "too many records");
  void* buf = nullptr;
  try {
    const size_t bytes = n * GD_REC_F4 * sizeof(float4);
    ckg(cudaMemset(g->grad, 0, GD_NPARAM * sizeof(float)), "cudaMemset");
    ckg(cudaMemset(g->loss, 0, sizeof(double)), "cudaMemset");
    if (n) {
      ckg(cudaMalloc(&buf, bytes), "cudaMalloc");
      ckg(cudaMemcpy(buf, records, bytes, cudaMemcpyHostToDevice), "cudaMemcpy H2D");
      launch_train(g, static_cast<const float4*>(buf), (uint32_t)n, 0);
      ckg(cudaGetLastError(), "guide train launch");
    }
    ckg(cudaMemcpy(grads, g->grad, GD_NPARAM * sizeof(float), cudaMemcpyDeviceToHost), "cudaMemcpy D2H");
    double l = 0.0;
    ckg(cudaMemcpy(&l, g->loss, sizeof l, cudaMemcpyDeviceToHost), "cudaMemcpy D2H");
    if (loss) *loss = l;
    ckg(cudaMemset(g->grad, 0, GD_NPARAM * sizeof(float)), "cudaMemset");
    if (buf) cudaFree(buf);
    buf = nullptr;
    uint32_t e = 0;
    ckg(cudaMemcpy(&e, g->err, sizeof e, cudaMemcpyDeviceToHost), "cudaMemcpy D2H");
    if (e) {
      cudaMemset(g->err, 0, sizeof e);
      return clv_internal_fail(CLV_E_DEVICE, "guide kernel timed out waiting for the tensor cores");
    }
  } catch (std::exception& ex) {
    if (buf) cudaFree(buf);
    return clv_internal_fail(CLV_E_CUDA, ex.what());
  }
  return CLV_OK;
}

int clv_guide_record_count(const clv_guide* g, uint64_t* n) {
  if (!g || !n) return clv_internal_fail(CLV_E_INVALID, "null argument");
  unsigned int c = 0;
  if (cudaMemcpy(&c, g->rec_count, sizeof c, cudaMemcpyDeviceToHost) != cudaSuccess)
    return clv_internal_fail(CLV_E_CUDA, "cudaMemcpy D2H");
  *n = std::min<uint64_t>(c, g->rec_cap);
  return CLV_OK;
}

int clv_guide_get_records(const clv_guide* g, float* out, uint64_t n) {
  if (!g || (n && !out)) return clv_internal_fail(CLV_E_INVALID, "null argument");
  if (n > g->rec_cap) return clv_internal_fail(CLV_E_INVALID, "more records than the capacity");
  if (n && cudaMemcpy(out, g->rec, n * GD_REC_F4 * sizeof(float4), cudaMemcpyDeviceToHost) != cudaSuccess)
    return clv_internal_fail(CLV_E_CUDA, "cudaMemcpy D2H");
  return CLV_OK;
}

int clv_guide_train(clv_guide* g, uint32_t steps, uint32_t batch, double* mean_loss, void* stream) {
  if (!g) return clv_internal_fail(CLV_E_INVALID, "null argument");
  cudaStream_t st = (cudaStream_t)stream;
  try {
    unsigned int c = 0;
    ckg(cudaMemcpyAsync(&c, g->rec_count, sizeof c, cudaMemcpyDeviceToHost, st), "cudaMemcpyAsync");
    ckg(cudaStreamSynchronize(st), "cudaStreamSynchronize");
    const uint32_t nrec = std::min<uint32_t>(c, g->rec_cap);
    if (nrec == 0 || steps == 0) {
      if (mean_loss) *mean_loss = 0.0;
      return CLV_OK;
    }
    ckg(cudaMemsetAsync(g->keep_count, 0, sizeof(unsigned int), st), "cudaMemsetAsync");
    guide_compact_kernel<<<(nrec + 255) / 256, 256, 0, st>>>(g->rec, nrec, g->rec_keep, g->keep_count);
    clv_internal_count_launches(1);
    ckg(cudaMemcpyAsync(&c, g->keep_count, sizeof c, cudaMemcpyDeviceToHost, st), "cudaMemcpyAsync");
    ckg(cudaStreamSynchronize(st), "cudaStreamSynchronize");
    const uint32_t n = std::min<uint32_t>(c, nrec);
    if (batch == 0) batch = 1u << 16;
    if (n == 0 || steps == 0) {
      if (mean_loss) *mean_loss = 0.0;
      return CLV_OK;
    }
    batch = std::min(batch, n);
    ckg(cudaMemsetAsync(g->loss, 0, sizeof(double), st), "cudaMemsetAsync");
    const float b1 = 0.9f, b2 = 0.99f;
    uint32_t off = 0;
    for (uint32_t s = 0; s < steps; ++s) {
      if (off + batch > n) off = 0;
      launch_train(g, g->rec_keep + (size_t)off * GD_REC_F4, batch, st);
      off += batch;
      ++g->step;
      const float bc1 = 1.0f - std::pow(b1, (float)g->step), bc2 = 1.0f - std::pow(b2, (float)g->step);
      guide_adam_kernel<<<(GD_NPARAM + 255) / 256, 256, 0, st>>>(g->params, g->adam_m, g->adam_v, g->grad,
                                                                 g->wblob, g->lr, b1, b2, 1e-8f, bc1, bc2,
                                                                 1.0f / (float)batch, 1);
      clv_internal_count_launches(1);
    }
    ckg(cudaGetLastError(), "guide train launch");
    if (mean_loss) {
      double l = 0.0;
      ckg(cudaMemcpyAsync(&l, g->loss, sizeof l, cudaMemcpyDeviceToHost, st), "cudaMemcpyAsync");
      ckg(cudaStreamSynchronize(st), "cudaStreamSynchronize");
      *mean_loss = l / ((double)steps * batch);
    }
  } catch (std::exception& ex) {
    return clv_internal_fail(CLV_E_CUDA, ex.what());
  }
  return CLV_OK;
}

int clv_guide_status(clv_guide* g, uint32_t* flags) {
  if (!g || !flags) return clv_internal_fail(CLV_E_INVALID, "null argument");
  uint32_t e = 0;
  if (cudaMemcpy(&e, g->err, sizeof e, cudaMemcpyDeviceToHost) != cudaSuccess)
    return clv_internal_fail(CLV_E_CUDA, "cudaMemcpy D2H");
  cudaMemset(g->err, 0, sizeof e);
  *flags = e;
  return CLV_OK;
}

int clv_guide_selftest_mma(uint32_t n, uint32_t k, uint64_t seed, float* d_out, float* max_abs_err) {
  if (!max_abs_err) return clv_internal_fail(CLV_E_INVALID, "null argument");
  if (n < 16 || n > 256 || n % 16 || k < 16 || k > 256 || k % 16)
    return clv_internal_fail(CLV_E_INVALID, "N and K must be multiples of 16 in [16, 256]");
  void* buf = nullptr;
  try {
    const size_t bo = (size_t)128 * n * sizeof(float);
    ckg(cudaMalloc(&buf, bo + 16), "cudaMalloc");
    float* dout = static_cast<float*>(buf);
    float* derr = reinterpret_cast<float*>(static_cast<char*>(buf) + bo);
    uint32_t* dflag = reinterpret_cast<uint32_t*>(derr + 1);
    ckg(cudaMemset(buf, 0, bo + 16), "cudaMemset");
    const int smem = (int)((128 + n) * k * 2 + 64);
    smem_attr(guide_selftest_kernel, smem);
    guide_selftest_kernel<<<1, 128, smem>>>(n, k, seed, dout, derr, dflag);
    clv_internal_count_launches(1);
    ckg(cudaGetLastError(), "selftest launch");
    float e = 0.0f;
    uint32_t fl = 0;
    ckg(cudaMemcpy(&e, derr, sizeof e, cudaMemcpyDeviceToHost), "cudaMemcpy D2H");
    ckg(cudaMemcpy(&fl, dflag, sizeof fl, cudaMemcpyDeviceToHost), "cudaMemcpy D2H");
    if (d_out) ckg(cudaMemcpy(d_out, dout, bo, cudaMemcpyDeviceToHost), "cudaMemcpy D2H");
    cudaFree(buf);
    buf = nullptr;
    if (fl) return clv_internal_fail(CLV_E_DEVICE, "tensor-core wait timed out");
    *max_abs_err = e;
  } catch (std::exception& ex) {
    if (buf) cudaFree(buf);
    return clv_internal_fail(CLV_E_CUDA, ex.what());
  }
  return CLV_OK;
}

// Runs guide_wait_selftest_kernel with a wait limit of `clocks` SM clocks
// (about 1 ms at 2e6).  flags receives the error bits the kernel raised
// (CLV_ERR_GUIDE expected) and freed = 1 when it reached its TMEM release.
int clv_guide_selftest_timeout(uint64_t clocks, uint32_t* flags, uint32_t* freed) {
  if (!flags || !freed) return clv_internal_fail(CLV_E_INVALID, "null argument");
  if (clocks == 0 || clocks > 4000000000ull) return clv_internal_fail(CLV_E_INVALID, "clocks must lie in (0, 4e9]");
  void* buf = nullptr;
  try {
    ckg(cudaMalloc(&buf, 8), "cudaMalloc");
    uint32_t* d = static_cast<uint32_t*>(buf);
    ckg(cudaMemset(buf, 0, 8), "cudaMemset");
    guide_wait_selftest_kernel<<<1, 128>>>(d, (long long)clocks, d + 1);
    clv_internal_count_launches(1);
    ckg(cudaGetLastError(), "selftest launch");
    uint32_t h[2] = {0u, 0u};
    ckg(cudaMemcpy(h, buf, sizeof h, cudaMemcpyDeviceToHost), "cudaMemcpy D2H");
    cudaFree(buf);
    buf = nullptr;
    *flags = h[0];
    *freed = h[1];
  } catch (std::exception& ex) {
    if (buf) cudaFree(buf);
    return clv_internal_fail(CLV_E_CUDA, ex.what());
  }
  return CLV_OK;
}

}  // extern "C"
