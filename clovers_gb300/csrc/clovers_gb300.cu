// Kernels and the C ABI (include/clovers_gpu.h) of the GB300 render path.
//
//  raycast_persist_kernel  closest-hit ray casts (the parity path), persistent
//                  threads over rays sorted by origin
//  debug_kernel    the debug render modes, one ray per pixel
//  resolve_kernel  f64 film -> mean XYZ(E) -> sRGB u8 (write.rs:39-44)
// Path tracing is the wavefront of wavefront.cuh.

#include <cuda_runtime.h>

#include <algorithm>
#include <atomic>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <memory>
#include <mutex>
#include <stdexcept>
#include <string>
#include <vector>

#include "clovers_gpu.h"
#include "clv_device.cuh"
#include "scene.hpp"
#include "wavefront.cuh"
#include "spectral.hpp"

using namespace clvd;

// ------------------------------------------------------------------ kernels --

// ---- ray order -----------------------------------------------------------
// Ray casts traverse their rays in the order of a Morton code of the origin
// (6 bits per axis of the scene box): warps then start from nearby points and
// share the nodes near the origins in L1/L2.  A counting sort (histogram,
// exclusive scan, scatter) gives the permutation; results go back to each
// ray's own index, so the order changes nothing but speed.
#define CLV_SORT_AXIS_BITS 6
#define CLV_SORT_BINS (1u << (3 * CLV_SORT_AXIS_BITS))
__device__ __forceinline__ uint32_t spread3(uint32_t x) {  // bit k of x -> bit 3k
  x = (x | (x << 16)) & 0x030000FFu;
  x = (x | (x << 8)) & 0x0300F00Fu;
  x = (x | (x << 4)) & 0x030C30C3u;
  x = (x | (x << 2)) & 0x09249249u;
  return x;
}
__device__ __forceinline__ uint32_t cell_of(float v, float lo, float scale) {
  const float c = (v - lo) * scale;
  return c > 0.0f ? (uint32_t)fminf(c, (float)((1u << CLV_SORT_AXIS_BITS) - 1)) : 0u;
}
__global__ void ray_key_hist(const float4* __restrict__ rays, uint64_t n, float3 lo, float3 scale,
                             uint32_t* __restrict__ key, uint32_t* __restrict__ hist) {
  const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
  for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride) {
    const float4 o = __ldg(rays + 2 * i);
    const uint32_t k = spread3(cell_of(o.x, lo.x, scale.x)) | (spread3(cell_of(o.y, lo.y, scale.y)) << 1) |
                       (spread3(cell_of(o.z, lo.z, scale.z)) << 2);
    key[i] = k;
    atomicAdd(hist + k, 1u);
  }
}
// Exclusive scan of CLV_SORT_BINS counts in place; one block of 1024 threads.
__global__ void __launch_bounds__(1024) ray_bins_scan(uint32_t* __restrict__ hist) {
  constexpr uint32_t per = CLV_SORT_BINS / 1024;
  __shared__ uint32_t warp_sum[32];
  const uint32_t t = threadIdx.x, lane = t & 31, w = t >> 5;
  uint32_t* h = hist + t * per;
  uint32_t sum = 0;
  for (uint32_t k = 0; k < per; ++k) sum += h[k];
  uint32_t incl = sum;  // inclusive scan over the block: warps, then warp totals
#pragma unroll
  for (int off = 1; off < 32; off <<= 1) {
    const uint32_t v = __shfl_up_sync(0xFFFFFFFFu, incl, off);
    if (lane >= (uint32_t)off) incl += v;
  }
  if (lane == 31) warp_sum[w] = incl;
  __syncthreads();
  if (w == 0) {
    uint32_t v = warp_sum[lane], x = v;
#pragma unroll
    for (int off = 1; off < 32; off <<= 1) {
      const uint32_t y = __shfl_up_sync(0xFFFFFFFFu, x, off);
      if (lane >= (uint32_t)off) x += y;
    }
    warp_sum[lane] = x - v;  // exclusive prefix of the warp totals
  }
  __syncthreads();
  uint32_t run = warp_sum[w] + incl - sum;
  for (uint32_t k = 0; k < per; ++k) {
    const uint32_t c = h[k];
    h[k] = run;
    run += c;
  }
}
__global__ void ray_scatter(const uint32_t* __restrict__ key, uint64_t n, uint32_t* __restrict__ offs,
                            uint32_t* __restrict__ perm) {
  const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
  for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride)
    perm[atomicAdd(offs + key[i], 1u)] = (uint32_t)i;
}

// Closest-hit ray casts (the parity path), persistent: each lane takes the
// next ray as soon as its traversal ends (one atomic per warp and step in
// which lanes are idle), so lanes do not sit out the longest ray of their
// warp (persistent threads with dynamic fetch, Aila & Laine 2009).  Every ray
// runs closest_hit's exact traversal.  COUNT: per-ray visit counts wanted.
#ifndef CLV_SHADE_BLOCKS
#define CLV_SHADE_BLOCKS 8  // shading-kernel blocks per SM when no tuned shape is set (one wave at 8 resident)
#endif
// Largest traversal-stack spill region (trees deeper than CLV_STACK levels):
// deep scenes run fewer threads or path slots rather than exceed it.
static constexpr uint64_t kSpillBudget = 4ull << 30;
#ifndef CLV_SHSTACK
// ray casts: the first 12 stack entries of each thread in shared memory (24 KB
// per block, the most that keeps 9 blocks per SM; measured best of 0..24)
#define CLV_SHSTACK 12
#endif
#ifndef CLV_LEAF_BATCH
#define CLV_LEAF_BATCH 8  // ray casts: a lane at a leaf waits until this many lanes are at one (0: never; 4..16 measured)
#endif
#ifndef CLV_MINB_RAY
#define CLV_MINB_RAY 9  // 56 registers, no spills: 36 warps per SM (measured best of 6..16)
#endif
// DEEP: trees deeper than CLV_STACK levels; stack entries beyond CLV_STACK go
// to `spill` (SpillStack, one column per thread of the grid, `cap` entries).
template <int CPLX, bool COUNT, int WT, bool DEEP = false>
__global__ void __launch_bounds__(128, CLV_MINB_RAY) raycast_persist_kernel(
    ClvDeviceScene S, const float4* __restrict__ rays, uint64_t n, uint32_t* __restrict__ prim,
    float* __restrict__ tout, uint32_t* __restrict__ nodes, uint32_t* __restrict__ tests, uint32_t* err,
    unsigned long long* next, const uint32_t* __restrict__ perm, float4* spill, int cap) {
  const int lane = threadIdx.x & 31;
  Trav T;
#if CLV_SHSTACK
  __shared__ float4 sh_stack[DEEP ? 1 : CLV_SHSTACK * 128];
#endif
  float4 loc_stack[DEEP ? CLV_STACK : CLV_STACK - CLV_SHSTACK];
  auto stack = [&] {
    if constexpr (DEEP) {
      return SpillStack{loc_stack, spill + (size_t)blockIdx.x * blockDim.x + threadIdx.x, gridDim.x * blockDim.x, cap};
    } else {
#if CLV_SHSTACK
      return HybridStack<CLV_SHSTACK>{sh_stack + threadIdx.x, loc_stack};
#else
      return (float4*)loc_stack;
#endif
    }
  }();
  Hit h;
  Counters c{0u, 0u};
  Ray r{};
  Rng rng;
  uint64_t i = 0;
  bool have = false;
  while (true) {
    const unsigned act = __activemask();
    const unsigned idle = __ballot_sync(act, !have);
    if (idle) {
      const int leader = __ffs(idle) - 1;
      unsigned long long base = 0;
      if (lane == leader) base = atomicAdd(next, (unsigned long long)__popc(idle));
      base = __shfl_sync(act, base, leader);
      if (!have) {
        const uint64_t k = base + __popc(idle & ((1u << lane) - 1u));
        if (k >= n) break;  // no rays left
        i = perm ? (uint64_t)__ldg(perm + k) : k;
        const float4 a = __ldcs(rays + 2 * i), b = __ldcs(rays + 2 * i + 1);
        r = Ray{mk(a.x, a.y, a.z), mk(b.x, b.y, b.z), 0.0f, 600};
        c = Counters{0u, 0u};
        rng.init(0, (uint32_t)i, 0);
        trav_begin<WT>(S, r, a.w, b.w, T, h);
        have = true;
      }
    }
    bool step = have;
    if (CLV_LEAF_BATCH > 0) {
      // Leaf tests in groups: a lane whose next step is a leaf waits while
      // fewer than CLV_LEAF_BATCH lanes are at one and some lane is at a node.
      // Each ray's own sequence of steps is unchanged.
      const bool at_leaf = have && CLV_REF_KIND(T.ref) != CLV_REF_NODE;
      const unsigned lm = __ballot_sync(act, at_leaf), hm = __ballot_sync(act, have);
      if (at_leaf && __popc(lm) < CLV_LEAF_BATCH && lm != hm) step = false;
    }
    if (step && !trav_step<CPLX, WT>(S, r, T, stack, &rng, h, nullptr, COUNT ? &c : nullptr, err)) {
      __stcs(prim + i, T.found ? hit_gid(S, h.ref) : 0xFFFFFFFFu);
      __stcs(tout + i, T.found ? h.t : 0.0f);
      if (COUNT) {
        if (nodes) nodes[i] = c.nodes;
        if (tests) tests[i] = c.prims;
      }
      have = false;
    }
  }
}

struct RenderParams {
  uint32_t width, height;
  uint32_t sample_offset;
  uint32_t mode;
  uint64_t seed;
  uint64_t npix;
};

// Debug render modes (draw_cpu.rs:148-207): one centred ray per pixel.
// spill (trees deeper than CLV_STACK levels, else null): stack entries beyond
// CLV_STACK, one column per pixel.
__global__ void debug_kernel(ClvDeviceScene S, RenderParams P, double* __restrict__ film, uint32_t* err,
                             float4* spill) {
  const uint64_t pix = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (pix >= P.npix) return;
  const uint32_t x = (uint32_t)(pix % P.width), row = (uint32_t)(pix / P.width);
  const uint32_t y = P.height - 1 - row;
  Rng rng;
  rng.init(P.seed, (uint32_t)pix, P.sample_offset);
  const int lambda = random_wavelength(rng);
  const float time = rng.f32();  // the ray's time: moving spheres are where they are at it
  const ClvCamera& C = S.camera;
  const float pu = (float)x / (float)P.width, pv = (float)y / (float)P.height;
  const V dir = sub(add(add(ld3(C.llc), scl(pu, ld3(C.horizontal))), scl(pv, ld3(C.vertical))), ld3(C.origin));
  Ray r{ld3(C.origin), unit(dir), time, lambda};
  float rgb[3] = {0.0f, 0.0f, 0.0f};  // linear sRGB
  Hit h;
  Rec full;
  Counters c{0u, 0u};
  float4 loc[CLV_STACK];
  SpillStack stack{loc, spill ? spill + pix : nullptr, (uint32_t)P.npix, spill ? (int)S.max_depth_tree : CLV_STACK};
  const bool any = closest_hit_stk<2, CLV_WT_SCENE>(S, r, CLV_EPS_ACNE, CLV_FLT_MAX, &rng, h, &full, &c, err, stack);
  if (P.mode == CLV_MODE_NORMAL_MAP) {  // normals.rs:11-37
    if (any) {
      Rec rec;
      hit_record(S, r, h, full, rec);
      const V n = mk(-rec.n.x, rec.n.y, -rec.n.z);
      rgb[0] = 0.5f + 0.5f * n.x;
      rgb[1] = 0.5f + 0.5f * n.y;
      rgb[2] = n.z < 0.0f ? 0.0f : n.z;
    }
  } else {  // debug_visualizations.rs:18-35 colour ramp
    const uint32_t d = P.mode == CLV_MODE_BVH_TEST_COUNT ? c.nodes : c.prims;
    if (d <= 255) { rgb[0] = rgb[1] = rgb[2] = (float)d / 255.0f; }
    else if (d <= 511) { rgb[0] = 1.0f; rgb[1] = 1.0f; }
    else if (d <= 1023) { rgb[0] = 1.0f; rgb[1] = 0.5f; }
    else { rgb[0] = 1.0f; }
  }
  // store linear sRGB in the film; the host converts to XYZ(E) with the same matrices
  double* f = film + 3 * pix;
  f[0] += rgb[0];
  f[1] += rgb[1];
  f[2] += rgb[2];
}

struct ResolveParams {
  double m[9];  // XYZ(E) -> linear sRGB (D65)
  double inv_spp;
  uint32_t width, height;
};
__global__ void resolve_kernel(ResolveParams R, const double* __restrict__ film, float* __restrict__ xyz,
                               uint8_t* __restrict__ rgb) {
  const uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= (uint64_t)R.width * R.height) return;
  float c[3];
#pragma unroll
  for (int k = 0; k < 3; ++k) c[k] = (float)(film[3 * i + k] * R.inv_spp);
  if (xyz) {
#pragma unroll
    for (int k = 0; k < 3; ++k) xyz[3 * i + k] = c[k];
  }
  if (rgb) {
#pragma unroll
    for (int r = 0; r < 3; ++r) {
      const float lin = (float)(R.m[r * 3] * (double)c[0] + R.m[r * 3 + 1] * (double)c[1] + R.m[r * 3 + 2] * (double)c[2]);
      const float e = lin <= 0.0031308f ? lin * 12.92f : 1.055f * powf(lin, 1.0f / 2.4f) - 0.055f;
      float v = roundf(e * 255.0f);
      if (!(v > 0.0f)) v = 0.0f;
      if (v > 255.0f) v = 255.0f;
      rgb[3 * i + r] = (uint8_t)v;
    }
  }
}

// Self-test of div_rn against IEEE division on random operands: a spans
// magnitudes 2^-40..2^40 with random signs, d spans 2^-70..2^70 including
// values outside div_rn's fast range, zeros and infinities.
__device__ __forceinline__ float selftest_coord(uint64_t h) {
  // 0, or a random float of magnitude 2^-70 .. 2^59
  if ((h & 63) == 0) return 0.0f;
  const uint32_t e = 127 - 70 + (uint32_t)((h >> 8) % 130);
  return __uint_as_float((uint32_t)(h >> 32) & 0x807FFFFFu | (e << 23));
}
// Self-test of the traversal's divisions against IEEE division.
// mode 0: div_rn on arbitrary operands (zeros, infinities, subnormals);
// mode 1: div_fast on the operands the traversal admits: a = b - o with b, o
//         0 or of magnitude 2^-70..2^59, |d| in 2^-60..2.
__global__ void selftest_division_kernel(uint64_t n, uint64_t seed, int mode, unsigned long long* bad) {
  const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
  unsigned long long local = 0;
  for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride) {
    const uint64_t h1 = mix64(seed ^ (i * 0x9E3779B97F4A7C15ull)), h2 = mix64(h1 + 0x632BE59BD9B4E019ull);
    const uint64_t h3 = mix64(h2 + 0x1234567ull);
    float a, d;
    if (mode == 0) {
      a = __uint_as_float((uint32_t)(h1 & 0x807FFFFFu) | ((uint32_t)(87 + (h1 >> 32) % 81) << 23));
      d = __uint_as_float((uint32_t)(h2 & 0x807FFFFFu) | ((uint32_t)(57 + (h2 >> 32) % 141) << 23));
      const uint32_t sel = (uint32_t)(h2 >> 56);
      if (sel == 0) d = 0.0f;
      if (sel == 1) d = -0.0f;
      if (sel == 2) a = 0.0f;
      if (sel == 3) d = __uint_as_float(0x7F800000u);
      if (sel == 4) d = __uint_as_float((uint32_t)(h2 & 0x807FFFFFu));  // subnormal
    } else {
      const float b = selftest_coord(h1), o = ((h3 >> 60) == 0) ? b : selftest_coord(h3);
      a = b - o;
      const uint32_t e = 127 - 60 + (uint32_t)((h2 >> 8) % 62);  // 2^-60 .. 2^1
      d = __uint_as_float(((uint32_t)(h2 >> 32) & 0x807FFFFFu) | (e << 23));
    }
    const float inv = 1.0f / d;
    float q;
    if (mode == 0) {
      const float ad = fabsf(d);
      const bool fast = ad >= 8.67361738e-19f && ad <= 1.15292150e18f;
      q = fast ? div_rn(a, d, inv) : a / d;
    } else {
      q = div_fast(a, d, inv);
    }
    const float e = a / d;
    // zero signs are irrelevant to the traversal (values only meet comparisons)
    if (__float_as_uint(q) != __float_as_uint(e) && !(q != q && e != e) && !(q == 0.0f && e == 0.0f)) ++local;
  }
  if (local) atomicAdd(bad, local);
}

// Self-test of the render path's logarithm (clv_log.h) over every f32 in
// (0, 1] (bit patterns 1 .. 0x3F800000): the largest error in f32 ulps against
// the GPU's double-precision log, and how many results are not the nearest
// f32 of that value.  The media's free-flight draws take logs of draws in
// [0, 1).
__global__ void selftest_log_kernel(unsigned long long* max_err_bits, unsigned long long* not_nearest) {
  const uint32_t top = 0x3F800000u;
  const uint32_t stride = gridDim.x * blockDim.x;
  double worst = 0.0;
  unsigned long long nn = 0;
  for (uint32_t b = 1u + blockIdx.x * blockDim.x + threadIdx.x; b <= top; b += stride) {
    const float x = __uint_as_float(b);
    const float y = clv_math::log_f32(x);
    const double r = log((double)x);
    if (r != 0.0) {
      int e;
      frexp(fabs(r), &e);
      const double err = fabs((double)y - r) / ldexp(1.0, e - 24);  // f32 ulp at |r|: 2^(e-24)
      worst = fmax(worst, err);
      if (y != (float)r) ++nn;
    } else if (y != 0.0f) {
      worst = 1e30;
    }
  }
#pragma unroll
  for (int off = 16; off > 0; off >>= 1) {
    worst = fmax(worst, __shfl_down_sync(0xFFFFFFFFu, worst, off));
    nn += __shfl_down_sync(0xFFFFFFFFu, nn, off);
  }
  if ((threadIdx.x & 31) == 0) {
    atomicMax(max_err_bits, (unsigned long long)__double_as_longlong(worst));  // non-negative: bits order as values
    if (nn) atomicAdd(not_nearest, nn);
  }
}
__global__ void log_eval_kernel(const float* __restrict__ x, float* __restrict__ y, uint64_t n) {
  const uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) y[i] = clv_math::log_f32(x[i]);
}

// --------------------------------------------------------------- host side --

namespace {

thread_local std::string g_error;
std::atomic<unsigned long long> g_launches{0};

int fail(int code, const std::string& msg) {
  g_error = msg;
  return code;
}

struct CudaError : std::runtime_error {
  using std::runtime_error::runtime_error;
};
void ck(cudaError_t e, const char* what) {
  if (e != cudaSuccess) throw CudaError(std::string(what) + ": " + cudaGetErrorString(e));
}

// Blocks of device memory, pinned words and streams that destroyed device
// scenes release are kept for the next scene on the same device: a host that
// uploads its scene for every frame would otherwise pay cudaMalloc / cudaFree
// of the path state (about 190 MB) every frame, and cudaFree synchronises the
// device.  A released block is reused for a request of at least half its size;
// at most kPoolBlocks blocks are kept, larger surpluses are freed.
namespace pool {
struct Block {
  int dev;
  void* p;
  size_t bytes;
};
static std::mutex mu;
static std::vector<Block> blocks;
static std::vector<std::pair<int, cudaStream_t>> streams;
static std::vector<unsigned int*> pinned;
static constexpr size_t kPoolBlocks = 8;
static int device() {
  int d = 0;
  cudaGetDevice(&d);
  return d;
}
// Device memory of at least `bytes`; *got receives the size of the block.
static void* alloc(size_t bytes, size_t* got, const char* what) {
  const int dev = device();
  {
    std::lock_guard<std::mutex> lock(mu);
    size_t best = blocks.size();
    for (size_t k = 0; k < blocks.size(); ++k)
      if (blocks[k].dev == dev && blocks[k].bytes >= bytes && blocks[k].bytes / 2 <= bytes &&
          (best == blocks.size() || blocks[k].bytes < blocks[best].bytes))
        best = k;
    if (best < blocks.size()) {
      const Block b = blocks[best];
      blocks.erase(blocks.begin() + (std::ptrdiff_t)best);
      *got = b.bytes;
      return b.p;
    }
  }
  void* p = nullptr;
  ck(cudaMalloc(&p, bytes), what);
  *got = bytes;
  return p;
}
// Hands a block back (the device is synchronised first: the releasing scene's
// kernels may still be running on a stream the library does not know).
static void release(void* p, size_t bytes) {
  if (!p) return;
  cudaDeviceSynchronize();
  cudaGetLastError();
  std::lock_guard<std::mutex> lock(mu);
  blocks.push_back(Block{device(), p, bytes});
  if (blocks.size() > kPoolBlocks) {  // free the oldest
    cudaFree(blocks.front().p);
    blocks.erase(blocks.begin());
  }
}
static cudaStream_t stream() {
  const int dev = device();
  {
    std::lock_guard<std::mutex> lock(mu);
    for (size_t k = 0; k < streams.size(); ++k)
      if (streams[k].first == dev) {
        const cudaStream_t st = streams[k].second;
        streams.erase(streams.begin() + (std::ptrdiff_t)k);
        return st;
      }
  }
  cudaStream_t st = nullptr;
  if (cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking) != cudaSuccess) {
    cudaGetLastError();
    return nullptr;
  }
  return st;
}
static void release_stream(cudaStream_t st) {
  if (!st) return;
  std::lock_guard<std::mutex> lock(mu);
  if (streams.size() < kPoolBlocks) streams.emplace_back(device(), st);
  else cudaStreamDestroy(st);
}
static unsigned int* pinned_word() {
  {
    std::lock_guard<std::mutex> lock(mu);
    if (!pinned.empty()) {
      unsigned int* w = pinned.back();
      pinned.pop_back();
      return w;
    }
  }
  unsigned int* w = nullptr;
  ck(cudaMallocHost(&w, sizeof(unsigned int)), "cudaMallocHost");
  return w;
}
static void release_pinned(unsigned int* w) {
  if (!w) return;
  std::lock_guard<std::mutex> lock(mu);
  pinned.push_back(w);
}
}  // namespace pool

// A scene's device arrays in one allocation: `add` records each array at a
// 256-byte aligned offset, `commit` allocates once and copies every array
// straight from its host vector, with one synchronisation at the end.
struct UploadPack {
  struct Item {
    const void* src;
    size_t bytes, offset;
    const void** dst;
  };
  std::vector<Item> items;
  size_t total = 0;
  template <class T>
  void add(const std::vector<T>& v, const T** dst) {
    *dst = nullptr;
    if (v.empty()) return;
    items.push_back(Item{v.data(), v.size() * sizeof(T), total, reinterpret_cast<const void**>(dst)});
    total += (v.size() * sizeof(T) + 255) / 256 * 256;
  }
  size_t reserve(size_t bytes) {  // device-only space (no host data)
    const size_t off = total;
    total += (bytes + 255) / 256 * 256;
    return off;
  }
  char* commit(std::vector<void*>& owned, size_t* owned_bytes) {
    void* base = pool::alloc(std::max<size_t>(total, 256), owned_bytes, "cudaMalloc scene");
    owned.push_back(base);
    char* b = static_cast<char*>(base);
    for (const Item& it : items) {
      ck(cudaMemcpyAsync(b + it.offset, it.src, it.bytes, cudaMemcpyHostToDevice, 0), "cudaMemcpyAsync H2D");
      *it.dst = b + it.offset;
    }
    ck(cudaStreamSynchronize(0), "cudaStreamSynchronize");
    return b;
  }
};

int sm_count() {
  static int n = 0;
  if (n == 0) {
    int dev = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev);
    if (n <= 0) n = 1;
  }
  return n;
}

// Grid of a shading kernel with `minb` resident blocks per SM (wf_shade_diffuse,
// wf_guide_post): the shading grid (tuned or default blocks per SM) scaled by
// minb over the other shading kernels' resident blocks.
uint32_t scaled_grid(uint32_t grid, uint32_t tuned_shade, uint32_t minb) {
  const uint64_t per_sm = (uint64_t)(tuned_shade ? tuned_shade : CLV_SHADE_BLOCKS) * minb / CLV_MINB_SHADE;
  return (uint32_t)std::min<uint64_t>(grid, (uint64_t)sm_count() * std::max<uint64_t>(1, per_sm));
}

// wf_shade_diffuse in the variant `blocks` (resident blocks per SM; 0 = the default).
template <bool BATCH>
void launch_shade_diffuse(uint32_t blocks, uint32_t grid, uint32_t tuned_shade, cudaStream_t s,
                          const ClvDeviceScene& S, const WfParams& P, const WfState& W, WfCounters* C, uint32_t* err,
                          const WfBatch& B) {
  if (blocks == CLV_MINB_DIFFUSE_ALT)
    wf_shade_diffuse<BATCH, CLV_MINB_DIFFUSE_ALT>
        <<<scaled_grid(grid, tuned_shade, CLV_MINB_DIFFUSE_ALT), 128, 0, s>>>(S, P, W, C, err, B);
  else
    wf_shade_diffuse<BATCH, CLV_MINB_DIFFUSE>
        <<<scaled_grid(grid, tuned_shade, CLV_MINB_DIFFUSE), 128, 0, s>>>(S, P, W, C, err, B);
}

}  // namespace

int clv_internal_fail(int code, const char* msg) { return fail(code, msg); }
void clv_internal_count_launches(unsigned long long n) { g_launches += n; }

struct clv_scene {
  clv::HostScene host;
  uint32_t watertight = 0;  // CLV_OPT_WATERTIGHT
};

// Whether every coordinate of every BVH box is 0 or of magnitude in
// [2^-70, 2^59] (the precondition of the traversal's unguarded division).
static bool boxes_div_safe(const clv::HostScene& h) {
  auto ok = [](float x) {
    const float a = std::fabs(x);
    return x == 0.0f || (a >= 8.47032947e-22f && a <= 5.76460752e17f);
  };
  for (int k = 0; k < 6; ++k)
    if (!ok(h.root_box[k])) return false;
  for (const ClvNode& n : h.nodes)
    for (int k = 0; k < 6; ++k)
      if (!ok(n.lbox[k]) || !ok(n.rbox[k])) return false;
  return true;
}

// Which traversal variant the scene needs: 0 primitives only, 1 wrapper
// chains handled inline (chain_hit), 2 media or lists (interpreter).  Only the
// objects the BVH's leaves reach count: a list or mesh given at the top level
// is flattened into the tree, and its own record is never visited.
static uint32_t compound_level(const clv::HostScene& h) {
  if (h.objs.empty()) return 0;
  std::vector<char> seen(h.objs.size(), 0);
  std::vector<uint32_t> todo;
  auto reach = [&](uint32_t r) {
    if (r == CLV_REF_EMPTY || CLV_REF_KIND(r) != CLV_REF_OBJ) return;
    const uint32_t i = CLV_REF_INDEX(r);
    if (i < h.objs.size() && !seen[i]) {
      seen[i] = 1;
      todo.push_back(i);
    }
  };
  reach(h.root);
  for (const ClvNode& n : h.nodes) {
    reach(n.left);
    reach(n.right);
  }
  uint32_t level = 0;
  while (!todo.empty()) {
    const uint32_t i = todo.back();
    todo.pop_back();
    const ClvObj& o = h.objs[i];
    level = std::max(level, 1u);
    if (o.kind == CLV_OBJ_MEDIUM || o.kind == CLV_OBJ_LIST) return 2;
    if (o.kind == CLV_OBJ_TRANSLATE || o.kind == CLV_OBJ_ROTATEY) {
      int depth = 0;
      uint32_t r = CLV_MAKE_REF(CLV_REF_OBJ, i);
      while (CLV_REF_KIND(r) == CLV_REF_OBJ) {
        const ClvObj& w = h.objs[CLV_REF_INDEX(r)];
        if (w.kind != CLV_OBJ_TRANSLATE && w.kind != CLV_OBJ_ROTATEY) break;
        ++depth;
        r = w.a;
      }
      if (depth > CLV_CHAIN) return 2;
      reach(o.a);
    }
  }
  return level;
}


struct clv_device_scene {
  ClvDeviceScene view{};
  std::vector<void*> owned;
  uint32_t* err = nullptr;  // device error word
  uint32_t width = 0, height = 0;
  bool has_camera = false;
  // scratch reused by the host-buffer entry points
  void* scratch = nullptr;
  size_t scratch_bytes = 0;
  // wavefront path state, sized on first use
  void* wf_mem = nullptr;
  size_t wf_bytes = 0;
  uint32_t wf_slots = 0;
  WfCounters* wf_counters = nullptr;
  unsigned int* wf_live_host = nullptr;  // pinned
  cudaStream_t cap_stream = nullptr;     // private stream for graph capture
  // wavefront shape chosen by clv_autotune (0: the built-in defaults)
  uint32_t tuned_slots = 0;      // paths in flight
  uint32_t tuned_shade = 0;      // shading-kernel blocks per SM
  uint32_t tuned_append = 0;     // intersect queue appends per warp (1) or per block (0), primitive-level scenes
  uint32_t tuned_diffuse = 0;    // wf_shade_diffuse variant: resident blocks per SM (0: CLV_MINB_DIFFUSE)
  unsigned long long* ray_next = nullptr;  // work counter of the persistent ray casts
  uint32_t* ray_sort = nullptr;            // ray order: histogram, keys, permutation
  uint64_t ray_sort_cap = 0;               // rays the sort scratch holds
  size_t ray_sort_bytes = 0;
  size_t owned_bytes = 0;                  // the scene arrays' block (owned[0])
  float4* spill = nullptr;   // traversal stack spill of trees deeper than CLV_STACK levels
  size_t spill_bytes = 0;
  float4* spill_region(size_t bytes) {
    if (bytes > spill_bytes) {
      pool::release(spill, spill_bytes);
      spill = nullptr;
      spill_bytes = 0;
      spill = static_cast<float4*>(pool::alloc(bytes, &spill_bytes, "cudaMalloc stack spill"));
    }
    return spill;
  }
  bool deep() const { return view.max_depth_tree > CLV_STACK; }
  // spilled entries per thread of a deep tree (the stack holds tree depth - 1 at most)
  uint32_t spill_entries() const { return deep() ? view.max_depth_tree - CLV_STACK : 0u; }
  uint32_t* ray_sort_scratch(uint64_t n) {
    if (n > ray_sort_cap) {
      pool::release(ray_sort, ray_sort_bytes);
      ray_sort = nullptr;
      ray_sort_cap = 0;
      ray_sort = static_cast<uint32_t*>(
          pool::alloc((CLV_SORT_BINS + 2 * n) * sizeof(uint32_t), &ray_sort_bytes, "cudaMalloc ray order"));
      ray_sort_cap = n;
    }
    return ray_sort;
  }
  cudaStream_t capture_stream() {
    if (!cap_stream) cap_stream = pool::stream();
    return cap_stream;
  }
  // A second stream and a fork / join event pair: wf_shade_specular runs beside
  // the diffuse and guided kernels of the same bounce (their queues hold
  // disjoint slots), so that each fills the other's tail.  False if any of
  // them cannot be created (the bounce then runs in one stream).
  cudaStream_t side_stream = nullptr;
  cudaEvent_t ev_fork = nullptr, ev_join = nullptr;
  bool fork_streams() {
    if (!side_stream) side_stream = pool::stream();
    if (!ev_fork && cudaEventCreateWithFlags(&ev_fork, cudaEventDisableTiming) != cudaSuccess) {
      cudaGetLastError();
      ev_fork = nullptr;
    }
    if (!ev_join && cudaEventCreateWithFlags(&ev_join, cudaEventDisableTiming) != cudaSuccess) {
      cudaGetLastError();
      ev_join = nullptr;
    }
    return side_stream && ev_fork && ev_join;
  }
  size_t counters_bytes = 0;
  ~clv_device_scene() {
    pool::release_stream(cap_stream);
    pool::release_stream(side_stream);
    if (ev_fork) cudaEventDestroy(ev_fork);
    if (ev_join) cudaEventDestroy(ev_join);
    pool::release(ray_sort, ray_sort_bytes);
    pool::release(spill, spill_bytes);
    if (!owned.empty()) pool::release(owned[0], owned_bytes);  // scene arrays, error word and ray counter
    pool::release(scratch, scratch_bytes);
    pool::release(wf_mem, wf_bytes);
    pool::release(wf_counters, counters_bytes);
    pool::release_pinned(wf_live_host);
  }
  WfState wavefront_state(uint32_t q) {
    if (q > wf_slots) {
      pool::release(wf_mem, wf_bytes);
      wf_mem = nullptr;
      wf_slots = 0;
      wf_mem = pool::alloc((size_t)q * kWfSlotBytes, &wf_bytes, "cudaMalloc path state");
      wf_slots = q;
    }
    if (!wf_counters)
      wf_counters = static_cast<WfCounters*>(pool::alloc(sizeof(WfCounters), &counters_bytes, "cudaMalloc"));
    if (!wf_live_host) wf_live_host = pool::pinned_word();
    char* p = static_cast<char*>(wf_mem);
    const size_t n = wf_slots;
    WfState W;
    W.o_time = reinterpret_cast<float4*>(p); p += n * 16;
    W.d_lambda = reinterpret_cast<float4*>(p); p += n * 16;
    W.beta = reinterpret_cast<float4*>(p); p += n * 16;
    W.meta = reinterpret_cast<uint4*>(p); p += n * 16;
    W.hit = reinterpret_cast<float4*>(p); p += n * 16;
    W.full = reinterpret_cast<float4*>(p); p += n * 48;
    W.key = reinterpret_cast<uint2*>(p); p += n * 8;
    W.queue = reinterpret_cast<uint32_t*>(p);
    W.Q = q;
    W.gslot = nullptr;
    W.grec = nullptr;
    W.grec_count = nullptr;
    W.grec_cap = 0;
    W.spill = nullptr;
    W.stack_cap = CLV_STACK;
    return W;
  }
  static constexpr size_t kWfSlotBytes = 16 * 5 + 48 + 8 + 16;
  void* ensure_scratch(size_t bytes) {
    if (bytes > scratch_bytes) {
      pool::release(scratch, scratch_bytes);
      scratch = nullptr;
      scratch_bytes = 0;
      scratch = pool::alloc(bytes, &scratch_bytes, "cudaMalloc scratch");
    }
    return scratch;
  }
};

// An instantiated CUDA graph, destroyed with its owner.
struct GraphExec {
  cudaGraphExec_t exec = nullptr;
  GraphExec() = default;
  GraphExec(const GraphExec&) = delete;
  GraphExec(GraphExec&& o) noexcept : exec(o.exec) { o.exec = nullptr; }
  GraphExec& operator=(GraphExec&& o) noexcept {
    std::swap(exec, o.exec);
    return *this;
  }
  ~GraphExec() {
    if (exec) cudaGraphExecDestroy(exec);
  }
};

// Captures what `enqueue` launches on the scene's private capture stream into
// an executable graph.  Returns an empty one if capture is not possible (the
// caller then launches directly).
template <class F>
static GraphExec capture_graph(clv_device_scene* d, F enqueue) {
  GraphExec g;
  cudaStream_t cs = d->capture_stream();
  if (!cs) return g;
  if (cudaStreamBeginCapture(cs, cudaStreamCaptureModeThreadLocal) != cudaSuccess) {
    cudaGetLastError();
    return g;
  }
  enqueue(cs);
  cudaGraph_t graph = nullptr;
  if (cudaStreamEndCapture(cs, &graph) != cudaSuccess || !graph) {
    cudaGetLastError();
    return g;
  }
  cudaGraphExec_t ex = nullptr;
  const cudaError_t e = cudaGraphInstantiate(&ex, graph, 0);
  cudaGraphDestroy(graph);
  if (e != cudaSuccess) {
    cudaGetLastError();
    return g;
  }
  g.exec = ex;
  return g;
}

static uint32_t launch_grid(uint64_t work, int block) {
  const uint64_t want = (work + block - 1) / block;
  const uint64_t cap = (uint64_t)sm_count() * 16;  // persistent-style grid-stride cap
  return (uint32_t)std::max<uint64_t>(1, std::min(want, cap));
}

static int check_opts(const clv_device_scene* d, const clv_render_opts* o) {
  if (!d || !o) return fail(CLV_E_INVALID, "null argument");
  if (!d->has_camera) return fail(CLV_E_INVALID, "this scene has no camera (mesh scenes are for ray casts)");
  if (o->width != d->width || o->height != d->height)
    return fail(CLV_E_INVALID, "render size differs from the size the scene was loaded with (camera aspect)");
  if (o->samples == 0) return fail(CLV_E_INVALID, "samples must be positive");
  if (o->sampler != 0) return fail(CLV_E_INVALID, "only the random sampler is supported (blue-noise tables are absent)");
  if (o->mode > CLV_MODE_PRIMITIVE_TEST_COUNT) return fail(CLV_E_INVALID, "unknown render mode");
  if ((uint64_t)o->width * o->height > 0x1FFFFFFFull) return fail(CLV_E_INVALID, "image too large");
  return CLV_OK;
}

static RenderParams make_params(const clv_render_opts* o) {
  RenderParams P{};
  P.width = o->width;
  P.height = o->height;
  P.sample_offset = o->sample_offset;
  P.mode = o->mode;
  P.seed = o->seed;
  P.npix = (uint64_t)o->width * o->height;
  return P;
}

extern "C" {

const char* clv_last_error(void) { return g_error.c_str(); }
const char* clv_version(void) { return "clovers_gb300 0.1 (sm_103a)"; }

uint64_t clv_kernel_launches(void) { return g_launches.load(); }

int clv_device_alloc(uint64_t bytes, void** out) {
  if (!out) return fail(CLV_E_INVALID, "null argument");
  const cudaError_t e = cudaMalloc(out, bytes ? bytes : 1);
  if (e != cudaSuccess) return fail(CLV_E_CUDA, std::string("cudaMalloc: ") + cudaGetErrorString(e));
  return CLV_OK;
}
void clv_device_free(void* p) {
  if (p) cudaFree(p);
}
int clv_memcpy(void* dst, const void* src, uint64_t bytes) {
  const cudaError_t e = cudaMemcpy(dst, src, bytes, cudaMemcpyDefault);
  if (e != cudaSuccess) return fail(CLV_E_CUDA, std::string("cudaMemcpy: ") + cudaGetErrorString(e));
  return CLV_OK;
}
int clv_memset(void* dst, int value, uint64_t bytes) {
  const cudaError_t e = cudaMemset(dst, value, bytes);
  if (e != cudaSuccess) return fail(CLV_E_CUDA, std::string("cudaMemset: ") + cudaGetErrorString(e));
  return CLV_OK;
}

static int render_wavefront(clv_device_scene* d, const clv_render_opts* o, double* film, cudaStream_t st,
                            clv_render_profile* prof, clv_guide* guide = nullptr, float alpha = 0.0f,
                            bool count = true);

int clv_render_profile_run(clv_device_scene* d, const clv_render_opts* o, double* film_dev, void* stream,
                           clv_render_profile* out) {
  int rc = check_opts(d, o);
  if (rc) return rc;
  if (!film_dev || !out) return fail(CLV_E_INVALID, "null argument");
  if (o->mode != CLV_MODE_PATH_TRACING)
    return fail(CLV_E_INVALID, "profiling covers the wavefront path tracer only");
  // device times of the production kernels ...
  rc = render_wavefront(d, o, film_dev, (cudaStream_t)stream, out, nullptr, 0.0f, false);
  if (rc) return rc;
  // ... and the traversal counts from the same render with the counting kernels, into a scratch film
  double* scratch = nullptr;
  try {
    ck(cudaMalloc(&scratch, (size_t)o->width * o->height * 3 * sizeof(double)), "cudaMalloc");
    ck(cudaMemsetAsync(scratch, 0, (size_t)o->width * o->height * 3 * sizeof(double), (cudaStream_t)stream),
       "cudaMemsetAsync");
  } catch (std::exception& e) {
    if (scratch) cudaFree(scratch);
    return fail(CLV_E_CUDA, e.what());
  }
  clv_render_profile counted{};
  rc = render_wavefront(d, o, scratch, (cudaStream_t)stream, &counted, nullptr, 0.0f, true);
  cudaStreamSynchronize((cudaStream_t)stream);
  cudaFree(scratch);
  if (rc) return rc;
  out->path_segments = counted.path_segments;
  out->node_visits = counted.node_visits;
  out->prim_tests = counted.prim_tests;
  return CLV_OK;
}

// Times the wavefront render `o` (a short one: a few samples per pixel) for
// every candidate shape -- paths in flight SMs x {1, 2, 4, 8, 16} x 1024,
// shading grids of {8, 16, 32} blocks per SM and intersect queue appends per
// block or per warp, the minimum of two runs each --
// and keeps the fastest in the scene for later renders that leave path_slots
// at 0 (clv_render, clv_render_device, clv_render_guided, clv_render_batch
// with this scene first).
int clv_autotune(clv_device_scene* d, const clv_render_opts* o, clv_tune_result* results, uint32_t max_results,
                 uint32_t* n_results, void* stream) {
  int rc = check_opts(d, o);
  if (rc) return rc;
  if (o->mode != CLV_MODE_PATH_TRACING)
    return fail(CLV_E_INVALID, "tuning covers the wavefront path tracer only");
  cudaStream_t st = (cudaStream_t)stream;
  double* film = nullptr;
  cudaEvent_t e0 = nullptr, e1 = nullptr;
  const uint32_t old_slots = d->tuned_slots, old_shade = d->tuned_shade, old_append = d->tuned_append,
                 old_diffuse = d->tuned_diffuse;
  auto cleanup = [&]() {
    if (film) cudaFree(film);
    if (e0) cudaEventDestroy(e0);
    if (e1) cudaEventDestroy(e1);
  };
  try {
    const size_t fb = (size_t)o->width * o->height * 3 * sizeof(double);
    ck(cudaMalloc(&film, fb), "cudaMalloc tuning film");
    ck(cudaEventCreate(&e0), "cudaEventCreate");
    ck(cudaEventCreate(&e1), "cudaEventCreate");
    const uint32_t sms = (uint32_t)sm_count();
    const uint32_t slot_mult[5] = {1, 2, 4, 8, 16};
    const uint32_t shade[3] = {8, 16, 32};
    clv_render_opts t = *o;
    t.path_slots = 0;
    float best = 3.0e38f;
    uint32_t best_slots = 0, best_shade = 0, best_append = 0, n = 0;
    auto time_shape = [&]() {  // best of two renders of the current shape
      float ms = 3.0e38f;
      for (int rep = 0; rep < 2; ++rep) {
        ck(cudaMemsetAsync(film, 0, fb, st), "cudaMemsetAsync");
        ck(cudaEventRecord(e0, st), "cudaEventRecord");
        rc = render_wavefront(d, &t, film, st, nullptr);
        if (rc) throw std::runtime_error(g_error);
        ck(cudaEventRecord(e1, st), "cudaEventRecord");
        ck(cudaEventSynchronize(e1), "cudaEventSynchronize");
        float m = 0.0f;
        ck(cudaEventElapsedTime(&m, e0, e1), "cudaEventElapsedTime");
        ms = std::min(ms, m);
      }
      const uint32_t db = d->tuned_diffuse ? d->tuned_diffuse : CLV_MINB_DIFFUSE;
      if (results && n < max_results)
        results[n] = clv_tune_result{d->tuned_slots, d->tuned_shade, d->tuned_append, db, ms};
      ++n;
      return ms;
    };
    d->tuned_diffuse = 0;
    for (uint32_t a = 0; a < 5; ++a)
      for (uint32_t b = 0; b < 3; ++b)
        for (uint32_t ap = 0; ap < (d->view.compound_level == 0 && !d->deep() ? 2u : 1u); ++ap) {
          d->tuned_slots = sms * slot_mult[a] * 1024u;
          d->tuned_shade = shade[b];
          d->tuned_append = ap;
          const float ms = time_shape();
          if (ms < best) {
            best = ms;
            best_slots = d->tuned_slots;
            best_shade = d->tuned_shade;
            best_append = ap;
          }
        }
    d->tuned_slots = best_slots;
    d->tuned_shade = best_shade;
    d->tuned_append = best_append;
    // the other wf_shade_diffuse variant at the chosen shape
    d->tuned_diffuse = CLV_MINB_DIFFUSE_ALT;
    if (!(time_shape() < best)) d->tuned_diffuse = 0;
    if (n_results) *n_results = n;
    cleanup();
    return CLV_OK;
  } catch (std::exception& ex) {
    d->tuned_slots = old_slots;
    d->tuned_shade = old_shade;
    d->tuned_append = old_append;
    d->tuned_diffuse = old_diffuse;
    cleanup();
    return fail(CLV_E_CUDA, ex.what());
  }
}

int clv_device_scene_set_shape(clv_device_scene* d, uint32_t path_slots, uint32_t shade_blocks_per_sm,
                               uint32_t warp_appends, uint32_t diffuse_blocks_per_sm) {
  if (!d) return fail(CLV_E_INVALID, "null argument");
  if (warp_appends > 1) return fail(CLV_E_INVALID, "warp_appends takes 0 or 1");
  if (warp_appends && (d->view.compound_level != 0 || d->deep()))
    return fail(CLV_E_INVALID, "per-warp appends exist for primitive-level scenes of at most 64 BVH levels");
  if (shade_blocks_per_sm > 64) return fail(CLV_E_INVALID, "shade_blocks_per_sm above 64");
  if (diffuse_blocks_per_sm && diffuse_blocks_per_sm != CLV_MINB_DIFFUSE && diffuse_blocks_per_sm != CLV_MINB_DIFFUSE_ALT)
    return fail(CLV_E_INVALID, "diffuse_blocks_per_sm takes 0, " + std::to_string(CLV_MINB_DIFFUSE) + " or " +
                                   std::to_string(CLV_MINB_DIFFUSE_ALT));
  d->tuned_slots = path_slots;
  d->tuned_shade = shade_blocks_per_sm;
  d->tuned_append = warp_appends;
  d->tuned_diffuse = diffuse_blocks_per_sm == CLV_MINB_DIFFUSE ? 0u : diffuse_blocks_per_sm;
  return CLV_OK;
}

int clv_selftest_division(uint64_t n, uint64_t seed, uint64_t* mismatches) {
  if (!mismatches) return fail(CLV_E_INVALID, "null argument");
  try {
    unsigned long long* bad = nullptr;
    ck(cudaMalloc(&bad, sizeof(unsigned long long)), "cudaMalloc");
    ck(cudaMemset(bad, 0, sizeof(unsigned long long)), "cudaMemset");
    selftest_division_kernel<<<launch_grid(n, 256), 256>>>(n, seed, 0, bad);
    selftest_division_kernel<<<launch_grid(n, 256), 256>>>(n, seed + 1, 1, bad);
    unsigned long long h = 0;
    const cudaError_t e = cudaMemcpy(&h, bad, sizeof h, cudaMemcpyDeviceToHost);
    cudaFree(bad);
    ck(e, "selftest");
    *mismatches = h;
    return CLV_OK;
  } catch (std::exception& e) {
    return fail(CLV_E_CUDA, e.what());
  }
}

int clv_selftest_log(const float* x, float* y, uint64_t n, double* max_ulp, uint64_t* not_nearest) {
  if (!max_ulp || !not_nearest || (n && (!x || !y))) return fail(CLV_E_INVALID, "null argument");
  void* buf = nullptr;
  try {
    const size_t io = (size_t)n * sizeof(float);
    ck(cudaMalloc(&buf, 16 + 2 * io), "cudaMalloc");
    unsigned long long* acc = static_cast<unsigned long long*>(buf);
    ck(cudaMemset(acc, 0, 16), "cudaMemset");
    selftest_log_kernel<<<sm_count() * 8, 256>>>(acc, acc + 1);
    g_launches += 1;
    if (n) {
      float* dx = reinterpret_cast<float*>(static_cast<char*>(buf) + 16);
      float* dy = dx + n;
      ck(cudaMemcpy(dx, x, io, cudaMemcpyHostToDevice), "cudaMemcpy H2D");
      log_eval_kernel<<<(uint32_t)((n + 255) / 256), 256>>>(dx, dy, n);
      g_launches += 1;
      ck(cudaMemcpy(y, dy, io, cudaMemcpyDeviceToHost), "cudaMemcpy D2H");
    }
    unsigned long long h[2];
    ck(cudaMemcpy(h, acc, sizeof h, cudaMemcpyDeviceToHost), "cudaMemcpy D2H");
    cudaFree(buf);
    buf = nullptr;
    double m;
    std::memcpy(&m, &h[0], sizeof m);
    *max_ulp = m;
    *not_nearest = h[1];
    return CLV_OK;
  } catch (std::exception& e) {
    if (buf) cudaFree(buf);
    return fail(CLV_E_CUDA, e.what());
  }
}

int clv_scene_load_json_text(const char* json, const char* base_dir, uint32_t width, uint32_t height, int bvh_alg,
                             clv_scene** out) {
  if (!json || !out) return fail(CLV_E_INVALID, "null argument");
  if (bvh_alg != CLV_BVH_SAH && bvh_alg != CLV_BVH_LAM) return fail(CLV_E_INVALID, "unknown BVH algorithm");
  try {
    std::unique_ptr<clv_scene> s(new clv_scene());
    s->host = clv::load_scene_text(json, width, height, base_dir ? base_dir : ".", bvh_alg == CLV_BVH_LAM);
    if (s->host.mis_depth > CLV_MIS_STACK) return fail(CLV_E_SCENE, "MIS tree deeper than its evaluation stack");
    *out = s.release();
    return CLV_OK;
  } catch (std::exception& e) {
    return fail(CLV_E_SCENE, e.what());
  }
}

int clv_scene_load_json(const char* path, uint32_t width, uint32_t height, int bvh_alg, clv_scene** out) {
  if (!path || !out) return fail(CLV_E_INVALID, "null argument");
  if (bvh_alg != CLV_BVH_SAH && bvh_alg != CLV_BVH_LAM) return fail(CLV_E_INVALID, "unknown BVH algorithm");
  try {
    std::unique_ptr<clv_scene> s(new clv_scene());
    s->host = clv::load_scene_json(path, width, height, bvh_alg == CLV_BVH_LAM);
    if (s->host.mis_depth > CLV_MIS_STACK) return fail(CLV_E_SCENE, "MIS tree deeper than its evaluation stack");
    *out = s.release();
    return CLV_OK;
  } catch (std::exception& e) {
    return fail(CLV_E_SCENE, e.what());
  }
}

int clv_scene_from_mesh(const float* verts, uint32_t nverts, const uint32_t* indices, uint32_t ntris,
                        clv_scene** out) {
  if (!verts || !indices || !out) return fail(CLV_E_INVALID, "null argument");
  try {
    std::unique_ptr<clv_scene> s(new clv_scene());
    s->host = clv::mesh_scene(verts, nverts, indices, ntris);
    *out = s.release();
    return CLV_OK;
  } catch (std::exception& e) {
    return fail(CLV_E_SCENE, e.what());
  }
}

int clv_scene_info_get(const clv_scene* s, clv_scene_info* out) {
  if (!s || !out) return fail(CLV_E_INVALID, "null argument");
  const clv::HostScene& h = s->host;
  out->objects = h.object_count;
  out->nodes = (uint32_t)h.nodes.size();
  out->triangles = (uint32_t)h.tris.size();
  out->quads = (uint32_t)h.quads.size();
  out->spheres = (uint32_t)(h.spheres.size() / 4);
  out->compound = (uint32_t)h.objs.size();
  out->materials = (uint32_t)h.materials.size();
  out->tree_depth = h.tree_depth;
  out->mis_nodes = (uint32_t)h.mis_nodes.size();
  out->width = h.width;
  out->height = h.height;
  out->traversal_level = compound_level(h);
  return CLV_OK;
}

void clv_scene_free(clv_scene* s) { delete s; }

int clv_scene_set_option(clv_scene* s, uint32_t option, uint32_t value) {
  if (!s) return fail(CLV_E_INVALID, "null argument");
  if (option == CLV_OPT_WATERTIGHT) {
    if (value > 1) return fail(CLV_E_INVALID, "CLV_OPT_WATERTIGHT takes 0 or 1");
    s->watertight = value;
    return CLV_OK;
  }
  return fail(CLV_E_INVALID, "unknown scene option");
}

int clv_scene_upload(const clv_scene* s, clv_device_scene** out) {
  if (!s || !out) return fail(CLV_E_INVALID, "null argument");
  try {
    const clv::HostScene& h = s->host;
    std::unique_ptr<clv_device_scene> d(new clv_device_scene());
    ClvDeviceScene& v = d->view;
    UploadPack pk;
    pk.add(h.nodes, &v.nodes);
    pk.add(h.tris, &v.tris);
    pk.add(h.quads, &v.quads);
    pk.add(h.spheres, &v.spheres);
    pk.add(h.objs, &v.objs);
    pk.add(h.obj_children, &v.obj_children);
    pk.add(h.tri_gid, &v.tri_gid);
    pk.add(h.quad_gid, &v.quad_gid);
    pk.add(h.sphere_gid, &v.sphere_gid);
    pk.add(h.obj_gid, &v.obj_gid);
    pk.add(h.tri_mat, &v.tri_mat);
    pk.add(h.quad_mat, &v.quad_mat);
    pk.add(h.sphere_mat, &v.sphere_mat);
    pk.add(h.tri_area, &v.tri_area);
    pk.add(h.quad_area, &v.quad_area);
    pk.add(h.materials, &v.materials);
    pk.add(h.spd, &v.spd);
    std::vector<float> ill((size_t)clv_tables::kNumIlluminants * 400);
    std::memcpy(ill.data(), clv_tables::kIlluminants, ill.size() * sizeof(float));
    pk.add(ill, &v.illuminant);
    std::vector<float> cmf(400 * 3);
    for (int i = 0; i < 400; ++i) clv::wavelength_to_xyz(380 + i, &cmf[3 * i]);
    pk.add(cmf, &v.cmf);
    pk.add(h.mis_nodes, &v.mis_nodes);
    v.tri_verts = nullptr;
    if (s->watertight && !h.tri_verts.empty()) pk.add(h.tri_verts, &v.tri_verts);
    const size_t off_err = pk.reserve(sizeof(uint32_t)), off_next = pk.reserve(sizeof(unsigned long long));
    char* base = pk.commit(d->owned, &d->owned_bytes);
    d->err = reinterpret_cast<uint32_t*>(base + off_err);
    d->ray_next = reinterpret_cast<unsigned long long*>(base + off_next);
    v.root = h.root;
    v.mis_root = h.mis_root;
    std::memcpy(v.root_box, h.root_box, sizeof v.root_box);
    v.background_spd = h.background_spd;
    v.n_nodes = (uint32_t)h.nodes.size();
    v.n_tris = (uint32_t)h.tris.size();
    v.n_quads = (uint32_t)h.quads.size();
    v.n_spheres = (uint32_t)(h.spheres.size() / 4);
    v.n_objs = (uint32_t)h.objs.size();
    v.n_materials = (uint32_t)h.materials.size();
    v.max_depth_tree = h.tree_depth;
    v.compound_level = compound_level(h);
    v.boxes_div_safe = boxes_div_safe(h) ? 1u : 0u;
    v.mis_depth = h.mis_depth;
    v.camera = h.camera;
    v.watertight = s->watertight;
    ck(cudaMemset(d->err, 0, sizeof(uint32_t)), "cudaMemset");
    d->width = h.width;
    d->height = h.height;
    d->has_camera = h.width > 0 && h.mis_root != CLV_REF_EMPTY;
    *out = d.release();
    return CLV_OK;
  } catch (std::exception& e) {
    return fail(CLV_E_CUDA, e.what());
  }
}

void clv_device_scene_free(clv_device_scene* d) { delete d; }

int clv_device_status(clv_device_scene* d, uint32_t* flags_out) {
  if (!d || !flags_out) return fail(CLV_E_INVALID, "null argument");
  try {
    ck(cudaMemcpy(flags_out, d->err, sizeof(uint32_t), cudaMemcpyDeviceToHost), "cudaMemcpy D2H");
    ck(cudaMemset(d->err, 0, sizeof(uint32_t)), "cudaMemset");
    return CLV_OK;
  } catch (std::exception& e) {
    return fail(CLV_E_CUDA, e.what());
  }
}

int clv_raycast_device(const clv_device_scene* d, const float* rays_dev, uint64_t n, uint32_t* prim_dev, float* t_dev,
                       uint32_t* nodes_dev, uint32_t* tests_dev, void* stream) {
  if (!d || (!rays_dev && n) || (!prim_dev && n) || (!t_dev && n)) return fail(CLV_E_INVALID, "null argument");
  if (n == 0) return CLV_OK;
  if ((reinterpret_cast<uintptr_t>(rays_dev) & 15u) != 0) return fail(CLV_E_INVALID, "rays must be 16-byte aligned");
  const int block = 128;
  g_launches += 1;
  // persistent grid: every resident block of the launch bound on every SM
  uint32_t grid = (uint32_t)std::max<uint64_t>(
      1, std::min<uint64_t>((n + block - 1) / block, (uint64_t)sm_count() * CLV_MINB_RAY));
  float4* spill = nullptr;
  const uint32_t spill_entries = d->spill_entries();
  if (spill_entries) {  // deep tree: fewer threads if the spill region would exceed its budget
    const uint64_t per_block = (uint64_t)block * spill_entries * sizeof(float4);
    grid = (uint32_t)std::max<uint64_t>(1, std::min<uint64_t>(grid, kSpillBudget / per_block));
    try {
      spill = const_cast<clv_device_scene*>(d)->spill_region(grid * per_block);
    } catch (std::exception& ex) {
      return fail(CLV_E_CUDA, ex.what());
    }
  }
  const float4* r4 = reinterpret_cast<const float4*>(rays_dev);
  cudaStream_t st = (cudaStream_t)stream;
  cudaError_t e = cudaMemsetAsync(d->ray_next, 0, sizeof(unsigned long long), st);
  if (e != cudaSuccess) return fail(CLV_E_CUDA, std::string("cudaMemsetAsync: ") + cudaGetErrorString(e));
  unsigned long long* nx = d->ray_next;
  const bool count = nodes_dev || tests_dev;
  // traversal order (small batches go in their own order)
  const uint32_t* perm = nullptr;
  if (n >= (1u << 16) && n <= 0xFFFFFFFFull) {
    uint32_t* hist = nullptr;
    try {
      hist = const_cast<clv_device_scene*>(d)->ray_sort_scratch(n);
    } catch (std::exception& ex) {
      return fail(CLV_E_CUDA, ex.what());
    }
    uint32_t* keys = hist + CLV_SORT_BINS;
    uint32_t* order = keys + n;
    const float* b = d->view.root_box;
    const float side = (float)(1u << CLV_SORT_AXIS_BITS);
    auto sc = [&](int a) { return b[2 * a + 1] > b[2 * a] ? side / (b[2 * a + 1] - b[2 * a]) : 0.0f; };
    const float3 lo = make_float3(b[0], b[2], b[4]), scale = make_float3(sc(0), sc(1), sc(2));
    const uint32_t sg = launch_grid(n, 256);
    e = cudaMemsetAsync(hist, 0, CLV_SORT_BINS * sizeof(uint32_t), st);
    if (e != cudaSuccess) return fail(CLV_E_CUDA, std::string("cudaMemsetAsync: ") + cudaGetErrorString(e));
    ray_key_hist<<<sg, 256, 0, st>>>(r4, n, lo, scale, keys, hist);
    ray_bins_scan<<<1, 1024, 0, st>>>(hist);
    ray_scatter<<<sg, 256, 0, st>>>(keys, n, hist, order);
    g_launches += 3;
    perm = order;
  }
#define CLV_RAYCAST(C, N, W) \
  raycast_persist_kernel<C, N, W><<<grid, block, 0, st>>>(d->view, r4, n, prim_dev, t_dev, nodes_dev, tests_dev, d->err, nx, perm, nullptr, 0)
  const int wt = d->view.watertight ? 1 : 0;
  const int cap = (int)d->view.max_depth_tree;
  if (spill_entries && count)
    raycast_persist_kernel<2, true, CLV_WT_SCENE, true><<<grid, block, 0, st>>>(
        d->view, r4, n, prim_dev, t_dev, nodes_dev, tests_dev, d->err, nx, perm, spill, cap);
  else if (spill_entries)
    raycast_persist_kernel<2, false, CLV_WT_SCENE, true><<<grid, block, 0, st>>>(
        d->view, r4, n, prim_dev, t_dev, nodes_dev, tests_dev, d->err, nx, perm, spill, cap);
  else switch ((d->view.compound_level * 2 + (count ? 1 : 0)) * 2 + wt) {
    case 0: CLV_RAYCAST(0, false, CLV_WT_OFF); break;
    case 1: CLV_RAYCAST(0, false, CLV_WT_ON); break;
    case 2: CLV_RAYCAST(0, true, CLV_WT_OFF); break;
    case 3: CLV_RAYCAST(0, true, CLV_WT_ON); break;
    case 4: CLV_RAYCAST(1, false, CLV_WT_OFF); break;
    case 5: CLV_RAYCAST(1, false, CLV_WT_ON); break;
    case 6: CLV_RAYCAST(1, true, CLV_WT_OFF); break;
    case 7: CLV_RAYCAST(1, true, CLV_WT_ON); break;
    case 8: CLV_RAYCAST(2, false, CLV_WT_OFF); break;
    case 9: CLV_RAYCAST(2, false, CLV_WT_ON); break;
    case 10: CLV_RAYCAST(2, true, CLV_WT_OFF); break;
    default: CLV_RAYCAST(2, true, CLV_WT_ON); break;
  }
#undef CLV_RAYCAST
  e = cudaGetLastError();
  if (e != cudaSuccess) return fail(CLV_E_CUDA, std::string("raycast launch: ") + cudaGetErrorString(e));
  return CLV_OK;
}

int clv_raycast(clv_device_scene* d, const float* rays, uint64_t n, uint32_t* prim, float* t, uint32_t* nodes,
                uint32_t* tests) {
  if (!d || (!rays && n) || (!prim && n) || (!t && n)) return fail(CLV_E_INVALID, "null argument");
  if (n == 0) return CLV_OK;
  try {
    const size_t rb = n * 32, ob = n * 4;
    const size_t total = rb + 4 * ob;
    char* base = static_cast<char*>(d->ensure_scratch(total));
    float* drays = reinterpret_cast<float*>(base);
    uint32_t* dprim = reinterpret_cast<uint32_t*>(base + rb);
    float* dt = reinterpret_cast<float*>(base + rb + ob);
    uint32_t* dnodes = nodes ? reinterpret_cast<uint32_t*>(base + rb + 2 * ob) : nullptr;
    uint32_t* dtests = tests ? reinterpret_cast<uint32_t*>(base + rb + 3 * ob) : nullptr;
    ck(cudaMemcpy(drays, rays, rb, cudaMemcpyHostToDevice), "cudaMemcpy H2D");
    int rc = clv_raycast_device(d, drays, n, dprim, dt, dnodes, dtests, nullptr);
    if (rc) return rc;
    ck(cudaMemcpy(prim, dprim, ob, cudaMemcpyDeviceToHost), "cudaMemcpy D2H");
    ck(cudaMemcpy(t, dt, ob, cudaMemcpyDeviceToHost), "cudaMemcpy D2H");
    if (nodes) ck(cudaMemcpy(nodes, dnodes, ob, cudaMemcpyDeviceToHost), "cudaMemcpy D2H");
    if (tests) ck(cudaMemcpy(tests, dtests, ob, cudaMemcpyDeviceToHost), "cudaMemcpy D2H");
    uint32_t flags = 0;
    ck(cudaMemcpy(&flags, d->err, 4, cudaMemcpyDeviceToHost), "cudaMemcpy D2H");
    if (flags) {
      cudaMemset(d->err, 0, 4);
      return fail(CLV_E_DEVICE, "kernel error flags " + std::to_string(flags));
    }
    return CLV_OK;
  } catch (std::exception& e) {
    return fail(CLV_E_CUDA, e.what());
  }
}

// Wavefront render loop.  With `prof` set, each intersect and shade launch is
// bracketed by events, and with `count` as well the intersect launches are the
// counting variants that also fill prof's traversal counts.  (The counting
// variants are slower, so device times come from a render without them.)
// bracketed by events and the traversal work is counted (diagnostic runs).
// With `guide` set, Lambertian bounces go through the guided kernels (a share
// alpha drawn from the guide network) and leave training records.
static int render_wavefront(clv_device_scene* d, const clv_render_opts* o, double* film, cudaStream_t st,
                            clv_render_profile* prof, clv_guide* guide, float alpha, bool count) {
  std::vector<cudaEvent_t> evs;
  unsigned long long* dcnt = nullptr;
  auto cleanup = [&]() {
    for (cudaEvent_t e : evs) cudaEventDestroy(e);
    evs.clear();
    if (dcnt) cudaFree(dcnt);
    dcnt = nullptr;
  };
  try {
    WfParams P;
    P.width = o->width;
    P.height = o->height;
    P.max_depth = o->max_depth;
    P.sample_offset = o->sample_offset;
    P.npix = (uint64_t)o->width * o->height;
    P.total = P.npix * o->samples;
    P.seed = o->seed;
    uint64_t q = o->path_slots ? o->path_slots : d->tuned_slots ? d->tuned_slots : (uint64_t)sm_count() * 2048 * 4;
    q = std::min<uint64_t>(q, P.total);
    const uint32_t spill_entries = d->spill_entries();
    if (spill_entries)  // deep tree: fewer paths in flight if their stack spill would exceed its budget
      q = std::min<uint64_t>(q, kSpillBudget / ((uint64_t)spill_entries * sizeof(float4)));
    q = std::max<uint64_t>(128, (q + 127) / 128 * 128);
    WfState W = d->wavefront_state((uint32_t)q);
    if (spill_entries) {
      W.spill = d->spill_region((size_t)q * spill_entries * sizeof(float4));
      W.stack_cap = d->view.max_depth_tree;
    }
    WfCounters c0{std::min<uint64_t>(q, P.total), 0u, {0u, 0u, 0u, 0u}};
    ck(cudaMemcpyAsync(d->wf_counters, &c0, sizeof c0, cudaMemcpyHostToDevice, st), "cudaMemcpyAsync");
    GuideDev G{};
    GdQueue GQ{};
    if (guide) {
      W.gslot = guide->ensure_slots((uint32_t)q);
      W.grec = guide->rec;
      W.grec_count = guide->rec_count;
      W.grec_cap = guide->rec_cap;
      gd_reset_records(guide, st);
      G = gd_view(guide, d->view.root_box, alpha);
      GQ = GdQueue{W.queue + (size_t)WF_Q_GUIDE * q, &d->wf_counters->queue[WF_Q_GUIDE], W.full, W.d_lambda, W.hit,
                   W.meta, W.key};
    }
    const int block = 128;
    const uint32_t grid = (uint32_t)((q + block - 1) / block);
    const uint32_t level = d->view.compound_level;
    const int batch = 8;  // bounces between polls of the live-path counter
    WfCounters* C = d->wf_counters;
    // shading kernels walk their queues with a grid-stride loop over a fixed grid
    const uint32_t qgrid =
        std::min<uint32_t>(grid, (uint32_t)sm_count() * (d->tuned_shade ? d->tuned_shade : CLV_SHADE_BLOCKS));
    const uint32_t pgrid = scaled_grid(grid, d->tuned_shade, CLV_MINB_GUIDE_POST);
    if (prof) {
      std::memset(prof, 0, sizeof *prof);
      ck(cudaMalloc(&dcnt, 3 * sizeof(unsigned long long)), "cudaMalloc");
      ck(cudaMemsetAsync(dcnt, 0, 3 * sizeof(unsigned long long), st), "cudaMemsetAsync");
      evs.resize(4 * batch + 2);
      for (auto& e : evs) ck(cudaEventCreate(&e), "cudaEventCreate");
      ck(cudaEventRecord(evs[4 * batch], st), "cudaEventRecord");
    }
    wf_init<false><<<grid, block, 0, st>>>(d->view, P, W, WfBatch{});
    g_launches += 1;
    if (prof) {
      ck(cudaEventRecord(evs[4 * batch + 1], st), "cudaEventRecord");
      ck(cudaEventSynchronize(evs[4 * batch + 1]), "cudaEventSynchronize");
      float ms = 0.0f;
      cudaEventElapsedTime(&ms, evs[4 * batch], evs[4 * batch + 1]);
      prof->ms_init = ms;
    }
    // one bounce: counters, closest hits, the shading passes, path ends
    const bool fork = d->fork_streams();
    auto bounce = [&](cudaStream_t s, int k) {
      cudaMemsetAsync(&d->wf_counters->live, 0, 5 * sizeof(unsigned int), s);  // live + 4 queue lengths
      if (prof) cudaEventRecord(evs[4 * k], s);
#define CLV_ISECT(L, N, T) \
  wf_intersect<L, N, false, T><<<grid, block, 0, s>>>(d->view, W, C, d->err, N ? dcnt : nullptr, WfBatch{}, -1)
      // per-warp appends (primitive-level scenes only, as tuned)
      const bool wapp = level == 0 && d->tuned_append && !spill_entries;
#define CLV_ISECT_W(N, T) \
  wf_intersect<0, N, false, T, false, true><<<grid, block, 0, s>>>(d->view, W, C, d->err, N ? dcnt : nullptr, WfBatch{}, -1)
      if (wapp) {
        const bool cnt = prof && count;
        if (d->view.watertight) {
          if (cnt) CLV_ISECT_W(true, CLV_WT_ON);
          else CLV_ISECT_W(false, CLV_WT_ON);
        } else {
          if (cnt) CLV_ISECT_W(true, CLV_WT_OFF);
          else CLV_ISECT_W(false, CLV_WT_OFF);
        }
      } else if (spill_entries && prof && count)
        wf_intersect<2, true, false, CLV_WT_SCENE, true><<<grid, block, 0, s>>>(d->view, W, C, d->err, dcnt,
                                                                                WfBatch{}, -1);
      else if (spill_entries)
        wf_intersect<2, false, false, CLV_WT_SCENE, true><<<grid, block, 0, s>>>(d->view, W, C, d->err, nullptr,
                                                                                 WfBatch{}, -1);
      else switch ((level * 2 + (prof && count ? 1 : 0)) * 2 + (d->view.watertight ? 1 : 0)) {
        case 0: CLV_ISECT(0, false, CLV_WT_OFF); break;
        case 1: CLV_ISECT(0, false, CLV_WT_ON); break;
        case 2: CLV_ISECT(0, true, CLV_WT_OFF); break;
        case 3: CLV_ISECT(0, true, CLV_WT_ON); break;
        case 4: CLV_ISECT(1, false, CLV_WT_OFF); break;
        case 5: CLV_ISECT(1, false, CLV_WT_ON); break;
        case 6: CLV_ISECT(1, true, CLV_WT_OFF); break;
        case 7: CLV_ISECT(1, true, CLV_WT_ON); break;
        case 8: CLV_ISECT(2, false, CLV_WT_OFF); break;
        case 9: CLV_ISECT(2, false, CLV_WT_ON); break;
        case 10: CLV_ISECT(2, true, CLV_WT_OFF); break;
        default: CLV_ISECT(2, true, CLV_WT_ON); break;
      }
#undef CLV_ISECT
#undef CLV_ISECT_W
      if (prof) cudaEventRecord(evs[4 * k + 1], s);
      if (prof) cudaEventRecord(evs[4 * k + 2], s);
      if (fork) {
        cudaEventRecord(d->ev_fork, s);
        cudaStreamWaitEvent(d->side_stream, d->ev_fork, 0);
      }
      wf_shade_specular<false><<<qgrid, block, 0, fork ? d->side_stream : s>>>(d->view, P, W, C, d->err, WfBatch{});
      if (fork) cudaEventRecord(d->ev_join, d->side_stream);
      launch_shade_diffuse<false>(d->tuned_diffuse, grid, d->tuned_shade, s, d->view, P, W, C, d->err, WfBatch{});
      if (guide) {
        wf_guide_pre<false><<<qgrid, block, 0, s>>>(d->view, W, C, alpha, WfBatch{});
        if (alpha > 0.0f) gd_launch_queue(G, GQ, (uint32_t)q, s);
        wf_guide_post<false><<<pgrid, block, 0, s>>>(d->view, P, W, C, d->err, G, WfBatch{});
      }
      if (fork) cudaStreamWaitEvent(s, d->ev_join, 0);
      wf_finish<false><<<qgrid, block, 0, s>>>(d->view, P, W, C, film, WfBatch{});
      if (prof) cudaEventRecord(evs[4 * k + 3], s);
    };
    const unsigned per_bounce = 4u + (guide ? (alpha > 0.0f ? 3u : 2u) : 0u);
    if (guide) gd_prepare();
    // the batch of bounces between polls, replayed as one CUDA graph (profiling
    // runs launch directly: their events bracket single kernels)
    GraphExec graph;
    if (!prof) graph = capture_graph(d, [&](cudaStream_t s) {
      for (int k = 0; k < batch; ++k) bounce(s, k);
    });
    for (uint64_t it = 0;; it += batch) {
      if (graph.exec) {
        ck(cudaGraphLaunch(graph.exec, st), "cudaGraphLaunch");
      } else {
        for (int k = 0; k < batch; ++k) bounce(st, k);
      }
      g_launches += per_bounce * batch;
      ck(cudaGetLastError(), "wavefront launch");
      ck(cudaMemcpyAsync(d->wf_live_host, &d->wf_counters->live, sizeof(unsigned int), cudaMemcpyDeviceToHost, st),
         "cudaMemcpyAsync");
      ck(cudaStreamSynchronize(st), "cudaStreamSynchronize");
      if (prof) {
        for (int k = 0; k < batch; ++k) {
          float a = 0.0f, b = 0.0f;
          cudaEventElapsedTime(&a, evs[4 * k], evs[4 * k + 1]);
          cudaEventElapsedTime(&b, evs[4 * k + 2], evs[4 * k + 3]);
          prof->ms_intersect += a;
          prof->ms_shade += b;
        }
        prof->intersect_launches += batch;
        prof->shade_launches += batch;
      }
      if (*d->wf_live_host == 0) break;
      if (it > (uint64_t)4 * (P.total / q + 1) * (o->max_depth + 2) + 64)
        throw std::runtime_error("wavefront did not drain");  // unreachable unless a kernel misbehaves
    }
    if (prof) {
      unsigned long long h[3];
      ck(cudaMemcpy(h, dcnt, sizeof h, cudaMemcpyDeviceToHost), "cudaMemcpy D2H");
      if (count) {
        prof->path_segments = h[0];
        prof->node_visits = h[1];
        prof->prim_tests = h[2];
      }
      prof->paths = P.total;
      prof->path_slots = q;
    }
    cleanup();
    return CLV_OK;
  } catch (std::exception& e) {
    cleanup();
    return fail(CLV_E_CUDA, e.what());
  }
}

// The multi-scene wavefront; with `guide`, Lambertian bounces of every scene
// go through the one guide (alpha as in clv_render_guided), positions
// normalised to each scene's own box.
// One wavefront over at most CLV_BATCH_MAX scenes (arguments checked by the caller).
// Holds the constant-memory scene tables until its last launch has finished.
static int render_batch_part(clv_device_scene* const* ds, const clv_render_opts* opts, double* const* films,
                             uint32_t n, cudaStream_t st, clv_guide* guide, float alpha, bool reset_records) {
  static std::mutex tables_mu;
  std::lock_guard<std::mutex> lock(tables_mu);
  void* dmem = nullptr;
  try {
    // The work items are laid out scene after scene, the scenes ordered by the
    // traversal level they need (a stable sort), so that for most of the render
    // the live paths belong to one level and the other levels' intersect
    // launches find next to nothing to do.  Films and random streams stay with
    // their scenes.
    std::vector<uint32_t> order(n);
    for (uint32_t k = 0; k < n; ++k) order[k] = k;
    std::stable_sort(order.begin(), order.end(), [&](uint32_t a, uint32_t b) {
      return ds[a]->view.compound_level < ds[b]->view.compound_level;
    });
    std::vector<ClvDeviceScene> views(n);
    std::vector<WfParams> params(n);
    std::vector<unsigned long long> prefix(n + 1, 0ull);
    std::vector<double*> fl(n);
    uint32_t levels = 0;  // bit L: some scene needs traversal level L
    for (uint32_t j = 0; j < n; ++j) {
      const uint32_t k = order[j];
      views[j] = ds[k]->view;
      fl[j] = films[k];
      const clv_render_opts& o = opts[k];
      WfParams& P = params[j];
      P.width = o.width;
      P.height = o.height;
      P.max_depth = o.max_depth;
      P.sample_offset = o.sample_offset;
      P.npix = (uint64_t)o.width * o.height;
      P.total = P.npix * o.samples;
      P.seed = o.seed;
      prefix[j + 1] = prefix[j] + P.total;
      levels |= 1u << ds[k]->view.compound_level;
    }
    const int nlevels = __builtin_popcount(levels);
    const unsigned long long total = prefix[n];
    // one staging allocation for the batch tables
    ck(cudaMemcpyToSymbolAsync(wf_bscene, views.data(), n * sizeof(ClvDeviceScene), 0, cudaMemcpyHostToDevice, st),
       "cudaMemcpyToSymbolAsync");
    ck(cudaMemcpyToSymbolAsync(wf_bparam, params.data(), n * sizeof(WfParams), 0, cudaMemcpyHostToDevice, st),
       "cudaMemcpyToSymbolAsync");
    const size_t b_prefix = (n + 1) * sizeof(unsigned long long), b_films = n * sizeof(double*);
    const size_t b_boxes = guide ? n * 6 * sizeof(float) : 0;
    auto up = [](size_t x) { return (x + 255) / 256 * 256; };
    const size_t bytes = up(b_prefix) + up(b_films) + up(b_boxes);
    ck(cudaMalloc(&dmem, bytes), "cudaMalloc batch tables");
    char* c = static_cast<char*>(dmem);
    WfBatch B;
    B.prefix = reinterpret_cast<const unsigned long long*>(c);
    ck(cudaMemcpyAsync(c, prefix.data(), b_prefix, cudaMemcpyHostToDevice, st), "cudaMemcpyAsync");
    c += up(b_prefix);
    B.films = reinterpret_cast<double* const*>(c);
    ck(cudaMemcpyAsync(c, fl.data(), b_films, cudaMemcpyHostToDevice, st), "cudaMemcpyAsync");
    c += up(b_films);
    std::vector<float> boxes(guide ? n * 6 : 0);
    for (uint32_t j = 0; guide && j < n; ++j)  // {bmin, 1 / extent} of each scene's box, batch order
      for (int a = 0; a < 3; ++a) {
        const float lo = views[j].root_box[2 * a], ext = views[j].root_box[2 * a + 1] - lo;
        boxes[6 * j + a] = lo;
        boxes[6 * j + 3 + a] = ext > 0.0f ? 1.0f / ext : 0.0f;
      }
    if (guide) ck(cudaMemcpyAsync(c, boxes.data(), b_boxes, cudaMemcpyHostToDevice, st), "cudaMemcpyAsync");
    const float* dboxes = guide ? reinterpret_cast<const float*>(c) : nullptr;
    B.n = n;
    B.total = total;
    clv_device_scene* d0 = ds[0];  // path state, counters and the error word come from the first scene
    // paths in flight: the caller's, the first scene's tuned pool, else a sixteenth
    // of the batch's work items between a single render's default and four times
    // that (a large batch has no per-scene tails to keep short: the 64 scenes of
    // C5, 2.66 G samples, at 4,980,736 paths 394.8 Msamples/s, at 1,245,184
    // 372.9; the same scenes at 128^2 x 16 spp, 16.8 M samples, 61.3 ms at
    // 1,245,184 paths and 71.8 ms at 4,980,736)
    const uint64_t q1 = (uint64_t)sm_count() * 2048 * 4;
    uint64_t q = opts[0].path_slots ? opts[0].path_slots
                 : d0->tuned_slots    ? d0->tuned_slots
                                      : std::min<uint64_t>(4 * q1, std::max<uint64_t>(q1, total / 16));
    q = std::min<uint64_t>(q, total);
    uint32_t spill_entries = 0, stack_cap = CLV_STACK;  // the deepest tree of the batch
    for (uint32_t k = 0; k < n; ++k) {
      spill_entries = std::max(spill_entries, ds[k]->spill_entries());
      stack_cap = std::max(stack_cap, ds[k]->view.max_depth_tree);
    }
    if (spill_entries) q = std::min<uint64_t>(q, kSpillBudget / ((uint64_t)spill_entries * sizeof(float4)));
    q = std::max<uint64_t>(128, (q + 127) / 128 * 128);
    WfState W = d0->wavefront_state((uint32_t)q);
    if (spill_entries) {
      W.spill = d0->spill_region((size_t)q * spill_entries * sizeof(float4));
      W.stack_cap = stack_cap;
    }
    WfCounters c0{std::min<unsigned long long>(q, total), 0u, {0u, 0u, 0u, 0u}};
    ck(cudaMemcpyAsync(d0->wf_counters, &c0, sizeof c0, cudaMemcpyHostToDevice, st), "cudaMemcpyAsync");
    WfCounters* C = d0->wf_counters;
    GuideDev G{};
    GdQueue GQ{};
    if (guide) {
      W.gslot = guide->ensure_slots((uint32_t)q);
      W.grec = guide->rec;
      W.grec_count = guide->rec_count;
      W.grec_cap = guide->rec_cap;
      if (reset_records) gd_reset_records(guide, st);
      G = gd_view(guide, d0->view.root_box, alpha);
      G.boxes = dboxes;
      GQ = GdQueue{W.queue + (size_t)WF_Q_GUIDE * q, &C->queue[WF_Q_GUIDE], W.full, W.d_lambda, W.hit, W.meta, W.key};
      gd_prepare();
    }
    const int block = 128;
    const uint32_t grid = (uint32_t)((q + block - 1) / block);
    const uint32_t qgrid =
        std::min<uint32_t>(grid, (uint32_t)sm_count() * (d0->tuned_shade ? d0->tuned_shade : CLV_SHADE_BLOCKS));
    const uint32_t pgrid = scaled_grid(grid, d0->tuned_shade, CLV_MINB_GUIDE_POST);
    const ClvDeviceScene& S0 = d0->view;
    const WfParams P0 = params[0];
    wf_init<true><<<grid, block, 0, st>>>(S0, P0, W, B);
    g_launches += 1;
    uint32_t max_depth = 0;
    for (uint32_t k = 0; k < n; ++k) max_depth = std::max(max_depth, opts[k].max_depth);
    const int batch = 8;
    const bool fork = d0->fork_streams();
    auto bounces = [&](cudaStream_t s) {
      for (int k = 0; k < batch; ++k) {
        cudaMemsetAsync(&C->live, 0, 5 * sizeof(unsigned int), s);
        // one intersect launch per traversal level present, each over its own scenes' slots
        // (a batch with a tree deeper than CLV_STACK levels: one generic launch with a spilling stack)
        // (several levels: the lowest level's launch runs on the second stream,
        // beside the others; their slots are disjoint)
        const int only = nlevels > 1 ? 0 : -1;
        if (spill_entries) {
          wf_intersect<2, false, true, CLV_WT_SCENE, true><<<grid, block, 0, s>>>(S0, W, C, d0->err, nullptr, B, -1);
        } else {
          const bool split = fork && nlevels > 1;
          if (split) {
            cudaEventRecord(d0->ev_fork, s);
            cudaStreamWaitEvent(d0->side_stream, d0->ev_fork, 0);
          }
          const uint32_t lowest = levels & (0u - levels);
          auto sl = [&](uint32_t bit) { return split && bit == lowest ? d0->side_stream : s; };
          if (levels & 1u)
            wf_intersect<0, false, true, CLV_WT_SCENE><<<grid, block, 0, sl(1u)>>>(S0, W, C, d0->err, nullptr, B, only);
          if (levels & 2u)
            wf_intersect<1, false, true, CLV_WT_SCENE><<<grid, block, 0, sl(2u)>>>(S0, W, C, d0->err, nullptr, B,
                                                                                  only < 0 ? -1 : 1);
          if (levels & 4u)
            wf_intersect<2, false, true, CLV_WT_SCENE><<<grid, block, 0, sl(4u)>>>(S0, W, C, d0->err, nullptr, B,
                                                                                  only < 0 ? -1 : 2);
          if (split) {
            cudaEventRecord(d0->ev_join, d0->side_stream);
            cudaStreamWaitEvent(s, d0->ev_join, 0);
          }
        }
        if (fork) {  // specular shading beside the diffuse and guided kernels
          cudaEventRecord(d0->ev_fork, s);
          cudaStreamWaitEvent(d0->side_stream, d0->ev_fork, 0);
        }
        wf_shade_specular<true><<<qgrid, block, 0, fork ? d0->side_stream : s>>>(S0, P0, W, C, d0->err, B);
        if (fork) cudaEventRecord(d0->ev_join, d0->side_stream);
        launch_shade_diffuse<true>(d0->tuned_diffuse, grid, d0->tuned_shade, s, S0, P0, W, C, d0->err, B);
        if (guide) {
          wf_guide_pre<true><<<qgrid, block, 0, s>>>(S0, W, C, alpha, B);
          if (alpha > 0.0f) gd_launch_queue(G, GQ, (uint32_t)q, s);
          wf_guide_post<true><<<pgrid, block, 0, s>>>(S0, P0, W, C, d0->err, G, B);
        }
        if (fork) cudaStreamWaitEvent(s, d0->ev_join, 0);
        wf_finish<true><<<qgrid, block, 0, s>>>(S0, P0, W, C, nullptr, B);
      }
    };
    GraphExec graph = capture_graph(d0, bounces);
    for (uint64_t it = 0;; it += batch) {
      if (graph.exec) ck(cudaGraphLaunch(graph.exec, st), "cudaGraphLaunch");
      else bounces(st);
      g_launches += (3 + (spill_entries ? 1 : nlevels) + (guide ? (alpha > 0.0f ? 3 : 2) : 0)) * batch;
      ck(cudaGetLastError(), "wavefront launch");
      ck(cudaMemcpyAsync(d0->wf_live_host, &C->live, sizeof(unsigned int), cudaMemcpyDeviceToHost, st),
         "cudaMemcpyAsync");
      ck(cudaStreamSynchronize(st), "cudaStreamSynchronize");
      if (*d0->wf_live_host == 0) break;
      if (it > (uint64_t)4 * (total / q + 1) * (max_depth + 2) + 64) throw std::runtime_error("wavefront did not drain");
    }
    cudaFree(dmem);
    return CLV_OK;
  } catch (std::exception& e) {
    if (dmem) {
      cudaStreamSynchronize(st);
      cudaFree(dmem);
    }
    return fail(CLV_E_CUDA, e.what());
  }
}

// A batch of more than CLV_BATCH_MAX scenes renders as consecutive wavefronts of
// CLV_BATCH_MAX scenes; a guided batch collects the training records of all of them.
static int render_batch(clv_device_scene* const* ds, const clv_render_opts* opts, double* const* films, uint32_t n,
                        void* stream, clv_guide* guide, float alpha) {
  if (!ds || !opts || !films || n == 0) return fail(CLV_E_INVALID, "null argument or empty batch");
  if (n > (1u << 24)) return fail(CLV_E_INVALID, "too many scenes in one batch");
  for (uint32_t k = 0; k < n; ++k) {
    const int rc = check_opts(ds[k], &opts[k]);
    if (rc) return rc;
    if (!films[k]) return fail(CLV_E_INVALID, "null film");
    if (opts[k].mode != CLV_MODE_PATH_TRACING) return fail(CLV_E_INVALID, "batches render path tracing only");
  }
  for (uint32_t k0 = 0; k0 < n; k0 += CLV_BATCH_MAX) {
    const uint32_t m = std::min<uint32_t>(CLV_BATCH_MAX, n - k0);
    const int rc = render_batch_part(ds + k0, opts + k0, films + k0, m, (cudaStream_t)stream, guide, alpha, k0 == 0);
    if (rc) return rc;
  }
  return CLV_OK;
}

int clv_render_batch(clv_device_scene* const* ds, const clv_render_opts* opts, double* const* films, uint32_t n,
                     void* stream) {
  return render_batch(ds, opts, films, n, stream, nullptr, 0.0f);
}

int clv_render_batch_guided(clv_device_scene* const* ds, const clv_render_opts* opts, double* const* films,
                            uint32_t n, clv_guide* g, float alpha, void* stream) {
  if (!g) return fail(CLV_E_INVALID, "null guide");
  if (!(alpha >= 0.0f && alpha <= 1.0f)) return fail(CLV_E_INVALID, "alpha must lie in [0, 1]");
  const int rc = render_batch(ds, opts, films, n, stream, g, alpha);
  if (rc) return rc;
  uint32_t e = 0;
  if (cudaMemcpy(&e, g->err, sizeof e, cudaMemcpyDeviceToHost) != cudaSuccess)
    return fail(CLV_E_CUDA, "cudaMemcpy D2H");
  if (e) {
    cudaMemset(g->err, 0, sizeof e);
    return fail(CLV_E_DEVICE, "guide kernel timed out waiting for the tensor cores");
  }
  return CLV_OK;
}

int clv_render_guided(clv_device_scene* d, const clv_render_opts* o, clv_guide* g, float alpha, double* film_dev,
                      void* stream) {
  int rc = check_opts(d, o);
  if (rc) return rc;
  if (!g || !film_dev) return fail(CLV_E_INVALID, "null argument");
  if (o->mode != CLV_MODE_PATH_TRACING)
    return fail(CLV_E_INVALID, "guided renders use the wavefront path tracer");
  if (!(alpha >= 0.0f && alpha <= 1.0f)) return fail(CLV_E_INVALID, "alpha must lie in [0, 1]");
  rc = render_wavefront(d, o, film_dev, (cudaStream_t)stream, nullptr, g, alpha);
  if (rc) return rc;
  uint32_t e = 0;
  if (cudaMemcpy(&e, g->err, sizeof e, cudaMemcpyDeviceToHost) != cudaSuccess)
    return fail(CLV_E_CUDA, "cudaMemcpy D2H");
  if (e) {
    cudaMemset(g->err, 0, sizeof e);
    return fail(CLV_E_DEVICE, "guide kernel timed out waiting for the tensor cores");
  }
  return CLV_OK;
}

int clv_render_device(clv_device_scene* d, const clv_render_opts* o, double* film_dev, void* stream) {
  int rc = check_opts(d, o);
  if (rc) return rc;
  if (!film_dev) return fail(CLV_E_INVALID, "null film");
  if (o->mode == CLV_MODE_PATH_TRACING) return render_wavefront(d, o, film_dev, (cudaStream_t)stream, nullptr);
  const int block = 128;
  const RenderParams P = make_params(o);
  float4* spill = nullptr;
  try {
    if (d->spill_entries()) spill = d->spill_region((size_t)P.npix * d->spill_entries() * sizeof(float4));
  } catch (std::exception& ex) {
    return fail(CLV_E_CUDA, ex.what());
  }
  g_launches += 1;
  debug_kernel<<<(uint32_t)((P.npix + block - 1) / block), block, 0, (cudaStream_t)stream>>>(d->view, P, film_dev,
                                                                                             d->err, spill);
  const cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return fail(CLV_E_CUDA, std::string("render launch: ") + cudaGetErrorString(e));
  return CLV_OK;
}

int clv_resolve_device(const double* film_dev, uint32_t width, uint32_t height, uint32_t spp, float* xyz_dev,
                       uint8_t* rgb_dev, void* stream) {
  if (!film_dev || spp == 0) return fail(CLV_E_INVALID, "bad argument");
  ResolveParams R;
  clv::m3_xyz_e_to_linsrgb(R.m);
  R.inv_spp = 1.0 / (double)spp;
  R.width = width;
  R.height = height;
  const uint64_t n = (uint64_t)width * height;
  if (n == 0) return CLV_OK;
  resolve_kernel<<<(uint32_t)((n + 255) / 256), 256, 0, (cudaStream_t)stream>>>(R, film_dev, xyz_dev, rgb_dev);
  g_launches += 1;
  const cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return fail(CLV_E_CUDA, std::string("resolve launch: ") + cudaGetErrorString(e));
  return CLV_OK;
}

int clv_render(clv_device_scene* d, const clv_render_opts* o, float* xyz_out, clv_stats* stats) {
  int rc = check_opts(d, o);
  if (rc) return rc;
  if (!xyz_out) return fail(CLV_E_INVALID, "null output");
  try {
    const uint64_t npix = (uint64_t)o->width * o->height;
    const size_t film_b = npix * 3 * sizeof(double), xyz_b = npix * 3 * sizeof(float);
    char* base = static_cast<char*>(d->ensure_scratch(film_b + xyz_b));
    double* film = reinterpret_cast<double*>(base);
    float* xyz = reinterpret_cast<float*>(base + film_b);
    cudaEvent_t e0, e1;
    ck(cudaEventCreate(&e0), "cudaEventCreate");
    ck(cudaEventCreate(&e1), "cudaEventCreate");
    ck(cudaMemsetAsync(film, 0, film_b, nullptr), "cudaMemset");
    ck(cudaEventRecord(e0, nullptr), "cudaEventRecord");
    rc = clv_render_device(d, o, film, nullptr);
    if (rc) {
      cudaEventDestroy(e0);
      cudaEventDestroy(e1);
      return rc;
    }
    ck(cudaEventRecord(e1, nullptr), "cudaEventRecord");
    if (o->mode == CLV_MODE_PATH_TRACING) {
      rc = clv_resolve_device(film, o->width, o->height, o->samples, xyz, nullptr, nullptr);
      if (rc) return rc;
      ck(cudaMemcpy(xyz_out, xyz, xyz_b, cudaMemcpyDeviceToHost), "cudaMemcpy D2H");
    } else {
      // debug modes store linear sRGB; convert to XYZ(E) like LinSrgb::adapt_into
      std::vector<double> tmp(npix * 3);
      ck(cudaMemcpy(tmp.data(), film, film_b, cudaMemcpyDeviceToHost), "cudaMemcpy D2H");
      for (uint64_t i = 0; i < npix; ++i) {
        const float lin[3] = {(float)tmp[3 * i], (float)tmp[3 * i + 1], (float)tmp[3 * i + 2]};
        clv::linsrgb_to_xyz_e(lin, xyz_out + 3 * i);
      }
    }
    float ms = 0.0f;
    ck(cudaEventSynchronize(e1), "cudaEventSynchronize");
    cudaEventElapsedTime(&ms, e0, e1);
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    uint32_t flags = 0;
    ck(cudaMemcpy(&flags, d->err, 4, cudaMemcpyDeviceToHost), "cudaMemcpy D2H");
    if (stats) {
      stats->gpu_ms = ms;
      stats->samples = npix * o->samples;
      stats->device_errors = flags;
      stats->kernel_launches = o->mode == CLV_MODE_PATH_TRACING ? 2 : 1;
    }
    if (flags) {
      cudaMemset(d->err, 0, 4);
      return fail(CLV_E_DEVICE, "kernel error flags " + std::to_string(flags));
    }
    return CLV_OK;
  } catch (std::exception& e) {
    return fail(CLV_E_CUDA, e.what());
  }
}

int clv_resolve_srgb(const float* xyz, uint32_t width, uint32_t height, uint8_t* rgb) {
  if (!xyz || !rgb) return fail(CLV_E_INVALID, "null argument");
  try {
    const uint64_t n = (uint64_t)width * height;
    if (n == 0) return CLV_OK;
    double* dfilm = nullptr;
    uint8_t* drgb = nullptr;
    ck(cudaMalloc(&dfilm, n * 3 * sizeof(double)), "cudaMalloc");
    ck(cudaMalloc(&drgb, n * 3), "cudaMalloc");
    std::vector<double> tmp(n * 3);
    for (uint64_t i = 0; i < n * 3; ++i) tmp[i] = (double)xyz[i];
    cudaMemcpy(dfilm, tmp.data(), n * 3 * sizeof(double), cudaMemcpyHostToDevice);
    int rc = clv_resolve_device(dfilm, width, height, 1, nullptr, drgb, nullptr);
    if (rc == CLV_OK) ck(cudaMemcpy(rgb, drgb, n * 3, cudaMemcpyDeviceToHost), "cudaMemcpy D2H");
    cudaFree(dfilm);
    cudaFree(drgb);
    return rc;
  } catch (std::exception& e) {
    return fail(CLV_E_CUDA, e.what());
  }
}

}  // extern "C"

// ------------------------------------------------------ render, no allocation --
//
// Some callers cannot allocate GPU memory when they render: an application
// that reserves the whole device for its own memory pool up front and gives
// libraries a fixed budget, a host that renders from a context where
// cudaMalloc is not allowed (it would synchronise the device or re-enter the
// caller's allocator), or a real-time caller that must never fail with
// out-of-memory in the middle of a frame.  clv_render_device_noalloc serves
// them: the wavefront's path state, shading queues and counters live in the
// file-scope array below instead of memory the library allocates.  The array
// is reserved on every GPU that loads this library and held until the process
// exits, so its size is kept modest: CLV_NOALLOC_SLOTS paths in flight.

#define CLV_NOALLOC_SLOTS 65536u
static constexpr size_t kNoallocHeader = 256;  // WfCounters, padded
static constexpr size_t kNoallocBytes = kNoallocHeader + (size_t)CLV_NOALLOC_SLOTS * clv_device_scene::kWfSlotBytes;
static __device__ __align__(256) unsigned char g_noalloc_scratch[kNoallocBytes];

// Device address of g_noalloc_scratch in the current context, looked up on
// every call (cheap, allocates nothing, and stays right if the context is
// torn down and the module loaded again at another address).
static int noalloc_scratch_address(void** out) {
  void* p = nullptr;
  const cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
  if (e != cudaSuccess || !p)
    return fail(CLV_E_CUDA, std::string("cudaGetSymbolAddress(g_noalloc_scratch): ") + cudaGetErrorString(e));
  *out = p;
  return CLV_OK;
}

__global__ void noalloc_counters_init(WfCounters* C, unsigned long long first_work) {
  C->next_work = first_work;
  C->live = 0u;
  C->queue[0] = C->queue[1] = C->queue[2] = C->queue[3] = 0u;
}

extern "C" int clv_render_device_noalloc(clv_device_scene* d, const clv_render_opts* o, double* film_dev,
                                         void* stream) {
  int rc = check_opts(d, o);
  if (rc) return rc;
  if (!film_dev) return fail(CLV_E_INVALID, "null film");
  if (o->mode != CLV_MODE_PATH_TRACING)
    return fail(CLV_E_INVALID, "the no-allocation render covers the wavefront path tracer only");
  if (o->path_slots > CLV_NOALLOC_SLOTS)
    return fail(CLV_E_INVALID, "path_slots " + std::to_string(o->path_slots) + " exceeds the static scratch of " +
                                   std::to_string(CLV_NOALLOC_SLOTS) + " paths");
  if (d->deep())
    return fail(CLV_E_INVALID, "the no-allocation render takes BVHs of at most " + std::to_string(CLV_STACK) +
                                   " levels (this one has " + std::to_string(d->view.max_depth_tree) + ")");
  void* base = nullptr;
  rc = noalloc_scratch_address(&base);
  if (rc) return rc;
  cudaStream_t st = (cudaStream_t)stream;
  WfParams P;
  P.width = o->width;
  P.height = o->height;
  P.max_depth = o->max_depth;
  P.sample_offset = o->sample_offset;
  P.npix = (uint64_t)o->width * o->height;
  P.total = P.npix * o->samples;
  P.seed = o->seed;
  // the scene's tuned shape (clv_autotune) where it fits the static array
  uint64_t q = o->path_slots ? o->path_slots : std::min<uint64_t>(d->tuned_slots ? d->tuned_slots : CLV_NOALLOC_SLOTS,
                                                                  CLV_NOALLOC_SLOTS);
  q = std::min<uint64_t>(q, P.total);
  q = (q + 127) / 128 * 128;  // at most CLV_NOALLOC_SLOTS, itself a multiple of 128
  // carve counters and path state out of the static array (the layout of clv_device_scene::wavefront_state)
  char* c = static_cast<char*>(base);
  WfCounters* C = reinterpret_cast<WfCounters*>(c);
  char* p = c + kNoallocHeader;
  const size_t n = q;
  WfState W;
  W.o_time = reinterpret_cast<float4*>(p); p += n * 16;
  W.d_lambda = reinterpret_cast<float4*>(p); p += n * 16;
  W.beta = reinterpret_cast<float4*>(p); p += n * 16;
  W.meta = reinterpret_cast<uint4*>(p); p += n * 16;
  W.hit = reinterpret_cast<float4*>(p); p += n * 16;
  W.full = reinterpret_cast<float4*>(p); p += n * 48;
  W.key = reinterpret_cast<uint2*>(p); p += n * 8;
  W.queue = reinterpret_cast<uint32_t*>(p);
  W.Q = (uint32_t)q;
  W.gslot = nullptr;
  W.grec = nullptr;
  W.grec_count = nullptr;
  W.grec_cap = 0;
  W.spill = nullptr;
  W.stack_cap = CLV_STACK;
  const int block = 128;
  const uint32_t grid = (uint32_t)((q + block - 1) / block);
  const uint32_t qgrid =
      std::min<uint32_t>(grid, (uint32_t)sm_count() * (d->tuned_shade ? d->tuned_shade : CLV_SHADE_BLOCKS));
  // the array keeps the previous call's contents: counters are reset here and
  // wf_init rewrites every path slot
  noalloc_counters_init<<<1, 1, 0, st>>>(C, std::min<uint64_t>(q, P.total));
  wf_init<false><<<grid, block, 0, st>>>(d->view, P, W, WfBatch{});
  g_launches += 2;
  const uint32_t level = d->view.compound_level;
  const int batch = 8;
  for (uint64_t it = 0;; it += batch) {
    for (int k = 0; k < batch; ++k) {
      cudaMemsetAsync(&C->live, 0, 5 * sizeof(unsigned int), st);
      switch (level * 2 + (d->view.watertight ? 1 : 0)) {
        case 0: wf_intersect<0, false, false, CLV_WT_OFF><<<grid, block, 0, st>>>(d->view, W, C, d->err, nullptr, WfBatch{}, -1); break;
        case 1: wf_intersect<0, false, false, CLV_WT_ON><<<grid, block, 0, st>>>(d->view, W, C, d->err, nullptr, WfBatch{}, -1); break;
        case 2: wf_intersect<1, false, false, CLV_WT_OFF><<<grid, block, 0, st>>>(d->view, W, C, d->err, nullptr, WfBatch{}, -1); break;
        case 3: wf_intersect<1, false, false, CLV_WT_ON><<<grid, block, 0, st>>>(d->view, W, C, d->err, nullptr, WfBatch{}, -1); break;
        case 4: wf_intersect<2, false, false, CLV_WT_OFF><<<grid, block, 0, st>>>(d->view, W, C, d->err, nullptr, WfBatch{}, -1); break;
        default: wf_intersect<2, false, false, CLV_WT_ON><<<grid, block, 0, st>>>(d->view, W, C, d->err, nullptr, WfBatch{}, -1); break;
      }
      wf_shade_specular<false><<<qgrid, block, 0, st>>>(d->view, P, W, C, d->err, WfBatch{});
      launch_shade_diffuse<false>(d->tuned_diffuse, grid, d->tuned_shade, st, d->view, P, W, C, d->err, WfBatch{});
      wf_finish<false><<<qgrid, block, 0, st>>>(d->view, P, W, C, film_dev, WfBatch{});
    }
    g_launches += 4 * batch;
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return fail(CLV_E_CUDA, std::string("wavefront launch: ") + cudaGetErrorString(e));
    unsigned int live = 0;
    e = cudaMemcpyAsync(&live, &C->live, sizeof live, cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    if (e != cudaSuccess) return fail(CLV_E_CUDA, std::string("wavefront poll: ") + cudaGetErrorString(e));
    if (live == 0) break;
    if (it > (uint64_t)4 * (P.total / q + 1) * (o->max_depth + 2) + 64)
      return fail(CLV_E_DEVICE, "wavefront did not drain");
  }
  return CLV_OK;
}
