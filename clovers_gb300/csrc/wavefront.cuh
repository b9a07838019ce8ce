// Wavefront path tracer: the recursion of clovers-cli/src/trace.rs:21-122
// unrolled over bounces and split into small kernels over structure-of-arrays
// path state in HBM.
//
//   wf_init            fills every path slot with the camera ray of one sample
//                      (work item w -> sample w / npix, pixel w % npix)
//   wf_intersect       closest hit of each live path (BVHNode::hit, bit-exact);
//                      appends the slot to the queue of its material class
//   wf_shade_specular  metal / dielectric / dispersive bounce
//   wf_shade_diffuse   Lambertian / isotropic bounce with MixturePDF light sampling
//   wf_guide_pre/post  guided Lambertian bounce around the guide network (guide.cu)
//   wf_finish          emission or background of paths that ended, deposit of
//                      their spectral powers in the f64 film (draw_cpu.rs:131-142);
//                      each freed slot takes the next work item (one atomic per
//                      block), so slots stay busy without compaction.
//
// The host replays [intersect, shade, finish] bounces in CUDA-graph batches of
// eight until no slot is live; the two shade kernels work on disjoint queues,
// so the specular one runs on a second stream beside the diffuse one.  The
// *_slot functions hold the per-path arithmetic; the same kernels render a
// single scene (BATCH false) or many (BATCH true: scene tables in constant memory).
#pragma once

#include "clv_device.cuh"
#include "guide.cuh"

namespace clvd {

struct WfState {
  uint32_t* queue;   // 4 * Q slot indices, one segment per class
  float4* o_time;    // origin.xyz, time
  float4* d_lambda;  // direction.xyz, wavelength (int bits)
  float4* beta;      // throughput per wavelength (only lights and the background
                     // emit, so a path's power is beta times its final emission)
  uint4* meta;       // pixel, depth, rng counter, flags (1 = live)
  uint2* key;        // rng key
  float4* hit;       // t, ref bits, a, b
  float4* full;      // 3 per slot: p.xyz u | n.xyz v | front, material
  uint32_t Q;
  // guided renders only (null otherwise): per slot the training-record ids of
  // the path's first two guided vertices and its hero throughput before each
  uint4* gslot;
  float4* grec;
  unsigned int* grec_count;
  uint32_t grec_cap;
  // scenes whose BVH is deeper than CLV_STACK levels: traversal stack entries
  // beyond CLV_STACK of slot i at spill[(k - CLV_STACK) * Q + i], stack_cap in all
  float4* spill;
  uint32_t stack_cap;
};

#define WF_Q_FINISH 0  // misses, emitters and paths ended in the shade kernels
// meta.w flag: the path ended in a shade kernel on a surface that emits nothing
// (depth limit or no scatter), so wf_finish has nothing to add for it
#define WF_ENDED_DARK 2u
#define WF_Q_SPEC 1    // metal, dielectric, dispersive
#define WF_Q_DIFF 2    // lambertian, isotropic (isotropic only in guided renders)
#define WF_Q_GUIDE 3   // lambertian in guided renders
struct WfCounters {
  unsigned long long next_work;  // next unassigned work item
  unsigned int live;             // live paths after the last shading pass
  unsigned int queue[4];         // per-class queue lengths of this bounce
};

struct WfParams {
  uint32_t width, height, max_depth, sample_offset;
  uint64_t npix, total;  // total work items = npix * spp
  uint64_t seed;
};

// Several scenes rendered by one wavefront: the work items of scene s are
// [prefix[s], prefix[s+1]); a path slot records its scene in meta.w >> 8.
// The scene views and render parameters of a batch sit in constant memory
// (wf_bscene / wf_bparam, at most CLV_BATCH_MAX scenes), so that the kernels
// read them through the constant cache, as a single-scene kernel reads its
// scene from the kernel parameters; the host writes the tables before the
// batch's launches and holds them until its last launch has finished.
#define CLV_BATCH_MAX 128
__constant__ ClvDeviceScene wf_bscene[CLV_BATCH_MAX];
__constant__ WfParams wf_bparam[CLV_BATCH_MAX];
struct WfBatch {
  const unsigned long long* prefix;  // n + 1 entries
  double* const* films;
  uint32_t n;
  unsigned long long total;
};
__device__ __forceinline__ uint32_t wf_scene_of(const WfBatch& B, unsigned long long w) {
  uint32_t lo = 0, hi = B.n;  // largest s with prefix[s] <= w
  while (hi - lo > 1) {
    const uint32_t mid = (lo + hi) >> 1;
    if (__ldg(B.prefix + mid) <= w) lo = mid;
    else hi = mid;
  }
  return lo;
}

__device__ __forceinline__ void wf_rotate(int hero, int w[4]) {
#pragma unroll
  for (int j = 0; j < 4; ++j) w[j] = 380 + (hero - 380 + j * 100) % 400;
}

// camera ray of work item w (draw_cpu.rs:113-127, camera.rs:103-126)
__device__ __forceinline__ Ray wf_camera_ray(const ClvDeviceScene& S, const WfParams& P, uint64_t w, Rng& rng,
                                             uint32_t& pixel) {
  const uint32_t sample = (uint32_t)(w / P.npix) + P.sample_offset;
  pixel = (uint32_t)(w % P.npix);
  const uint32_t x = pixel % P.width, row = pixel / P.width;
  rng.init(P.seed, pixel, sample);
  const float ox = rng.f32(), oy = rng.f32();
  float lx, ly;
  random_in_unit_disk(rng, lx, ly);
  const float time = rng.f32();
  const int lambda = random_wavelength(rng);
  const uint32_t y = P.height - 1 - row;
  const float pu = ((float)x + ox) / (float)P.width;
  const float pv = ((float)y + oy) / (float)P.height;
  const ClvCamera& C = S.camera;
  lx *= C.lens_radius;
  ly *= C.lens_radius;
  const V off = add(scl(lx, ld3(C.u)), scl(ly, ld3(C.v)));
  const V dir = sub(sub(add(add(ld3(C.llc), scl(pu, ld3(C.horizontal))), scl(pv, ld3(C.vertical))), ld3(C.origin)), off);
  return Ray{add(ld3(C.origin), off), unit(dir), time, lambda};
}

__device__ __forceinline__ void wf_start_path(const ClvDeviceScene& S, const WfParams& P, const WfState& W, uint32_t i,
                                              uint64_t w, uint32_t sid) {
  Rng rng;
  uint32_t pixel;
  const Ray r = wf_camera_ray(S, P, w, rng, pixel);
  W.o_time[i] = make_float4(r.o.x, r.o.y, r.o.z, r.time);
  W.d_lambda[i] = make_float4(r.d.x, r.d.y, r.d.z, __int_as_float(r.lambda));
  W.beta[i] = make_float4(1.0f, 1.0f, 1.0f, 1.0f);
  W.meta[i] = make_uint4(pixel, 0u, rng.counter, 1u | (sid << 8));
  W.key[i] = make_uint2((uint32_t)rng.key, (uint32_t)(rng.key >> 32));
  if (W.gslot) W.gslot[i] = make_uint4(0xFFFFFFFFu, 0xFFFFFFFFu, 0u, 0u);
}

template <bool BATCH>
__global__ void wf_init(ClvDeviceScene S, WfParams P, WfState W, WfBatch B) {
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= W.Q) return;
  if constexpr (BATCH) {
    if ((unsigned long long)i < B.total) {
      const uint32_t sid = wf_scene_of(B, i);
      wf_start_path(wf_bscene[sid], wf_bparam[sid], W, i, i - B.prefix[sid], sid);
      return;
    }
  } else {
    if ((uint64_t)i < P.total) {
      wf_start_path(S, P, W, i, i, 0u);
      return;
    }
  }
  W.meta[i] = make_uint4(0u, 0u, 0u, 0u);
}

// counters (optional): [0] live paths intersected, [1] BVHNode::hit calls, [2] primitive tests
__device__ __forceinline__ void warp_add_counts(unsigned long long* cnt, uint32_t live, uint32_t nodes,
                                                uint32_t prims) {
#pragma unroll
  for (int off = 16; off > 0; off >>= 1) {
    live += __shfl_down_sync(0xFFFFFFFFu, live, off);
    nodes += __shfl_down_sync(0xFFFFFFFFu, nodes, off);
    prims += __shfl_down_sync(0xFFFFFFFFu, prims, off);
  }
  if ((threadIdx.x & 31) == 0) {
    atomicAdd(cnt, (unsigned long long)live);
    atomicAdd(cnt + 1, (unsigned long long)nodes);
    atomicAdd(cnt + 2, (unsigned long long)prims);
  }
}

#ifndef CLV_MINB_SHADE
#define CLV_MINB_SHADE 8  // resident blocks per SM asked of the shading kernels (64 registers)
#endif
// wf_shade_diffuse comes in two variants, its grid scaled to its resident blocks:
// 5 blocks per SM (96 registers, 28 bytes of spills; the default: enclosed box
// 686 against 679 Msamples/s) and 8 (64 registers, 232 bytes of spills; the
// caustic prism 1380 against 1360).  clv_autotune picks one per scene.
#define CLV_MINB_DIFFUSE 5
#define CLV_MINB_DIFFUSE_ALT 8
#ifndef CLV_MINB_GUIDE
#define CLV_MINB_GUIDE CLV_MINB_SHADE  // the same for wf_guide_pre
#endif
#ifndef CLV_MINB_GUIDE_POST
#define CLV_MINB_GUIDE_POST CLV_MINB_SHADE  // the same for wf_guide_post (its grid scales with it)
#endif
// Appends each thread's slot i to queue `cls` (cls < 0: nothing) with one
// atomic per class for the whole block; every thread of the 128-thread block
// calls it.
__device__ __forceinline__ void wf_enqueue_block(const WfState& W, WfCounters* C, int cls, uint32_t i) {
  __shared__ uint32_t cnt[4][4];  // [class][warp]
  __shared__ uint32_t base[4];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  unsigned mine = 0u;
#pragma unroll
  for (int c = 0; c < 4; ++c) {
    const unsigned m = __ballot_sync(0xFFFFFFFFu, cls == c);
    if (lane == 0) cnt[c][warp] = (uint32_t)__popc(m);
    if (cls == c) mine = m;
  }
  __syncthreads();
  if (threadIdx.x < 4) {
    const int c = threadIdx.x;
    const uint32_t tot = cnt[c][0] + cnt[c][1] + cnt[c][2] + cnt[c][3];
    base[c] = tot ? atomicAdd(&C->queue[c], tot) : 0u;
  }
  __syncthreads();
  if (cls >= 0) {
    uint32_t pos = base[cls] + (uint32_t)__popc(mine & ((1u << lane) - 1u));
    for (int w = 0; w < warp; ++w) pos += cnt[cls][w];
    W.queue[(size_t)cls * W.Q + pos] = i;
  }
}
// Appends each thread's slot i to queue `cls` (cls < 0: nothing) with one
// atomic per class for the warp and no block barrier; every lane of the warp
// calls it.  Faster than wf_enqueue_block where traversal lengths within a
// block vary widely (warps that finish early do not wait at the barrier).
__device__ __forceinline__ void wf_enqueue_warp(const WfState& W, WfCounters* C, int cls, uint32_t i) {
  const int lane = threadIdx.x & 31;
#pragma unroll
  for (int c = 0; c < 4; ++c) {
    const unsigned m = __ballot_sync(0xFFFFFFFFu, cls == c);
    if (!m) continue;
    const int leader = __ffs(m) - 1;
    uint32_t base = 0;
    if (lane == leader) base = atomicAdd(&C->queue[c], (uint32_t)__popc(m));
    base = __shfl_sync(0xFFFFFFFFu, base, leader);
    if (cls == c) W.queue[(size_t)c * W.Q + base + __popc(m & ((1u << lane) - 1u))] = i;
  }
}
// Appends the slots of the threads with `want` to queue `cls`, one atomic for
// the block; every thread of the 128-thread block calls it, in every round.
__device__ __forceinline__ void wf_enqueue_block_one(const WfState& W, WfCounters* C, int cls, bool want, uint32_t i) {
  __shared__ uint32_t cnt1[4];
  __shared__ uint32_t base1;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const unsigned m = __ballot_sync(0xFFFFFFFFu, want);
  if (lane == 0) cnt1[warp] = (uint32_t)__popc(m);
  __syncthreads();
  if (threadIdx.x == 0) {
    const uint32_t tot = cnt1[0] + cnt1[1] + cnt1[2] + cnt1[3];
    base1 = tot ? atomicAdd(&C->queue[cls], tot) : 0u;
  }
  __syncthreads();
  if (want) {
    uint32_t pos = base1 + (uint32_t)__popc(m & ((1u << lane) - 1u));
    for (int w = 0; w < warp; ++w) pos += cnt1[w];
    W.queue[(size_t)cls * W.Q + pos] = i;
  }
  __syncthreads();  // cnt1 and base1 are rewritten next round
}
// The live-path count of a shading kernel: one atomic per warp for all its rounds.
__device__ __forceinline__ void wf_add_live(WfCounters* C, uint32_t n) {
  n = __reduce_add_sync(0xFFFFFFFFu, n);
  if ((threadIdx.x & 31) == 0 && n) atomicAdd(&C->live, n);
}

__device__ __forceinline__ int material_class(const ClvDeviceScene& S, uint32_t mat, bool guided) {
  const uint32_t k = S.materials[mat].kind;
  if (k == CLV_MAT_LAMBERTIAN) return guided ? WF_Q_GUIDE : WF_Q_DIFF;
  if (k == CLV_MAT_ISOTROPIC) return WF_Q_DIFF;
  if (k == CLV_MAT_DIFFUSELIGHT || k == CLV_MAT_CONELIGHT) return WF_Q_FINISH;
  return WF_Q_SPEC;
}

// Every lane of the warp calls this (go: the slot holds a live path); returns
// the queue class of the slot's next step, -1 without a path.
template <int CPLX, bool COUNT, int WT, bool DEEP = false>
__device__ __forceinline__ int intersect_slot(const ClvDeviceScene& S, const WfState& W, uint32_t* err, uint32_t i,
                                              const uint4& m, bool go, Counters& c) {
  constexpr bool WARP = CPLX > 0;
  if (!WARP && !go) return -1;
  Ray r{mk(0.0f, 0.0f, 0.0f), mk(0.0f, 0.0f, 1.0f), 0.0f, 0};
  if (go) {
    const float4 a = W.o_time[i], b = W.d_lambda[i];
    r = Ray{mk(a.x, a.y, a.z), mk(b.x, b.y, b.z), a.w, __float_as_int(b.w)};
  }
  Hit h;
  Rec full;
  Rng rng;
  if (CPLX == 2 && go) {  // media draw randomness inside the traversal
    const uint2 k = W.key[i];
    rng.key = (uint64_t)k.x | ((uint64_t)k.y << 32);
    rng.counter = m.z;
  }
  bool any;
  if constexpr (DEEP) {  // generic traversal (CPLX 2) with a spilling stack
    float4 loc[CLV_STACK];
    SpillStack stack{loc, W.spill + i, W.Q, (int)W.stack_cap};
    any = closest_hit_warp<CPLX, WT>(S, r, go, CLV_EPS_ACNE, CLV_FLT_MAX, CPLX == 2 ? &rng : nullptr, h, &full,
                                     COUNT ? &c : nullptr, err, stack);
    if (!go) return -1;
  } else if constexpr (WARP) {
    any = closest_hit_warp<CPLX, WT>(S, r, go, CLV_EPS_ACNE, CLV_FLT_MAX, CPLX == 2 ? &rng : nullptr, h, &full,
                                     COUNT ? &c : nullptr, err);
    if (!go) return -1;
  } else {
    any = closest_hit<CPLX, WT>(S, r, CLV_EPS_ACNE, CLV_FLT_MAX, CPLX == 2 ? &rng : nullptr, h,
                                CPLX ? &full : nullptr, COUNT ? &c : nullptr, err);
  }
  if (CPLX == 2 && rng.counter != m.z) W.meta[i].z = rng.counter;
  int cls = WF_Q_FINISH;
  if (any) {
    const uint32_t kind = CLV_REF_KIND(h.ref), idx = CLV_REF_INDEX(h.ref);
    uint32_t mat;
    if (kind == CLV_REF_TRI) mat = S.tri_mat[idx];
    else if (kind == CLV_REF_QUAD) mat = S.quad_mat[idx];
    else if (kind == CLV_REF_SPHERE) mat = S.sphere_mat[idx];
    else mat = full.mat;
    cls = material_class(S, mat, W.gslot != nullptr);
    if (CPLX && kind == CLV_REF_OBJ) {
      W.full[3 * i] = make_float4(full.p.x, full.p.y, full.p.z, full.u);
      W.full[3 * i + 1] = make_float4(full.n.x, full.n.y, full.n.z, full.v);
      W.full[3 * i + 2] = make_float4(full.front ? 1.0f : 0.0f, __uint_as_float(full.mat), 0.0f, 0.0f);
    }
  }
  W.hit[i] = make_float4(any ? h.t : 0.0f, __uint_as_float(any ? h.ref : CLV_REF_EMPTY), h.a, h.b);
  return cls;
}

// WT: CLV_WT_OFF / CLV_WT_ON for one scene, CLV_WT_SCENE for batches.
// only_level >= 0 (batches): only the slots of scenes at that traversal level,
// so that a batch runs each scene with the variant its objects need.
// DEEP: trees deeper than CLV_STACK levels (CPLX 2 only), stack entries spilled to W.spill.
// WAPP: queue appends per warp instead of per block (primitive-level scenes that
// clv_autotune finds faster so; a separate instantiation, because even an unused
// run-time branch to the warp form slowed the wrapper-chain variant by 11 %).
template <int CPLX, bool COUNT, bool BATCH, int WT, bool DEEP = false, bool WAPP = false>
__global__ void __launch_bounds__(128, CPLX == 1 ? CLV_MINB_CHAIN : CPLX == 2 ? CLV_MINB_MEDIUM : CLV_MINB) wf_intersect(ClvDeviceScene S, WfState W, WfCounters* C, uint32_t* err,
                                                              unsigned long long* cnt, WfBatch B, int only_level) {
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  Counters c{0u, 0u};
  uint32_t live = 0;
  const uint4 m = i < W.Q ? W.meta[i] : make_uint4(0u, 0u, 0u, 0u);
  bool go = (m.w & 1u) != 0u;
  if (BATCH && go && only_level >= 0) go = wf_bscene[m.w >> 8].compound_level == (uint32_t)only_level;
  live = go ? 1u : 0u;
  int cls;
  if constexpr (BATCH) cls = intersect_slot<CPLX, COUNT, WT, DEEP>(wf_bscene[go ? m.w >> 8 : 0u], W, err, i, m, go, c);
  else cls = intersect_slot<CPLX, COUNT, WT, DEEP>(S, W, err, i, m, go, c);
  if constexpr (WAPP) wf_enqueue_warp(W, C, cls, i);
  else wf_enqueue_block(W, C, cls, i);
  if (COUNT) warp_add_counts(cnt, live, c.nodes, c.prims);
}

__device__ __forceinline__ bool wf_is_normal_pos(float v) {
  const float a = fabsf(v);
  return v > 0.0f && a >= 1.17549435e-38f && a <= 3.40282347e+38f;
}

struct WfPath {
  Ray ray;
  float beta[4];
  uint4 meta;
  Rng rng;
};
__device__ __forceinline__ void wf_load(const WfState& W, uint32_t i, WfPath& P) {
  const float4 a = W.o_time[i], b = W.d_lambda[i];
  P.ray = Ray{mk(a.x, a.y, a.z), mk(b.x, b.y, b.z), a.w, __float_as_int(b.w)};
  const float4 bv = W.beta[i];
  P.beta[0] = bv.x; P.beta[1] = bv.y; P.beta[2] = bv.z; P.beta[3] = bv.w;
  P.meta = W.meta[i];
  const uint2 k = W.key[i];
  P.rng.key = (uint64_t)k.x | ((uint64_t)k.y << 32);
  P.rng.counter = P.meta.z;
}
__device__ __forceinline__ void wf_hit_record(const ClvDeviceScene& S, const WfState& W, uint32_t i, const Ray& ray,
                                              Hit& h, Rec& rec) {
  const float4 hv = W.hit[i];
  h.t = hv.x;
  h.ref = __float_as_uint(hv.y);
  h.a = hv.z;
  h.b = hv.w;
  Rec full;
  if (h.ref != CLV_REF_EMPTY && CLV_REF_KIND(h.ref) == CLV_REF_OBJ) {
    const float4 f0 = W.full[3 * i], f1 = W.full[3 * i + 1], f2 = W.full[3 * i + 2];
    full.t = h.t;
    full.p = mk(f0.x, f0.y, f0.z);
    full.u = f0.w;
    full.n = mk(f1.x, f1.y, f1.z);
    full.v = f1.w;
    full.front = f2.x != 0.0f;
    full.mat = __float_as_uint(f2.y);
  }
  if (h.ref != CLV_REF_EMPTY) hit_record(S, ray, h, full, rec);
}
// attenuation of trace.rs:61-70: hero only on wavelength-dependent materials
__device__ __forceinline__ void wf_attenuation(const ClvDeviceScene& S, const ClvMaterial& m, const Ray& ray,
                                               const Rec& rec, float atten[4]) {
  const int hero = ray.lambda;
  if (m.wavelength_dependent) {
    atten[0] = mat_color(S, m, ray, hero, rec);
    atten[1] = atten[2] = atten[3] = 0.0f;
  } else {
    int waves[4];
    wf_rotate(hero, waves);
#pragma unroll
    for (int j = 0; j < 4; ++j) atten[j] = mat_color(S, m, ray, waves[j], rec);
  }
}
// continue the path with `nd` (depth + 1) or end it at the depth limit
__device__ __forceinline__ bool wf_advance(const WfParams& P, const WfState& W, WfCounters* C, uint32_t i, WfPath& p,
                                           V origin, V nd) {
  const uint32_t depth = p.meta.y + 1;
  if (depth > P.max_depth) {  // trace at depth > max_depth returns 0
    W.meta[i] = make_uint4(p.meta.x, p.meta.y, p.rng.counter, p.meta.w | WF_ENDED_DARK);
    return false;
  }
  W.o_time[i] = make_float4(origin.x, origin.y, origin.z, p.ray.time);
  W.d_lambda[i] = make_float4(nd.x, nd.y, nd.z, __int_as_float(p.ray.lambda));
  W.beta[i] = make_float4(p.beta[0], p.beta[1], p.beta[2], p.beta[3]);
  W.meta[i] = make_uint4(p.meta.x, depth, p.rng.counter, (p.meta.w & ~0xFFu) | 1u);
  return true;
}

// Specular bounce: Metal (metal.rs:27-51), Dielectric / Dispersive (dielectric.rs:37-81, dispersive.rs:58-123)
__device__ __forceinline__ bool specular_slot(const ClvDeviceScene& S, const WfParams& P, const WfState& W,
                                              WfCounters* C, uint32_t i) {
  WfPath p;
  wf_load(W, i, p);
  Hit h;
  Rec rec;
  wf_hit_record(S, W, i, p.ray, h, rec);
  const ClvMaterial& m = S.materials[rec.mat];
  V nd;
  if (m.kind == CLV_MAT_METAL) {
    nd = unit(add(reflect(p.ray.d, rec.n), scl(m.fuzz, random_unit_vector(p.rng))));
  } else {
    const float ri = m.kind == CLV_MAT_DIELECTRIC ? m.refractive_index : dispersive_index(m, p.ray.lambda);
    const float ratio = rec.front ? 1.0f / ri : ri;
    const float ct = fminf(-dot(p.ray.d, rec.n), 1.0f);
    const float st = sqrtf(1.0f - ct * ct);
    if (ratio * st > 1.0f) {
      nd = reflect(p.ray.d, rec.n);
    } else {
      const float rp = schlick(ct, ratio);
      nd = p.rng.f32() < rp ? reflect(p.ray.d, rec.n) : refract(p.ray.d, rec.n, ratio);
    }
  }
  float atten[4];
  wf_attenuation(S, m, p.ray, rec, atten);
#pragma unroll
  for (int j = 0; j < 4; ++j) p.beta[j] = p.beta[j] * atten[j];
  return wf_advance(P, W, C, i, p, rec.p, nd);
}

template <bool BATCH>
__global__ void __launch_bounds__(128, CLV_MINB_SHADE) wf_shade_specular(ClvDeviceScene S, WfParams P, WfState W, WfCounters* C,
                                                         uint32_t* err, WfBatch B) {
  const uint32_t n = C->queue[WF_Q_SPEC];
  const uint32_t stride = gridDim.x * blockDim.x;
  const uint32_t first = blockIdx.x * blockDim.x + threadIdx.x;
  const uint32_t rounds = (n + stride - 1) / stride;
  uint32_t nlive = 0;
  for (uint32_t r = 0; r < rounds; ++r) {
    const uint32_t q = first + r * stride;
    bool live = false;
    uint32_t i = 0;
    if (q < n) {
      i = W.queue[(size_t)WF_Q_SPEC * W.Q + q];
      if constexpr (BATCH) {
        const uint32_t sid = W.meta[i].w >> 8;
        live = specular_slot(wf_bscene[sid], wf_bparam[sid], W, C, i);
      } else {
        live = specular_slot(S, P, W, C, i);
      }
    }
    wf_enqueue_block_one(W, C, WF_Q_FINISH, q < n && !live, i);
    nlive += live ? 1u : 0u;
  }
  wf_add_live(C, nlive);
}

// Diffuse bounce: MixturePDF(HitablePDF(priority tree), Cosine/SpherePDF), pdf.rs:122-140, trace.rs:80-119
__device__ __forceinline__ bool diffuse_slot(const ClvDeviceScene& S, const WfParams& P, const WfState& W,
                                             WfCounters* C, uint32_t* err, uint32_t i) {
  WfPath p;
  wf_load(W, i, p);
  Hit h;
  Rec rec;
  wf_hit_record(S, W, i, p.ray, h, rec);
  const ClvMaterial& m = S.materials[rec.mat];
  const bool lamb = m.kind == CLV_MAT_LAMBERTIAN;
  V gen;
  if (p.rng.boolean()) {
    gen = mis_random(S, rec.p, p.rng);
  } else if (lamb) {  // ONB::build_from_w(normal).local(random_cosine_direction)
    const V w = rec.n;
    const V a = fabsf(w.x) > 0.9f ? unit(mk(0.0f, 1.0f, 0.0f)) : unit(mk(1.0f, 0.0f, 0.0f));
    const V vv = unit(cross(w, a));
    const V uu = unit(cross(w, vv));
    const V c = random_cosine_direction(p.rng);
    gen = unit(add(add(scl(c.x, uu), scl(c.y, vv)), scl(c.z, w)));
  } else {
    gen = random_unit_vector(p.rng);
  }
  const V nd = unit(gen);
  const float light_v = mis_pdf(S, rec.p, nd, p.ray.lambda, p.ray.time, err);
  float bsdf_v;
  if (lamb) {
    const float cosine = dot(unit(nd), rec.n);
    bsdf_v = cosine <= 0.0f ? 0.0f : cosine / CLV_PI;
  } else {
    bsdf_v = 1.0f / (4.0f * CLV_PI);
  }
  const float mis = 0.5f * light_v + 0.5f * bsdf_v;
  float spdf;
  bool scatter = true;
  if (lamb) {  // Lambertian::scattering_pdf: None below the surface -> emitted (0) only
    const float cs = dot(rec.n, unit(nd));
    scatter = !(cs < 0.0f);
    spdf = cs / CLV_PI;
  } else {
    spdf = 1.0f / (4.0f * CLV_PI);
  }
  if (!scatter) {
    W.meta[i] = make_uint4(p.meta.x, p.meta.y, p.rng.counter, p.meta.w | WF_ENDED_DARK);
    return false;
  }
  float atten[4];
  wf_attenuation(S, m, p.ray, rec, atten);
#pragma unroll
  for (int j = 0; j < 4; ++j) p.beta[j] = p.beta[j] * (atten[j] * spdf / mis);
  return wf_advance(P, W, C, i, p, rec.p, nd);
}

template <bool BATCH, int MINB>
__global__ void __launch_bounds__(128, MINB) wf_shade_diffuse(ClvDeviceScene S, WfParams P, WfState W, WfCounters* C,
                                                        uint32_t* err, WfBatch B) {
  const uint32_t n = C->queue[WF_Q_DIFF];
  const uint32_t stride = gridDim.x * blockDim.x;
  const uint32_t first = blockIdx.x * blockDim.x + threadIdx.x;
  const uint32_t rounds = (n + stride - 1) / stride;
  uint32_t nlive = 0;
  for (uint32_t r = 0; r < rounds; ++r) {
    const uint32_t q = first + r * stride;
    bool live = false;
    uint32_t i = 0;
    if (q < n) {
      i = W.queue[(size_t)WF_Q_DIFF * W.Q + q];
      if constexpr (BATCH) {
        const uint32_t sid = W.meta[i].w >> 8;
        live = diffuse_slot(wf_bscene[sid], wf_bparam[sid], W, C, err, i);
      } else {
        live = diffuse_slot(S, P, W, C, err, i);
      }
    }
    wf_enqueue_block_one(W, C, WF_Q_FINISH, q < n && !live, i);
    nlive += live ? 1u : 0u;
  }
  wf_add_live(C, nlive);
}

// ---- guided Lambertian bounces: pre -> guide network (guide.cu) -> post ----
// pre: the hit record goes to the slot's record area (W.full) and a coin picks
// the strategy; bounces that use the reference's MixturePDF (probability
// 1 - alpha) draw their direction here, exactly as diffuse_slot does.
// W.hit then holds {direction, 0} or {-, 1} (guide to sample); the hit's t and
// reference move to W.full[3i+2].zw so a path that ends in guide_post can hand
// wf_finish its hit again.
__device__ __forceinline__ void guide_pre_slot(const ClvDeviceScene& S, const WfState& W, float alpha, uint32_t i) {
  WfPath p;
  wf_load(W, i, p);
  Hit h;
  Rec rec;
  wf_hit_record(S, W, i, p.ray, h, rec);
  W.full[3 * i] = make_float4(rec.p.x, rec.p.y, rec.p.z, rec.u);
  W.full[3 * i + 1] = make_float4(rec.n.x, rec.n.y, rec.n.z, rec.v);
  W.full[3 * i + 2] = make_float4(rec.front ? 1.0f : 0.0f, __uint_as_float(rec.mat), h.t, __uint_as_float(h.ref));
  float4 out = make_float4(0.0f, 0.0f, 0.0f, 1.0f);
  if (!(p.rng.f32() < alpha)) {
    V gen;
    if (p.rng.boolean()) {
      gen = mis_random(S, rec.p, p.rng);
    } else {
      const V w = rec.n;
      const V a = fabsf(w.x) > 0.9f ? unit(mk(0.0f, 1.0f, 0.0f)) : unit(mk(1.0f, 0.0f, 0.0f));
      const V vv = unit(cross(w, a));
      const V uu = unit(cross(w, vv));
      const V c = random_cosine_direction(p.rng);
      gen = unit(add(add(scl(c.x, uu), scl(c.y, vv)), scl(c.z, w)));
    }
    const V nd = unit(gen);
    out = make_float4(nd.x, nd.y, nd.z, 0.0f);
  }
  W.hit[i] = out;
  W.meta[i].z = p.rng.counter;
}

template <bool BATCH>
__global__ void __launch_bounds__(128, CLV_MINB_GUIDE) wf_guide_pre(ClvDeviceScene S, WfState W, WfCounters* C, float alpha,
                                                    WfBatch B) {
  const uint32_t n = C->queue[WF_Q_GUIDE];
  const uint32_t stride = gridDim.x * blockDim.x;
  for (uint32_t q = blockIdx.x * blockDim.x + threadIdx.x; q < n; q += stride) {
    const uint32_t i = W.queue[(size_t)WF_Q_GUIDE * W.Q + q];
    if constexpr (BATCH) guide_pre_slot(wf_bscene[W.meta[i].w >> 8], W, alpha, i);
    else guide_pre_slot(S, W, alpha, i);
  }
}

// post: W.hit = {direction, guide density}.  One-sample MIS over the guide
// (alpha) and the reference's MixturePDF (1 - alpha): the bounce is weighted
// by attenuation * scattering_pdf / (alpha q + (1 - alpha) p_mixture).  The
// first two guided vertices of a path leave a training record.
__device__ __forceinline__ bool guide_post_slot(const ClvDeviceScene& S, const WfParams& P, const WfState& W,
                                                WfCounters* C, uint32_t* err, const GuideDev& G, uint32_t i) {
  WfPath p;
  wf_load(W, i, p);
  const float4 f0 = W.full[3 * i], f1 = W.full[3 * i + 1], f2 = W.full[3 * i + 2];
  Rec rec;
  rec.t = 0.0f;
  rec.p = mk(f0.x, f0.y, f0.z);
  rec.u = f0.w;
  rec.n = mk(f1.x, f1.y, f1.z);
  rec.v = f1.w;
  rec.front = f2.x != 0.0f;
  rec.mat = __float_as_uint(f2.y);
  const float4 hv = W.hit[i];
  const V nd = mk(hv.x, hv.y, hv.z);
  const float q = G.alpha > 0.0f ? hv.w : 0.0f;
  const float light_v = mis_pdf(S, rec.p, nd, p.ray.lambda, p.ray.time, err);
  const float cosine = dot(unit(nd), rec.n);
  const float bsdf_v = cosine <= 0.0f ? 0.0f : cosine / CLV_PI;
  const float pdf = G.alpha * q + (1.0f - G.alpha) * (0.5f * light_v + 0.5f * bsdf_v);
  const float cs = dot(rec.n, unit(nd));
  // a path ending here goes to wf_finish, which reads its hit (a Lambertian
  // surface: no emission) from W.hit
  if (cs < 0.0f || p.meta.y + 1 > P.max_depth) W.hit[i] = make_float4(f2.z, f2.w, 0.0f, 0.0f);
  // training record of this vertex (warp-aggregated slot reservation)
  uint4 gs = W.gslot[i];
  const bool want = gs.y == 0xFFFFFFFFu && !(cs < 0.0f);
  const unsigned act = __activemask();
  const unsigned wm = __ballot_sync(act, want);
  if (wm) {
    const int lane = threadIdx.x & 31, leader = __ffs(wm) - 1;
    unsigned base = 0;
    if (lane == leader) base = atomicAdd(W.grec_count, (unsigned)__popc(wm));
    base = __shfl_sync(act, base, leader);
    if (want) {
      const unsigned r = base + __popc(wm & ((1u << lane) - 1u));
      if (r < W.grec_cap) {
        const float4 dl = W.d_lambda[i];
        float4* out = W.grec + GD_REC_F4 * (size_t)r;
        float lo[3], inv[3];
        gd_box(G, p.meta.w, lo, inv);
        out[0] = make_float4(fminf(1.0f, fmaxf(0.0f, (rec.p.x - lo[0]) * inv[0])),
                             fminf(1.0f, fmaxf(0.0f, (rec.p.y - lo[1]) * inv[1])),
                             fminf(1.0f, fmaxf(0.0f, (rec.p.z - lo[2]) * inv[2])),
                             fminf(1.0f, fmaxf(0.0f, 0.5f - 0.5f * dl.x)));
        out[1] = make_float4(fminf(1.0f, fmaxf(0.0f, 0.5f - 0.5f * dl.y)),
                             fminf(1.0f, fmaxf(0.0f, 0.5f - 0.5f * dl.z)),
                             ((float)__float_as_int(dl.w) - 380.0f) * 0.0025f, 0.0f);
        out[2] = make_float4(nd.x, nd.y, nd.z, 0.0f);
        if (gs.x == 0xFFFFFFFFu) {
          gs.x = r;
          gs.z = __float_as_uint(p.beta[0]);
        } else {
          gs.y = r;
          gs.w = __float_as_uint(p.beta[0]);
        }
        W.gslot[i] = gs;
      }
    }
  }
  if (cs < 0.0f) {  // Lambertian::scattering_pdf is None below the surface
    W.meta[i].w = p.meta.w | WF_ENDED_DARK;
    return false;
  }
  const float spdf = cs / CLV_PI;
  const ClvMaterial& m = S.materials[rec.mat];
  float atten[4];
  wf_attenuation(S, m, p.ray, rec, atten);
#pragma unroll
  for (int j = 0; j < 4; ++j) p.beta[j] = p.beta[j] * (atten[j] * spdf / pdf);
  return wf_advance(P, W, C, i, p, rec.p, nd);
}

template <bool BATCH>
__global__ void __launch_bounds__(128, CLV_MINB_GUIDE_POST) wf_guide_post(ClvDeviceScene S, WfParams P, WfState W, WfCounters* C,
                                                     uint32_t* err, GuideDev G, WfBatch B) {
  const uint32_t n = C->queue[WF_Q_GUIDE];
  const uint32_t stride = gridDim.x * blockDim.x;
  const uint32_t first = blockIdx.x * blockDim.x + threadIdx.x;
  const uint32_t rounds = (n + stride - 1) / stride;
  uint32_t nlive = 0;
  for (uint32_t r = 0; r < rounds; ++r) {
    const uint32_t q = first + r * stride;
    bool live = false;
    const uint32_t i = q < n ? W.queue[(size_t)WF_Q_GUIDE * W.Q + q] : 0u;
    if (q < n) {
      if constexpr (BATCH) {
        const uint32_t sid = W.meta[i].w >> 8;
        live = guide_post_slot(wf_bscene[sid], wf_bparam[sid], W, C, err, G, i);
      } else {
        live = guide_post_slot(S, P, W, C, err, G, i);
      }
    }
    wf_enqueue_block_one(W, C, WF_Q_FINISH, q < n && !live, i);
    nlive += live ? 1u : 0u;
  }
  wf_add_live(C, nlive);
}

// film rule of draw_cpu.rs:131-142, deposited as f64 sums
__device__ __forceinline__ void film_deposit(const ClvDeviceScene& S, double* film, uint32_t pixel, int hero,
                                             const float p[4]) {
  int waves[4];
  wf_rotate(hero, waves);
  double a0 = 0.0, a1 = 0.0, a2 = 0.0;
  if (p[1] == 0.0f && p[2] == 0.0f && p[3] == 0.0f) {
    const float* c = S.cmf + 3 * (waves[0] - 380);
    a0 = (double)(__ldg(c) * p[0]);
    a1 = (double)(__ldg(c + 1) * p[0]);
    a2 = (double)(__ldg(c + 2) * p[0]);
  } else {
#pragma unroll
    for (int i = 0; i < 4; ++i) {
      if (wf_is_normal_pos(p[i])) {
        const float* c = S.cmf + 3 * (waves[i] - 380);
        a0 += (double)(__ldg(c) * p[i] / 4.0f);
        a1 += (double)(__ldg(c + 1) * p[i] / 4.0f);
        a2 += (double)(__ldg(c + 2) * p[i] / 4.0f);
      }
    }
  }
  double* f = film + 3 * (size_t)pixel;
  if (a0 != 0.0) atomicAdd(f, a0);
  if (a1 != 0.0) atomicAdd(f + 1, a1);
  if (a2 != 0.0) atomicAdd(f + 2, a2);
}

// Background on a miss (trace.rs:42-48) or emission of a light (trace.rs:51-58), then the film deposit.
__device__ __forceinline__ void finish_slot(const ClvDeviceScene& S, const WfState& W, double* film, uint32_t i) {
  if (W.meta[i].w & WF_ENDED_DARK) {  // ended on a surface that emits nothing: skip its hit record
    if (W.gslot) {  // the path's recorded vertices carry zero radiance
      const uint4 gs = W.gslot[i];
      if (gs.x != 0xFFFFFFFFu) reinterpret_cast<float*>(W.grec + GD_REC_F4 * (size_t)gs.x + 2)[3] = 0.0f;
      if (gs.y != 0xFFFFFFFFu) reinterpret_cast<float*>(W.grec + GD_REC_F4 * (size_t)gs.y + 2)[3] = 0.0f;
    }
    return;
  }
  const float4 a = W.o_time[i], b = W.d_lambda[i];
  const Ray ray{mk(a.x, a.y, a.z), mk(b.x, b.y, b.z), a.w, __float_as_int(b.w)};
  const float4 bv = W.beta[i];
  const float beta[4] = {bv.x, bv.y, bv.z, bv.w};
  float L[4] = {0.0f, 0.0f, 0.0f, 0.0f};
  int waves[4];
  wf_rotate(ray.lambda, waves);
  Hit h;
  Rec rec;
  wf_hit_record(S, W, i, ray, h, rec);
  if (h.ref == CLV_REF_EMPTY) {
#pragma unroll
    for (int j = 0; j < 4; ++j) L[j] += beta[j] * spd_get(S, S.background_spd, waves[j]);
  } else {
    const ClvMaterial& m = S.materials[rec.mat];
    if (m.kind == CLV_MAT_DIFFUSELIGHT || m.kind == CLV_MAT_CONELIGHT) {
#pragma unroll
      for (int j = 0; j < 4; ++j) L[j] += beta[j] * mat_emit(S, m, ray, waves[j], rec);
    }
    // (paths that the shade kernels ended never get here: WF_ENDED_DARK above)
  }
  film_deposit(S, film, W.meta[i].x, ray.lambda, L);
  if (W.gslot) {  // training weights: hero power of the path / hero throughput before each recorded vertex
    const uint4 gs = W.gslot[i];
    if (gs.x != 0xFFFFFFFFu) {
      const float b = __uint_as_float(gs.z);
      reinterpret_cast<float*>(W.grec + GD_REC_F4 * (size_t)gs.x + 2)[3] = b > 0.0f ? L[0] / b : 0.0f;
    }
    if (gs.y != 0xFFFFFFFFu) {
      const float b = __uint_as_float(gs.w);
      reinterpret_cast<float*>(W.grec + GD_REC_F4 * (size_t)gs.y + 2)[3] = b > 0.0f ? L[0] / b : 0.0f;
    }
  }
}

// Ends paths, then each freed slot takes the next work item (one atomic per block and round).
template <bool BATCH>
__global__ void __launch_bounds__(128, CLV_MINB_SHADE) wf_finish(ClvDeviceScene S, WfParams P, WfState W, WfCounters* C,
                                                 double* __restrict__ film, WfBatch B) {
  const uint32_t n = C->queue[WF_Q_FINISH];
  const uint32_t stride = gridDim.x * blockDim.x;
  const uint32_t first = blockIdx.x * blockDim.x + threadIdx.x;
  const uint32_t rounds = (n + stride - 1) / stride;
  uint32_t nlive = 0;
  for (uint32_t r = 0; r < rounds; ++r) {
    const uint32_t q = first + r * stride;
    bool need = false;
    uint32_t i = 0;
    if (q < n) {
      i = W.queue[(size_t)WF_Q_FINISH * W.Q + q];
      if constexpr (BATCH) {
        const uint32_t sid = W.meta[i].w >> 8;
        finish_slot(wf_bscene[sid], W, B.films[sid], i);
      } else {
        finish_slot(S, W, film, i);
      }
      need = true;
    }
    const unsigned mask = __ballot_sync(0xFFFFFFFFu, need);
    bool live = false;
    const int lane = threadIdx.x & 31;
    unsigned long long base = 0;
    {  // one reservation of work items for the block
      __shared__ uint32_t wcnt[4];
      __shared__ unsigned long long wbase;
      const int warp = threadIdx.x >> 5;
      if (lane == 0) wcnt[warp] = (uint32_t)__popc(mask);
      __syncthreads();
      uint32_t before = 0, total = 0;
#pragma unroll
      for (int k = 0; k < 4; ++k) {
        before += k < warp ? wcnt[k] : 0u;
        total += wcnt[k];
      }
      if (threadIdx.x == 0 && total) wbase = atomicAdd(&C->next_work, (unsigned long long)total);
      __syncthreads();
      if (total) base = wbase + before;
      __syncthreads();  // wcnt and wbase are rewritten next round
    }
    if (mask) {
      if (need) {
        const uint64_t w = base + __popc(mask & ((1u << lane) - 1u));
        if constexpr (BATCH) {
          if (w < B.total) {
            const uint32_t sid = wf_scene_of(B, w);
            wf_start_path(wf_bscene[sid], wf_bparam[sid], W, i, w - B.prefix[sid], sid);
            live = true;
          } else {
            W.meta[i].w = 0u;
          }
        } else {
          if (w < P.total) {
            wf_start_path(S, P, W, i, w, 0u);
            live = true;
          } else {
            W.meta[i].w = 0u;
          }
        }
      }
    }
    nlive += live ? 1u : 0u;
  }
  wf_add_live(C, nlive);
}

}  // namespace clvd
