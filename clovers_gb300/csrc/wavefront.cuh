// Wavefront path tracer: the recursion of clovers-cli/src/trace.rs:21-122
// unrolled over bounces and split into small kernels over structure-of-arrays
// path state in HBM.
//
//   wf_init       fills every path slot with the camera ray of one sample
//                 (work item w -> sample w / npix, pixel w % npix)
//   wf_intersect  closest hit of each live path (BVHNode::hit, bit-exact)
//   wf_shade      one bounce: emission, scatter, MixturePDF light sampling,
//                 throughput update; a finished path deposits its spectral
//                 powers in the f64 film (draw_cpu.rs:131-142) and its slot
//                 takes the next work item (warp-aggregated atomic fetch), so
//                 slots stay busy without compaction.
//
// The host runs [intersect, shade] in CUDA-graph batches until no slot is live.
#pragma once

#include "clv_device.cuh"

namespace clvd {

struct WfState {
  float4* o_time;    // origin.xyz, time
  float4* d_lambda;  // direction.xyz, wavelength (int bits)
  float4* beta;      // throughput per wavelength
  float4* L;         // accumulated spectral power per wavelength
  uint4* meta;       // pixel, depth, rng counter, flags (1 = live)
  uint2* key;        // rng key
  float4* hit;       // t, ref bits, a, b
  float4* full;      // 3 per slot: p.xyz u | n.xyz v | front, material
  uint32_t Q;
};

struct WfCounters {
  unsigned long long next_work;  // next unassigned work item
  unsigned int live;             // live paths after the last shade pass
  unsigned int pad;
};

struct WfParams {
  uint32_t width, height, max_depth, sample_offset;
  uint64_t npix, total;  // total work items = npix * spp
  uint64_t seed;
};

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
                                              uint64_t w) {
  Rng rng;
  uint32_t pixel;
  const Ray r = wf_camera_ray(S, P, w, rng, pixel);
  W.o_time[i] = make_float4(r.o.x, r.o.y, r.o.z, r.time);
  W.d_lambda[i] = make_float4(r.d.x, r.d.y, r.d.z, __int_as_float(r.lambda));
  W.beta[i] = make_float4(1.0f, 1.0f, 1.0f, 1.0f);
  W.L[i] = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
  W.meta[i] = make_uint4(pixel, 0u, rng.counter, 1u);
  W.key[i] = make_uint2((uint32_t)rng.key, (uint32_t)(rng.key >> 32));
}

__global__ void wf_init(ClvDeviceScene S, WfParams P, WfState W) {
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= W.Q) return;
  if ((uint64_t)i < P.total) {
    wf_start_path(S, P, W, i, i);
  } else {
    W.meta[i] = make_uint4(0u, 0u, 0u, 0u);
  }
}

template <bool COMPLEX>
__global__ void __launch_bounds__(128) wf_intersect(ClvDeviceScene S, WfState W, uint32_t* err) {
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= W.Q) return;
  const uint4 m = W.meta[i];
  if (!(m.w & 1u)) return;
  const float4 a = W.o_time[i], b = W.d_lambda[i];
  const Ray r{mk(a.x, a.y, a.z), mk(b.x, b.y, b.z), a.w, __float_as_int(b.w)};
  Hit h;
  if (COMPLEX) {
    Rng rng;
    const uint2 k = W.key[i];
    rng.key = (uint64_t)k.x | ((uint64_t)k.y << 32);
    rng.counter = m.z;
    Rec full;
    const bool any = closest_hit<true>(S, r, CLV_EPS_ACNE, CLV_FLT_MAX, &rng, h, &full, nullptr, err);
    if (rng.counter != m.z) W.meta[i].z = rng.counter;  // media drew randomness
    if (any && CLV_REF_KIND(h.ref) == CLV_REF_OBJ) {
      W.full[3 * i] = make_float4(full.p.x, full.p.y, full.p.z, full.u);
      W.full[3 * i + 1] = make_float4(full.n.x, full.n.y, full.n.z, full.v);
      W.full[3 * i + 2] = make_float4(full.front ? 1.0f : 0.0f, __uint_as_float(full.mat), 0.0f, 0.0f);
    }
    W.hit[i] = make_float4(any ? h.t : 0.0f, __uint_as_float(any ? h.ref : CLV_REF_EMPTY), h.a, h.b);
  } else {
    const bool any = closest_hit<false>(S, r, CLV_EPS_ACNE, CLV_FLT_MAX, nullptr, h, nullptr, nullptr, err);
    W.hit[i] = make_float4(any ? h.t : 0.0f, __uint_as_float(any ? h.ref : CLV_REF_EMPTY), h.a, h.b);
  }
}

__device__ __forceinline__ bool wf_is_normal_pos(float v) {
  const float a = fabsf(v);
  return v > 0.0f && a >= 1.17549435e-38f && a <= 3.40282347e+38f;
}

// One bounce of trace().  Returns false when the path ends (its L is final).
__device__ __forceinline__ bool shade_bounce(const ClvDeviceScene& S, Ray& ray, float beta[4], float L[4],
                                             const Hit& h, const Rec& full, Rng& rng, uint32_t* err) {
  const int hero = ray.lambda;
  int waves[4];
  wf_rotate(hero, waves);
  if (h.ref == CLV_REF_EMPTY) {  // background (trace.rs:42-48)
#pragma unroll
    for (int i = 0; i < 4; ++i) L[i] += beta[i] * spd_get(S, S.background_spd, waves[i]);
    return false;
  }
  Rec rec;
  hit_record(S, ray, h, full, rec);
  const ClvMaterial& m = S.materials[rec.mat];
  const uint32_t kind = m.kind;
  if (kind == CLV_MAT_DIFFUSELIGHT || kind == CLV_MAT_CONELIGHT) {  // no scatter: emitted only
#pragma unroll
    for (int i = 0; i < 4; ++i) L[i] += beta[i] * mat_emit(S, m, ray, waves[i], rec);
    return false;
  }
  // the other kinds emit 0 (MaterialTrait::emit default)
  V nd;
  bool specular = true;
  float spdf = 0.0f, mis = 1.0f;
  if (kind == CLV_MAT_METAL) {  // metal.rs:27-51
    const V refl = reflect(ray.d, rec.n);
    nd = unit(add(refl, scl(m.fuzz, random_unit_vector(rng))));
  } else if (kind == CLV_MAT_DIELECTRIC || kind == CLV_MAT_DISPERSIVE) {  // dielectric.rs, dispersive.rs
    const float ri = kind == CLV_MAT_DIELECTRIC ? m.refractive_index : dispersive_index(m, ray.lambda);
    const float ratio = rec.front ? 1.0f / ri : ri;
    const float ct = fminf(-dot(ray.d, rec.n), 1.0f);
    const float st = sqrtf(1.0f - ct * ct);
    if (ratio * st > 1.0f) {
      nd = reflect(ray.d, rec.n);
    } else {
      const float rp = schlick(ct, ratio);
      nd = rng.f32() < rp ? reflect(ray.d, rec.n) : refract(ray.d, rec.n, ratio);
    }
  } else {  // Lambertian (CosinePDF) / Isotropic (SpherePDF) mixed 50/50 with the light tree (pdf.rs:122-140)
    specular = false;
    const bool lamb = kind == CLV_MAT_LAMBERTIAN;
    V gen;
    if (rng.boolean()) {
      gen = mis_random(S, rec.p, rng);
    } else if (lamb) {  // ONB::build_from_w(normal).local(random_cosine_direction)
      const V w = rec.n;
      const V a = fabsf(w.x) > 0.9f ? unit(mk(0.0f, 1.0f, 0.0f)) : unit(mk(1.0f, 0.0f, 0.0f));
      const V vv = unit(cross(w, a));
      const V uu = unit(cross(w, vv));
      const V c = random_cosine_direction(rng);
      gen = unit(add(add(scl(c.x, uu), scl(c.y, vv)), scl(c.z, w)));
    } else {
      gen = random_unit_vector(rng);
    }
    nd = unit(gen);
    const float light_v = mis_pdf(S, rec.p, nd, hero, ray.time, err);
    float bsdf_v;
    if (lamb) {
      const float cosine = dot(unit(nd), rec.n);
      bsdf_v = cosine <= 0.0f ? 0.0f : cosine / CLV_PI;
    } else {
      bsdf_v = 1.0f / (4.0f * CLV_PI);
    }
    mis = 0.5f * light_v + 0.5f * bsdf_v;
    if (lamb) {  // Lambertian::scattering_pdf: None below the surface -> emitted (0) only
      const float c = dot(rec.n, unit(nd));
      if (c < 0.0f) return false;
      spdf = c / CLV_PI;
    } else {
      spdf = 1.0f / (4.0f * CLV_PI);
    }
  }
  float atten[4];  // hero only on wavelength-dependent materials (trace.rs:61-70)
  if (m.wavelength_dependent) {
    atten[0] = mat_color(S, m, ray, hero, rec);
    atten[1] = atten[2] = atten[3] = 0.0f;
  } else {
#pragma unroll
    for (int i = 0; i < 4; ++i) atten[i] = mat_color(S, m, ray, waves[i], rec);
  }
  if (specular) {
#pragma unroll
    for (int i = 0; i < 4; ++i) beta[i] = beta[i] * atten[i];
  } else {
#pragma unroll
    for (int i = 0; i < 4; ++i) beta[i] = beta[i] * (atten[i] * spdf / mis);
  }
  ray.o = rec.p;
  ray.d = nd;
  return true;
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

__global__ void __launch_bounds__(128) wf_shade(ClvDeviceScene S, WfParams P, WfState W, WfCounters* C,
                                                double* __restrict__ film, uint32_t* err) {
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  bool live = false, need = false;
  if (i < W.Q) {
    uint4 m = W.meta[i];
    if (m.w & 1u) {
      const float4 a = W.o_time[i], b = W.d_lambda[i];
      Ray ray{mk(a.x, a.y, a.z), mk(b.x, b.y, b.z), a.w, __float_as_int(b.w)};
      const float4 hv = W.hit[i];
      Hit h;
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
      Rng rng;
      const uint2 k = W.key[i];
      rng.key = (uint64_t)k.x | ((uint64_t)k.y << 32);
      rng.counter = m.z;
      const float4 bv = W.beta[i], lv = W.L[i];
      float beta[4] = {bv.x, bv.y, bv.z, bv.w}, L[4] = {lv.x, lv.y, lv.z, lv.w};
      const int hero = ray.lambda;
      bool cont = shade_bounce(S, ray, beta, L, h, full, rng, err);
      const uint32_t depth = m.y + 1;
      if (cont && depth > P.max_depth) cont = false;  // trace at depth > max_depth returns 0
      if (cont) {
        W.o_time[i] = make_float4(ray.o.x, ray.o.y, ray.o.z, ray.time);
        W.d_lambda[i] = make_float4(ray.d.x, ray.d.y, ray.d.z, __int_as_float(ray.lambda));
        W.beta[i] = make_float4(beta[0], beta[1], beta[2], beta[3]);
        W.L[i] = make_float4(L[0], L[1], L[2], L[3]);
        W.meta[i] = make_uint4(m.x, depth, rng.counter, 1u);
        live = true;
      } else {
        film_deposit(S, film, m.x, hero, L);
        need = true;
      }
    }
  }
  // finished paths take new work items, one atomic per warp
  const unsigned mask = __ballot_sync(0xFFFFFFFFu, need);
  if (mask) {
    const int lane = threadIdx.x & 31;
    const int leader = __ffs(mask) - 1;
    unsigned long long base = 0;
    if (lane == leader) base = atomicAdd(&C->next_work, (unsigned long long)__popc(mask));
    base = __shfl_sync(0xFFFFFFFFu, base, leader);
    if (need) {
      const uint64_t w = base + __popc(mask & ((1u << lane) - 1u));
      if (w < P.total) {
        wf_start_path(S, P, W, i, w);
        live = true;
      } else {
        W.meta[i].w = 0u;
      }
    }
  }
  const unsigned lm = __ballot_sync(0xFFFFFFFFu, live);
  if ((threadIdx.x & 31) == 0 && lm) atomicAdd(&C->live, (unsigned)__popc(lm));
}

}  // namespace clvd
