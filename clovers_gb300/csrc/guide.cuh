// Learned path guiding: a small MLP maps a diffuse path vertex (position,
// outgoing direction, hero wavelength) to an 8-lobe von Mises-Fisher mixture
// over incident directions.  The renderer draws a share `alpha` of its diffuse
// bounces from that mixture and the rest from the reference's own
// BSDF + light MixturePDF, and weights every bounce by the blended density
// (one-sample MIS), so the estimator stays unbiased whatever the network says.
// The network is trained online on the radiance the renderer's own paths
// carry.  The reference renderer has no guiding; this is an addition to its
// render path.
//
// Network (BF16 operands, FP32 accumulation on the tcgen05 tensor cores):
//   inputs   u[7] in [0,1]: position normalised to the scene box (3),
//            outgoing direction * 0.5 + 0.5 (3), (lambda - 380) / 400 (1)
//   encoding x[176]: x[24j + 2k] = sin(2^k pi u_j), x[24j + 2k + 1] =
//            cos(2^k pi u_j) for j < 7, k < 12 (168 values), x[168 + j] = u_j,
//            x[175] = 1 (bias of layer 1)
//   layers   h1 = relu(W1 x), h2 = relu(W2 h1), h3 = relu(W3 h2), o = W4 h3;
//            W1 64x176, W2 and W3 64x64, W4 40x64.  Hidden unit 63 of h1..h3
//            is forced to 1 and carries the next layer's bias.
//   head     lobe k uses o[5k..5k+4]: mean direction = normalize(o[5k..5k+2]),
//            concentration = exp(clamp(o[5k+3], GD_LOGK_MIN, GD_LOGK_MAX)),
//            mixture weight = softmax over o[5k+4].
// Training minimises  -f * log q(w)  per record (w the sampled direction,
// f = integrand / sampling density of that bounce, hero wavelength), the
// Monte-Carlo form of the KL divergence from the radiance-weighted target
// (Mueller et al. 2019, "Neural Importance Sampling"; the vMF mixture head
// follows Dong et al. 2023, "Neural Parametric Mixtures for Path Guiding").
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#define GD_IN 176
#define GD_H 64
#define GD_OUT 40
#define GD_OUTP 48  // output rows padded to the MMA's N granularity (16)
#define GD_LOBES 8
#define GD_FREQ 12
#define GD_TILE 128  // records / queries per MMA tile (M)
#define GD_LOGK_MIN (-3.0f)
#define GD_LOGK_MAX 8.0f

// fp32 master parameters, row-major [out][in]
#define GD_P_W1 0
#define GD_P_W2 (GD_H * GD_IN)
#define GD_P_W3 (GD_P_W2 + GD_H * GD_H)
#define GD_P_W4 (GD_P_W3 + GD_H * GD_H)
#define GD_NPARAM (GD_P_W4 + GD_OUT * GD_H)  // 22016

// BF16 operand blob: every matrix in the no-swizzle K-major canonical layout
// of the tensor-core shared-memory descriptors (8-row x 16-byte core matrices,
// K-adjacent core matrices 128 bytes apart, 8-row groups K/8*128 bytes apart),
// so one bulk copy puts it in shared memory ready for tcgen05.mma.
// Forward operands are W (N = out, K = in); backward operands are W^T
// (N = in, K = out) for dH = dZ W.
#define GD_B_W1 0
#define GD_B_W2 (GD_B_W1 + GD_H * GD_IN * 2)        // 22528
#define GD_B_W3 (GD_B_W2 + GD_H * GD_H * 2)         // 30720
#define GD_B_W4 (GD_B_W3 + GD_H * GD_H * 2)         // 38912
#define GD_B_FWD (GD_B_W4 + GD_OUTP * GD_H * 2)     // 45056
#define GD_B_W4T GD_B_FWD                           // [in 64][out 48]
#define GD_B_W3T (GD_B_W4T + GD_H * GD_OUTP * 2)    // 51200
#define GD_B_W2T (GD_B_W3T + GD_H * GD_H * 2)       // 59392
#define GD_B_ALL (GD_B_W2T + GD_H * GD_H * 2)       // 67584

// byte offset of element (row r, column k) of a K-major matrix with K columns
__host__ __device__ constexpr uint32_t gd_cofs(uint32_t r, uint32_t k, uint32_t K) {
  return (r >> 3) * (K >> 3) * 128u + (k >> 3) * 128u + (r & 7u) * 16u + (k & 7u) * 2u;
}

#define CLV_ERR_GUIDE 8u  // a tensor-core wait of the guide ran out of time

// Training record: 3 float4 = {u0 u1 u2 u3} {u4 u5 u6 -} {w.xyz, f}
#define GD_REC_F4 3

// What the guide kernels need, passed by value.
struct GuideDev {
  const unsigned char* wblob;  // GD_B_ALL bytes
  float4* rec;                 // GD_REC_F4 float4 per record
  unsigned int* rec_count;     // records written by the current render pass
  uint32_t rec_cap;
  uint4* slot;                 // per path slot: record ids of its first two guided
                               // vertices and the hero throughput before each
  float bmin[3], binv[3];      // position normalisation (scene box)
  const float* boxes;          // batches: per scene {bmin[3], binv[3]}, indexed by the slot's scene
                               // (meta.w >> 8); null: bmin / binv
  float alpha;                 // share of guided samples in the blend
  uint32_t* err;
};
// Position normalisation of a slot's scene: {bmin, binv} of the batch table or the single scene.
__device__ __forceinline__ void gd_box(const GuideDev& G, uint32_t meta_w, float lo[3], float inv[3]) {
  if (G.boxes) {
    const float* b = G.boxes + 6 * (size_t)(meta_w >> 8);
#pragma unroll
    for (int a = 0; a < 3; ++a) {
      lo[a] = b[a];
      inv[a] = b[3 + a];
    }
  } else {
#pragma unroll
    for (int a = 0; a < 3; ++a) {
      lo[a] = G.bmin[a];
      inv[a] = G.binv[a];
    }
  }
}

// The guided-vertex queue of one bounce and the path state it reads.
struct GdQueue {
  const uint32_t* queue;
  const unsigned int* count;
  const float4* full;      // 3 per slot: p.xyz u | n.xyz v | front, material
  const float4* d_lambda;  // direction.xyz, wavelength bits
  float4* hit;             // in: plain direction + flag; out: direction + guide density
  uint4* meta;             // rng counter in .z
  const uint2* key;
};

// Host side of a guide (defined in guide.cu).
struct clv_guide {
  float* params = nullptr;  // fp32 master weights (device)
  float* adam_m = nullptr;
  float* adam_v = nullptr;
  float* grad = nullptr;
  unsigned char* wblob = nullptr;
  float4* rec = nullptr;
  unsigned int* rec_count = nullptr;
  uint32_t rec_cap = 0;
  float4* rec_keep = nullptr;          // records with f > 0, gathered before training
  unsigned int* keep_count = nullptr;
  uint4* slot = nullptr;
  uint32_t slots = 0;
  uint32_t* err = nullptr;
  double* loss = nullptr;  // device accumulator of the last training batch
  float lr = 5e-3f;
  uint64_t step = 0;
  ~clv_guide();
  uint4* ensure_slots(uint32_t q);
};

// Host launchers (guide.cu); all asynchronous on `st`.
// gd_launch_queue neither counts its launch nor sets kernel attributes, so it
// can be captured into a graph; call gd_prepare once before.
void gd_prepare();
void gd_launch_queue(const GuideDev& G, const GdQueue& Q, uint32_t max_queries, cudaStream_t st);
void gd_reset_records(clv_guide* g, cudaStream_t st);
GuideDev gd_view(clv_guide* g, const float root_box[6], float alpha);

// Shared with the main translation unit: error text and launch counting.
int clv_internal_fail(int code, const char* msg);
void clv_internal_count_launches(unsigned long long n);
