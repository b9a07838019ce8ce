/* clovers_gpu.h -- C ABI of the GB300 (sm_103a) render path of clovers.
 *
 * This library replaces the reference's CPU render driver
 * (clovers-cli/src/draw_cpu.rs:26-31, `draw(global, render_options, scene,
 * sampler) -> Vec<Xyz<E>>`) and the scene it consumes
 * (clovers-cli/src/json_scene.rs:12-27, `initialize(path, bvh, w, h) ->
 * Scene`).  The reference has no FFI of its own (it is one Rust binary); these
 * are the entry points a Rust `extern "C"` block in clovers-cli would bind.
 *
 * Conventions: every function returns 0 on success or a negative CLV_E*
 * status; clv_last_error() then holds a message (per thread).  No exception
 * crosses this boundary.  Output buffers are owned by the caller.  Handles are
 * opaque; one handle must not be used by two threads at the same time.
 * Functions named *_device take device pointers and a cudaStream_t passed as
 * void*, and are asynchronous with respect to the host.
 */
#ifndef CLOVERS_GPU_H
#define CLOVERS_GPU_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define CLV_OK 0
#define CLV_E_INVALID -1   /* bad argument or unsupported option            */
#define CLV_E_SCENE -2     /* scene file / mesh cannot be loaded            */
#define CLV_E_CUDA -3      /* CUDA runtime error (message has the details)  */
#define CLV_E_DEVICE -4    /* a kernel reported an error flag (stack, nesting) */

#define CLV_BVH_LAM 0 /* BvhAlgorithm::Lam (bvh/build/longest_axis_midpoint.rs) */
#define CLV_BVH_SAH 1 /* BvhAlgorithm::Sah (the clovers-cli default, render.rs:43-44) */

/* RenderMode, clovers-cli/src/render.rs:51-61 */
#define CLV_MODE_PATH_TRACING 0
#define CLV_MODE_NORMAL_MAP 1
#define CLV_MODE_BVH_TEST_COUNT 2
#define CLV_MODE_PRIMITIVE_TEST_COUNT 3

typedef struct clv_scene clv_scene;               /* host-side flattened scene */
typedef struct clv_device_scene clv_device_scene; /* scene resident in GPU memory */

/* RenderOptions (clovers-cli/src/render.rs:16-49) minus the file options,
 * plus the seed of the counter-based random streams. */
typedef struct clv_render_opts {
  uint32_t width;               /* -w, default 1024 */
  uint32_t height;              /* -h, default 1024 */
  uint32_t samples;             /* -s, samples per pixel, default 64 */
  uint32_t max_depth;           /* -d, default 64 */
  uint32_t mode;                /* CLV_MODE_*, default path tracing */
  uint32_t sampler;             /* 0 = random (default); 1 = blue noise: unsupported */
  uint64_t seed;                /* stream seed; identical seeds give identical images */
  uint32_t sample_offset;       /* index of the first sample (progressive rendering) */
  uint32_t path_slots;          /* wavefront paths in flight, 0 = automatic */
} clv_render_opts;

typedef struct clv_scene_info {
  uint64_t objects;     /* top-level objects after list flattening */
  uint32_t nodes;       /* BVH nodes */
  uint32_t triangles, quads, spheres, compound;
  uint32_t materials;
  uint32_t tree_depth;  /* BVH depth (root = 1) */
  uint32_t mis_nodes;
  uint32_t width, height;
  uint32_t traversal_level; /* intersect variant the scene needs: 0 primitives only, 1 wrapper
                               chains (Translate/RotateY over Boxy, spheres, quads, triangles),
                               2 media or nested lists; only objects the BVH reaches count */
} clv_scene_info;

typedef struct clv_stats {
  double gpu_ms;           /* device time of the render kernels */
  uint64_t samples;        /* width * height * spp */
  uint32_t device_errors;  /* CLV_ERR_* bits reported by kernels (0 = none) */
  uint32_t kernel_launches;
} clv_stats;

/* ---- scenes ------------------------------------------------------------ */

/* json_scene::initialize (clovers-cli/src/json_scene.rs:12-27): parse a
 * clovers scene file, build the SAH BVH and the MIS (priority) BVH on the
 * host.  width/height fix the camera aspect ratio. */
int clv_scene_load_json(const char* path, uint32_t width, uint32_t height, int bvh_alg, clv_scene** out);

/* Same, from the JSON text itself; relative STL paths resolve against base_dir. */
int clv_scene_load_json_text(const char* json, const char* base_dir, uint32_t width, uint32_t height, int bvh_alg,
                             clv_scene** out);

/* A triangle-only scene: Triangle::from_coordinates per index triple
 * (clovers/src/objects/triangle.rs:106-117), all with the default material.
 * Used for ray-cast workloads; it has no camera and no priority objects. */
int clv_scene_from_mesh(const float* verts, uint32_t nverts, const uint32_t* indices, uint32_t ntris,
                        clv_scene** out);

/* Scene options, set before clv_scene_upload.  No counterpart in the
 * reference (an opt-in precision mode).
 * CLV_OPT_WATERTIGHT 1: triangles use the watertight test of Woop, Benthin
 * and Wald 2013 (shear-frame edge functions, double-precision fallback on a
 * zero edge function) on their vertices as given, so rays through shared
 * edges and vertices of a closed mesh never slip through.  It also drops the
 * reference's rejection of rays within 1e-4 of the plane.  Results then
 * differ from the reference's Triangle::hit on edge and grazing hits; the
 * default 0 keeps the reference's test and its bit-exact hit ids. */
#define CLV_OPT_WATERTIGHT 1u
int clv_scene_set_option(clv_scene* scene, uint32_t option, uint32_t value);

int clv_scene_info_get(const clv_scene* scene, clv_scene_info* out);
void clv_scene_free(clv_scene* scene);

/* Copies the flattened scene to GPU memory (BVH nodes, primitive records,
 * materials, spectral tables, MIS tree). */
int clv_scene_upload(const clv_scene* scene, clv_device_scene** out);
void clv_device_scene_free(clv_device_scene* dscene);

/* ---- render: the draw() replacement ------------------------------------ */

/* draw_cpu::draw (clovers-cli/src/draw_cpu.rs:26-146): renders and writes the
 * mean XYZ(E) per pixel, row-major with row 0 at the top of the image (the
 * reference's pixelbuffer order), xyz_out = width*height*3 floats on the host.
 * opts->width/height must match the scene's.  Blocks until done. */
int clv_render(clv_device_scene* dscene, const clv_render_opts* opts, float* xyz_out, clv_stats* stats);

/* Device variant: ADDS the per-pixel sums of film deposits (f64, not divided
 * by spp) into film_dev (width*height*3 doubles, caller-zeroed), on `stream`.
 * The wavefront engine polls a live-path counter from the host, so the call
 * returns once the film is complete. */
int clv_render_device(clv_device_scene* dscene, const clv_render_opts* opts, double* film_dev, void* stream);

/* Renders n scenes in one wavefront: the (pixel, sample) work of all scenes
 * shares one set of path slots and one sequence of kernel launches per bounce,
 * so scenes of uneven size keep the GPU full.  Each scene adds its film sums
 * into films[k] (width*height*3 doubles, caller-zeroed), exactly as n calls of
 * clv_render_device with the same options would (same random streams).  The
 * path state of the batch lives in dscenes[0].  Up to 128 scenes share one
 * wavefront (their views sit in constant memory, so concurrent batch calls
 * run one after another); larger batches render as consecutive wavefronts of
 * 128 scenes.  No counterpart in the reference, which renders one scene per
 * process. */
int clv_render_batch(clv_device_scene* const* dscenes, const clv_render_opts* opts, double* const* films, uint32_t n,
                     void* stream);

/* No counterpart in the reference.  The same render as clv_render_device
 * (wavefront path tracing only) for callers that cannot allocate GPU memory
 * while they render -- a host that pre-reserves device memory for its own
 * pool, or a real-time caller that must not hit out-of-memory mid-frame.  It
 * calls no cudaMalloc/cudaFree: path state, queues and counters live in one
 * static device array of 65536 path slots (about 10 MB, reserved on every GPU
 * that loads the library until the process exits).  opts->path_slots above
 * 65536 is rejected with CLV_E_INVALID; 0 means 65536.  The scene's tuned
 * wavefront shape applies (its path slots capped at 65536); scenes whose BVH
 * is deeper than 64 levels are refused (their traversal stacks would need
 * device memory).  Every call shares the array and leaves its contents
 * behind: calls that overlap on the GPU (other streams, other threads) race
 * and must be serialised by the caller.  The call synchronises its stream
 * (it polls the live-path count), so it cannot be captured into a CUDA
 * graph; it returns once the film is complete, like clv_render_device. */
int clv_render_device_noalloc(clv_device_scene* dscene, const clv_render_opts* opts, double* film_dev, void* stream);

/* Film resolve (clovers-cli/src/write.rs:39-44): mean = film / spp (f64) ->
 * f32 XYZ(E) -> D65 -> sRGB -> u8.  xyz_out_dev (optional) receives the f32
 * means.  Device pointers. */
int clv_resolve_device(const double* film_dev, uint32_t width, uint32_t height, uint32_t spp, float* xyz_out_dev,
                       uint8_t* rgb_out_dev, void* stream);

/* Host variant of the resolve for XYZ(E) means already on the host. */
int clv_resolve_srgb(const float* xyz, uint32_t width, uint32_t height, uint8_t* rgb_out);

/* Wavefront shape tuning (no counterpart in the reference; part of the
 * batching and autotuning layer).  Renders `opts` -- pass a short render, a few samples per
 * pixel of the workload to tune for -- twice for each candidate shape: paths
 * in flight (path_slots) SMs x {1, 2, 4, 8, 16} x 1024, shading grids of
 * {8, 16, 32} blocks per SM, and, for primitive-level scenes (traversal level
 * 0, BVH of at most 64 levels), the intersect's queue appends per block (one
 * atomic per class and block, behind two block barriers) or per warp (no
 * barrier: better where traversal lengths vary widely within a block); then,
 * at the fastest of those, the diffuse shading kernel at 8 instead of 5
 * resident blocks per SM (64 instead of 96 registers).  It keeps the fastest
 * in the scene: later wavefront renders of this scene with
 * opts->path_slots = 0 use it.  results (optional) receives up to max_results
 * timings, n_results their count (31 for primitive-level scenes, else 16).
 * Allocates a film and the largest path state it tries. */
typedef struct clv_tune_result {
  uint32_t path_slots;
  uint32_t shade_blocks_per_sm;
  uint32_t warp_appends;          /* 1: the intersect appends its queues per warp, 0: per block */
  uint32_t diffuse_blocks_per_sm; /* resident blocks per SM of the diffuse shading kernel (5 or 8) */
  float ms;
} clv_tune_result;
int clv_autotune(clv_device_scene* dscene, const clv_render_opts* opts, clv_tune_result* results,
                 uint32_t max_results, uint32_t* n_results, void* stream);

/* Sets the wavefront shape clv_autotune would keep (0 = the built-in default
 * for path_slots, shade_blocks_per_sm and diffuse_blocks_per_sm), e.g. to
 * reuse a shape tuned in an earlier run.  warp_appends = 1 is valid for
 * primitive-level scenes only (clv_scene_info.traversal_level 0, BVH of at
 * most 64 levels); diffuse_blocks_per_sm takes 0, 5 or 8. */
int clv_device_scene_set_shape(clv_device_scene* dscene, uint32_t path_slots, uint32_t shade_blocks_per_sm,
                               uint32_t warp_appends, uint32_t diffuse_blocks_per_sm);

/* ---- ray casts --------------------------------------------------------- */

/* Closest hit of each ray with BVHNode::hit's exact decision order
 * (clovers/src/bvh/hitable_trait.rs:15-81).  rays = n x {ox,oy,oz,tmin,
 * dx,dy,dz,tmax} (32 bytes each, directions unit length); prim_id = index of
 * the top-level object hit (0xFFFFFFFF on a miss), t = hit distance.
 * node_visits / prim_tests (optional, may be NULL) count BVHNode::hit calls
 * (clovers/src/bvh/testcount.rs:23) and primitive tests per ray.  Host buffers;
 * blocks until done. */
int clv_raycast(clv_device_scene* dscene, const float* rays, uint64_t n, uint32_t* prim_id, float* t,
                uint32_t* node_visits, uint32_t* prim_tests);

/* Device variant, asynchronous on `stream`.  Batches of 65536 rays or more
 * are traversed in the order of a Morton code of their origins (a counting
 * sort on the device; results still go to each ray's own index); the sort's
 * scratch (8 bytes per ray) is kept by the scene and grown on demand, so a
 * call with more rays than any before it allocates. */
int clv_raycast_device(const clv_device_scene* dscene, const float* rays_dev, uint64_t n, uint32_t* prim_id_dev,
                       float* t_dev, uint32_t* node_visits_dev, uint32_t* prim_tests_dev, void* stream);

/* ---- learned path guiding (no counterpart in the reference) -------------
 *
 * A small MLP (inputs: position in the scene box, outgoing direction, hero
 * wavelength; 12-frequency sin/cos encoding; three hidden layers of 64; BF16
 * weights with FP32 accumulation on the tensor cores) outputs an 8-lobe von
 * Mises-Fisher mixture over incident directions at Lambertian vertices.  A
 * guided render draws a share `alpha` of its Lambertian bounces from that
 * mixture and the rest from the reference's MixturePDF, and weights each
 * bounce by the blended density, so the image stays an unbiased estimate for
 * any network.  It also stores training records (inputs, sampled direction,
 * integrand / density of the hero wavelength) of the first two Lambertian
 * vertices of each path; clv_guide_train takes Adam steps on them. */
typedef struct clv_guide clv_guide;
typedef struct clv_guide_opts {
  uint32_t record_capacity; /* training records kept per render call, 0 = 2^21 */
  float learning_rate;      /* Adam step size, 0 = 5e-3 */
  uint64_t seed;            /* weight initialisation */
} clv_guide_opts;
#define CLV_GUIDE_PARAMS 22016  /* fp32 weights: W1 64x176, W2 64x64, W3 64x64, W4 40x64, row-major */
#define CLV_GUIDE_OUTPUTS 40    /* raw outputs: 8 lobes x (mean direction xyz, log concentration, logit) */

int clv_guide_create(const clv_guide_opts* opts, clv_guide** out);
void clv_guide_free(clv_guide* guide);
int clv_guide_get_params(const clv_guide* guide, float* params);
int clv_guide_set_params(clv_guide* guide, const float* params);

/* Path tracing like clv_render_device, with a share alpha in [0, 1] of the
 * Lambertian bounces drawn from the guide.  Replaces the guide's training
 * records with those of this call.  alpha = 0 renders the reference's
 * estimator (other random streams than clv_render_device) and still records. */
int clv_render_guided(clv_device_scene* dscene, const clv_render_opts* opts, clv_guide* guide, float alpha,
                      double* film_dev, void* stream);

/* clv_render_batch with the guide: the Lambertian bounces of every scene of
 * the batch are drawn (share alpha) from the one guide, its inputs normalised
 * to each scene's own box, and they leave training records for
 * clv_guide_train, as clv_render_guided does for one scene.  No counterpart in
 * the reference. */
int clv_render_batch_guided(clv_device_scene* const* dscenes, const clv_render_opts* opts, double* const* films,
                            uint32_t n, clv_guide* guide, float alpha, void* stream);

/* `steps` Adam steps on consecutive batches of `batch` records (0 = 65536)
 * of the last guided render, taken from the records that carry light (f > 0;
 * the others add nothing to the gradient); mean_loss (optional) receives the
 * mean of -f log q over the records used. */
int clv_guide_train(clv_guide* guide, uint32_t steps, uint32_t batch, double* mean_loss, void* stream);
int clv_guide_record_count(const clv_guide* guide, uint64_t* n);
/* records: n x 12 floats {u0..u6, 0, w.x, w.y, w.z, f} (u: normalised inputs) */
int clv_guide_get_records(const clv_guide* guide, float* records, uint64_t n);

/* Network on host arrays (tests, diagnostics).  queries: n x 8 floats {u0..u6,
 * 0}, inputs already normalised to [0, 1]; out: n x 40 raw outputs. */
int clv_guide_forward(clv_guide* guide, const float* queries, uint64_t n, float* out);
/* Sum over the records (n x 12 floats as above) of the gradient of -f log q(w)
 * with respect to the fp32 weights (CLV_GUIDE_PARAMS floats); loss = the sum
 * of -f log q.  No weight update. */
int clv_guide_gradient(clv_guide* guide, const float* records, uint64_t n, float* grads, double* loss);
/* Error bits of the guide kernels since the last call (clears them). */
int clv_guide_status(clv_guide* guide, uint32_t* flags);
/* One 128 x n x k BF16 tensor-core product through the guide's operand
 * layouts, against a CUDA-core sum of the same products: max |difference|. */
int clv_guide_selftest_mma(uint32_t n, uint32_t k, uint64_t seed, float* d_out, float* max_abs_err);

/* ---- status ------------------------------------------------------------ */

/* Error bits raised by kernels since the last call (clears them). */
int clv_device_status(clv_device_scene* dscene, uint32_t* flags_out);

const char* clv_last_error(void);
const char* clv_version(void);

/* Device memory plumbing for callers without their own CUDA runtime binding
 * (films and ray buffers of the *_device entry points).  clv_memcpy copies in
 * any direction (unified addressing); both block. */
int clv_device_alloc(uint64_t bytes, void** out);
void clv_device_free(void* ptr);
int clv_memcpy(void* dst, const void* src, uint64_t bytes);
int clv_memset(void* dst, int value, uint64_t bytes);

/* Number of kernels this library has launched since it was loaded. */
uint64_t clv_kernel_launches(void);

/* ---- diagnostics (no counterpart in the reference) ----------------------- */

/* One wavefront render with per-kernel device times and traversal counts.
 * The times are those of the production kernels; the counts come from a
 * second render of the same samples with the counting kernels (into scratch
 * memory, so film_dev holds one render). */
typedef struct clv_render_profile {
  double ms_init, ms_intersect, ms_shade;  /* summed device time per kernel type */
  uint64_t intersect_launches, shade_launches;
  uint64_t paths;          /* samples traced */
  uint64_t path_segments;  /* closest-hit queries (one per bounce of a live path) */
  uint64_t node_visits;    /* BVHNode::hit calls over all queries */
  uint64_t prim_tests;     /* primitive tests over all queries */
  uint64_t path_slots;     /* paths in flight */
} clv_render_profile;
int clv_render_profile_run(clv_device_scene* dscene, const clv_render_opts* opts, double* film_dev, void* stream,
                           clv_render_profile* out);

/* Checks the traversal's fast slab division (reciprocal + one FMA correction)
 * against IEEE division on n random operand pairs; mismatches must be 0. */
int clv_selftest_division(uint64_t n, uint64_t seed, uint64_t* mismatches);

/* Checks the render path's own natural logarithm (used by ConstantMedium's
 * free-flight draw, clovers/src/objects/constant_medium.rs:102, in place of
 * the library logf whose last bit differs between CUDA and host libms) over
 * every f32 in (0, 1]: max_ulp = largest error in f32 ulps against the GPU's
 * double-precision log, not_nearest = results that are not the nearest f32 of
 * it.  With x and y (host arrays of n floats) it also evaluates the routine on
 * x, for bitwise comparison with the CPU build of the same routine. */
int clv_selftest_log(const float* x, float* y, uint64_t n, double* max_ulp, uint64_t* not_nearest);

/* Exercises the guide kernels' bounded-wait error path: one CTA allocates
 * TMEM, waits on an mbarrier that nothing arrives on (no copy or MMA is in
 * flight) for `clocks` SM clocks, then raises the timeout flag, frees its
 * TMEM and returns.  flags = the error bits raised (CLV_ERR_GUIDE, 8),
 * freed = 1 when the kernel reached its TMEM release. */
int clv_guide_selftest_timeout(uint64_t clocks, uint32_t* flags, uint32_t* freed);

#ifdef __cplusplus
}
#endif

#endif /* CLOVERS_GPU_H */
