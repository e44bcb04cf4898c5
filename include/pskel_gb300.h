/*
 * pskel_gb300 -- C ABI of the GB300 (sm_103a) iterative-stencil library.
 *
 * This is the drop-in boundary under PSkel's C++ skeleton API. The header
 * templates in include/PSkel*.h (and any FFI binding) call these functions;
 * they take plain pointers, sizes and descriptors, never C++ or torch types.
 *
 * Array layouts are the reference's (PSkelArray.hpp:349-352, 658-677): 2D
 * element (h, w) at [h * pitch + w]; 3D element (h, w, d) at
 * [(h * width + w) * depth + d] (d fastest).
 *
 * Semantics of one iterative run follow StencilBase::runIterativeGPU /
 * runIterativeCPU (PSkelStencil.hpp:880-938, 1046-1097):
 *   - iteration k reads one buffer and writes the other (ping-pong);
 *   - 2D: only cells with r <= h < H-r and r <= w < W-r are written
 *     (r = mask range), so each buffer keeps its own ring;
 *   - 3D: every cell is written, neighbours outside the grid read
 *     mask.halo_value (Mask3D::get, PSkelMask.hpp:186-199);
 *   - after `iterations` steps the result is in `out` when iterations is odd
 *     and in `in` when it is even (the device state runIterativeGPU copies
 *     back from, :1083-1090). The *_host entry points do that copy back.
 *
 * Device entry points are asynchronous on `stream` (a cudaStream_t, NULL for
 * the legacy default stream). Kernel-side errors (a bounded wait that ran
 * out, a Life cell outside {0,1}) are latched in a per-device error word;
 * pskel_sync() waits for the stream and reports and clears it. Host entry
 * points are synchronous and check it themselves.
 *
 * Not thread-safe, like the reference (its GA tuner uses a global evaluator,
 * PSkelStencil.hpp:1866-1881): one caller thread per process. The device
 * entry points of one device share its scratch (Life bit planes, multi-pass
 * counters, residual partials), so calls that overlap on the GPU (issued on
 * two streams without an ordering between them) race.
 */
#ifndef PSKEL_GB300_H
#define PSKEL_GB300_H

#include <stddef.h>
#include <stdint.h>

#if defined(__GNUC__)
#define PSKEL_API __attribute__((visibility("default")))
#else
#define PSKEL_API
#endif

#ifdef __cplusplus
extern "C" {
#endif

typedef int32_t pskel_status;
#define PSKEL_OK 0
#define PSKEL_ERR_INVALID 1     /* bad argument: null pointer, size, mask shape */
#define PSKEL_ERR_UNSUPPORTED 2 /* valid request outside the implemented kernels */
#define PSKEL_ERR_CUDA 3        /* a CUDA runtime call failed (pskel_last_error) */
#define PSKEL_ERR_DEVICE 4      /* a kernel latched an error (pskel_last_error) */
#define PSKEL_ERR_NOMEM 5       /* device or pinned host allocation failed */

typedef enum pskel_dtype {
  PSKEL_U8 = 0,   /* uint8 cells (Game of Life) */
  PSKEL_F32 = 1,  /* fp32 storage, fp32 arithmetic */
  PSKEL_BF16 = 2  /* bf16 storage (rounded to nearest even every step), fp32 arithmetic */
} pskel_dtype;

typedef enum pskel_op {
  /* out = sum_n weights[n] * in(neighbour n), products and sums in mask
   * order without contraction. */
  PSKEL_OP_LINEAR = 0,
  /* Game of Life over the mask neighbourhood: s = sum of neighbours,
   * out = (s == 3 || (s == 2 && c == 1)); the mask must be the 8 Moore
   * offsets (any order). */
  PSKEL_OP_LIFE = 1,
  /* Upwind advection-diffusion on the 4-neighbour cross with per-cell winds
   * (the arithmetic of the reference's CLOUDSIM kernel, PSkelStencil.hpp:347-387). */
  PSKEL_OP_ADVECT = 2
} pskel_op;

/* Mirror of MaskBase/Mask2D/Mask3D (PSkelMask.h:48-218). */
typedef struct pskel_mask {
  int32_t size;           /* number of entries */
  int32_t dimension;      /* 2 or 3 */
  const int32_t* offsets; /* size*dimension host ints: (dh, dw[, dd]) per entry */
  const float* weights;   /* size host floats (ignored by LIFE and ADVECT) */
  float halo_value;       /* value read outside a 3D grid (Mask3D haloValue) */
  int32_t range;          /* 0: max |offset| (MaskBase::getRange) */
} pskel_mask;

typedef struct pskel_stencil {
  pskel_op op;
  pskel_dtype dtype;
  pskel_mask mask;
  /* ADVECT only: per-cell wind fields, same dtype and layout as the grid.
   * Device pointers for the device entry points, host pointers for *_host. */
  const void* wind_u;
  const void* wind_v;
  float diffusivity; /* ADVECT: K */
  float dt;          /* ADVECT: time step */
  float inv_dx;      /* ADVECT: 1/dx */
} pskel_stencil;

/* Execution schedule. Changes only speed, never results. Zero fields take the
 * library's defaults. */
typedef struct pskel_schedule {
  int32_t tile_w;     /* core tile width (cells) */
  int32_t tile_h;     /* core tile height (cells) */
  int32_t tile_d;     /* 3D: core tile depth (cells) */
  int32_t time_steps; /* steps fused per pass over the grid (temporal block) */
  int32_t ctas;       /* persistent CTAs per launch */
} pskel_schedule;

/* Library version (major*10000 + minor*100 + patch). */
PSKEL_API int32_t pskel_version(void);

/* Message for the last failing call on this thread, "" if none. */
PSKEL_API const char* pskel_last_error(void);

/* Kernel launches (memsets not counted) issued by the calling thread's last
 * pskel_iterate2d call; 0 after a call that failed before launching. No
 * reference counterpart (a diagnostic: the reference launches one kernel per
 * step, PSkelStencil.hpp:1078-1082). */
PSKEL_API int64_t pskel_last_launches2d(void);

/* Wait for `stream`, then report and clear the device error word. */
PSKEL_API pskel_status pskel_sync(void* stream);

/* Splits `iterations` steps into passes of at most `time_steps` steps, each
 * of an odd length, so that after every pass the state sits in the buffer
 * (and next to the ring) where a step-by-step ping-pong has it. An even
 * `time_steps` is lowered by one. Writes at most `cap` pass lengths to
 * `passes` and returns the number of passes (host only). */
PSKEL_API int32_t pskel_plan_passes(int64_t iterations, int32_t time_steps, int32_t* passes, int32_t cap);

/* Iterative 2D stencil on device buffers.
 * Replaces StencilBase::runIterativeGPU(iterations, bx, by) and
 * runIterativeGPU(iterations, pyramidHeight, bx, by) (PSkelStencil.h:258-259,
 * PSkelStencil.hpp:943-1097) and runIterativeTilingGPU's inner temporal
 * blocking (PSkelStencil.h:292, PSkelStencil.hpp:1663-1862): schedule.time_steps
 * plays pyramidHeight / innerIterations, schedule.tile_* the tiling sizes.
 * `pitch` is the row pitch in elements (0 = width). The result ends in `out`
 * (odd iterations) or `in` (even), with its ring untouched; the other
 * buffer's contents afterwards are unspecified (the float paths ping-pong
 * through it, Life runs on internal bit planes and does not write it).
 * Reach-1 shapes and advection with several passes on grids of at most three
 * waves of tiles run every pass in one persistent launch (tiles wait for
 * their neighbourhood of the previous pass); the environment variable
 * PSKEL_FAST2D_MULTIPASS=1 / 0 forces that launch on / off. Results are the
 * same either way. */
PSKEL_API pskel_status pskel_iterate2d(const pskel_stencil* st, void* in, void* out, int64_t width, int64_t height,
                             int64_t pitch, int64_t iterations, const pskel_schedule* sched, void* stream);

/* Iterative 2D stencil on host arrays: the whole of runIterativeGPU
 * (PSkelStencil.hpp:1046-1097): copy in, iterate, copy the result into
 * `out_host`. `in_host` is not modified; `out_host` must hold the output
 * array's initial contents: its ring (cells outside r <= h < H-r,
 * r <= w < W-r) is read by every second step, as in runIterativeCPU, and only
 * that ring is copied to the device. Synchronous. */
PSKEL_API pskel_status pskel_run2d_host(const pskel_stencil* st, const void* in_host, void* out_host, int64_t width,
                              int64_t height, int64_t iterations, const pskel_schedule* sched);

/* Iterative 3D stencil on device buffers (linear mask, f32 or bf16).
 * Replaces Stencil3D::runIterativeGPU / runIterativeTilingGPU
 * (PSkelStencil.h:258, 292; PSkelStencil.hpp:1046-1097, 1663-1862), whose 3D
 * instantiation the reference cannot compile, with the semantics of
 * Stencil3D::runIterativeCPU (PSkelStencil.hpp:880-938, 2104-2113): every cell
 * is written each step, out-of-grid neighbours read mask.halo_value.
 * schedule.time_steps steps are fused per pass (2.5D streaming along h).
 * When residual_every > 0, residuals[k/residual_every - 1] receives the fp64
 * norm ||u_k - u_{k-1}||_2 for every k that is a multiple of residual_every
 * (device array of iterations/residual_every doubles). */
PSKEL_API pskel_status pskel_iterate3d(const pskel_stencil* st, void* in, void* out, int64_t width, int64_t height,
                                       int64_t depth, int64_t iterations, const pskel_schedule* sched,
                                       int64_t residual_every, double* residuals, void* stream);

/* Iterative 3D stencil on host arrays (copy in, iterate, copy the result into
 * out_host, residual norms into residuals_host). `in_host` is not modified;
 * the output array's initial contents are never read. Synchronous. For the
 * 7-point cross at one step per pass on grids of 128+ planes and up to 256
 * iterations, the copies overlap the compute: chunks of planes are copied in
 * while the first steps run on the planes already there, and final planes
 * are copied out while the last steps run on the others (same results). */
PSKEL_API pskel_status pskel_run3d_host(const pskel_stencil* st, const void* in_host, void* out_host, int64_t width,
                                        int64_t height, int64_t depth, int64_t iterations,
                                        const pskel_schedule* sched, int64_t residual_every,
                                        double* residuals_host);

/* ------------------------------------------------------------ out of core
 * Grids kept in host memory and streamed through the GPU in slabs of whole
 * rows (2D) or whole h-planes (3D), for grids larger than device memory.
 * Replaces the host tiling of runIterativeTilingGPU / runTilingGPU /
 * runAutoGPU (PSkelStencil.hpp:766-861, 1663-1760; tile geometry in
 * PSkelStencilTiling.h:75-140). Each slab is copied to the device with a halo
 * of ring + (T-1)*reach rows (2D) or T*reach planes (3D), iterated T =
 * inner_iterations steps there (the last pass fewer) and its core copied back;
 * copies in, compute and copies out of three consecutive slabs overlap on
 * three streams. Results are those of pskel_run2d_host / pskel_run3d_host,
 * bit for bit: `in_host` is not modified, the result lands in `out_host`
 * (2D: `out_host` must hold the output array's initial ring, as for
 * pskel_run2d_host). slab_rows = 0 sizes the slabs from `device_bytes`
 * (0 = 90% of the free device memory); inner_iterations = 0 takes 15; an even
 * inner_iterations is lowered by one. The first pass reads `in_host`, later
 * passes update `out_host` in place. Host arrays that are not pinned are
 * registered for the call; the device slots (2 + ceil(halo/slab_rows), at
 * least 3) stay allocated for later calls. 3D: no residual norms.
 * Synchronous. */
PSKEL_API pskel_status pskel_run2d_host_tiled(const pskel_stencil* st, const void* in_host, void* out_host,
                                              int64_t width, int64_t height, int64_t iterations, int64_t slab_rows,
                                              int32_t inner_iterations, int64_t device_bytes,
                                              const pskel_schedule* sched);
PSKEL_API pskel_status pskel_run3d_host_tiled(const pskel_stencil* st, const void* in_host, void* out_host,
                                              int64_t width, int64_t height, int64_t depth, int64_t iterations,
                                              int64_t slab_planes, int32_t inner_iterations, int64_t device_bytes,
                                              const pskel_schedule* sched);

/* The slab plan the two calls above would use (host only unless both
 * slab_rows and device_bytes are 0): plan[0] core rows per slab, plan[1] the
 * widest halo (rows), plan[2] slabs per pass, plan[3] device bytes allocated.
 * `depth` is ignored for a 2D mask. */
PSKEL_API pskel_status pskel_tiled_plan(const pskel_stencil* st, int64_t width, int64_t height, int64_t depth,
                                        int64_t iterations, int64_t slab_rows, int32_t inner_iterations,
                                        int64_t device_bytes, int64_t plan[4]);

/* ---------------------------------------------------------------- batches
 * Many 2D grids, each with its own size, iteration count and schedule, run by
 * ONE persistent kernel launch recorded once in a CUDA graph. There is no
 * counterpart in the reference, whose skeletons run one grid per call
 * (StencilBase::runIterativeGPU, PSkelStencil.hpp:1046-1097); a batch gives
 * every grid exactly the result pskel_iterate2d would (in `out` for an odd
 * iteration count, in `in` for an even one). The stencil must be a linear
 * mask of reach 1 in one of the shapes N,S,W,E / C,N,S,W,E / 3x3 row-major,
 * storage f32 or bf16, buffers and row pitches 16-byte aligned. */
typedef struct pskel_batch_grid {
  void* in;                /* device buffer, 16-byte aligned */
  void* out;               /* device buffer, 16-byte aligned */
  int64_t width, height;   /* grid size */
  int64_t pitch;           /* row pitch in elements (0 = width) */
  int64_t iterations;      /* steps for this grid */
  pskel_schedule schedule; /* time_steps used (0 = default) */
} pskel_batch_grid;

typedef struct pskel_batch pskel_batch;

/* Prepares a batch: per-grid geometry, tensor maps, the work list and the
 * CUDA graph of the run. The grids' buffers must stay valid until destroy. */
PSKEL_API pskel_status pskel_batch_create(const pskel_stencil* st, const pskel_batch_grid* grids, int32_t n,
                                          pskel_batch** out);
/* Launches the batch's graph on `stream` (asynchronous; see pskel_sync). */
PSKEL_API pskel_status pskel_batch_run(pskel_batch* b, void* stream);
/* Total cell updates of one run (sum of width * height * iterations). */
PSKEL_API int64_t pskel_batch_cell_updates(const pskel_batch* b);
PSKEL_API pskel_status pskel_batch_destroy(pskel_batch* b);

/* --------------------------------------------------------- schedule search
 * Replaces runIterativeAutoGPU's genetic search (PSkelStencil.hpp:1865-2076),
 * which needs GAlib and evaluates an analytic objective, with measured
 * timings and a learned cost model. None of these change results. */

/* Candidate schedules the library can run for this 2D stencil; writes at most
 * `cap` to `out` and returns how many there are. Host only. */
PSKEL_API int32_t pskel_candidates2d(const pskel_stencil* st, int64_t width, int64_t height, int64_t iterations,
                                     pskel_schedule* out, int32_t cap);

/* Times `n` schedules on device buffers (their contents are overwritten): one
 * untimed run each, then the median of `reps` runs in ms, CUDA events on
 * `stream`. The exhaustive tuner is this over pskel_candidates2d. */
PSKEL_API pskel_status pskel_time2d(const pskel_stencil* st, void* in, void* out, int64_t width, int64_t height,
                                    int64_t pitch, int64_t iterations, const pskel_schedule* scheds, int32_t n,
                                    int32_t reps, double* ms, void* stream);

/* The cost of one grid inside a batched launch (pskel_batch_*), for tuning
 * batches: for each schedule, `copies` copies of a width x height grid with
 * buffers carved from the caller's device `pool` (cleared to zero first) run
 * as one batch, `reps` timed runs after an untimed one; ms[i] = median batch
 * time / copies. The copies give the GPU about two waves of tiles, as many as
 * the pool holds; copies_used (may be NULL) receives their number. */
PSKEL_API pskel_status pskel_time_batch2d(const pskel_stencil* st, void* pool, int64_t pool_bytes, int64_t width,
                                          int64_t height, int64_t iterations, const pskel_schedule* scheds,
                                          int32_t n, int32_t reps, double* ms, int32_t* copies_used, void* stream);

/* The reference's GA with its analytic objective (solve2D/objective2D,
 * PSkelStencil.hpp:1883-1941: simple GA, two 16-bit genes, population
 * `popsize`, `ngen` generations, pmut 0.01, pcross 0.6), its (tile height,
 * steps) pick mapped onto this library's schedule. Host only. */
PSKEL_API pskel_status pskel_ga_schedule2d(const pskel_stencil* st, int64_t width, int64_t height, int64_t iterations,
                                           uint64_t seed, int32_t popsize, int32_t ngen, pskel_schedule* out,
                                           double* score);

/* The 11 cost-model input features of one (grid, schedule): log2 width,
 * log2 height, log2 iterations, steps per pass / 8, tall-tile flag, bytes per
 * cell / 4, op, log2 passes, log2 of the redundant-halo factor (loaded tile
 * area / core tile area), log2 tiles per pass, log2 cell updates including
 * the redundant ones. Writes 11 floats and returns 11. Host only. */
PSKEL_API int32_t pskel_schedule_features2d(const pskel_stencil* st, int64_t width, int64_t height,
                                            int64_t iterations, const pskel_schedule* s, float* out);

/* The schedule runIterativeAutoGPU uses: the candidate with the lowest time
 * predicted by the registered cost model (pskel_set_cost_model, or the file
 * named by the PSKEL_COST_MODEL environment variable), else the default. */
PSKEL_API pskel_status pskel_auto_schedule2d(const pskel_stencil* st, int64_t width, int64_t height,
                                             int64_t iterations, pskel_schedule* out);

/* ------------------------------------------------------------- cost model
 * A small MLP (dense tanh layers, linear output) trained and evaluated by this
 * library's CUDA kernels (forward, backward, Adam; full-batch MSE). */
typedef struct pskel_mlp pskel_mlp;
PSKEL_API pskel_status pskel_mlp_create(int32_t in_dim, int32_t hidden, int32_t layers, uint64_t seed,
                                        pskel_mlp** out);
PSKEL_API int64_t pskel_mlp_num_params(const pskel_mlp* m);
PSKEL_API void pskel_mlp_shape(const pskel_mlp* m, int32_t* in_dim, int32_t* hidden, int32_t* layers);
PSKEL_API pskel_status pskel_mlp_get_params(const pskel_mlp* m, float* host);
PSKEL_API pskel_status pskel_mlp_set_params(pskel_mlp* m, const float* host);
/* y[n] = model(x[n][in_dim]) (host arrays) */
PSKEL_API pskel_status pskel_mlp_predict(pskel_mlp* m, const float* x_host, int32_t n, float* y_host);
/* gradient of mean((model(x) - y)^2) w.r.t. the parameters, and that loss */
PSKEL_API pskel_status pskel_mlp_gradient(pskel_mlp* m, const float* x_host, const float* y_host, int32_t n,
                                          float* grads_host, float* loss);
/* `epochs` full-batch Adam steps with learning rate lr; final loss */
PSKEL_API pskel_status pskel_mlp_train(pskel_mlp* m, const float* x_host, const float* y_host, int32_t n,
                                       int32_t epochs, float lr, float* final_loss);
PSKEL_API pskel_status pskel_mlp_save(const pskel_mlp* m, const char* path);
PSKEL_API pskel_status pskel_mlp_load(const char* path, pskel_mlp** out);
PSKEL_API pskel_status pskel_mlp_destroy(pskel_mlp* m);
/* Registers the model pskel_auto_schedule2d uses (NULL: the default schedule). */
PSKEL_API pskel_status pskel_set_cost_model(pskel_mlp* m);

/* Self-test of the kernels' bounded waits (no counterpart in the reference):
 * launches a kernel that waits on an mbarrier phase that never completes
 * (which = 0) or on a device flag that nothing sets (which = 1) for at most
 * `polls` polls (1..2^20), then records the timeout in the device error word
 * and returns; which = 2 launches the persistent Life kernel at pass 1 of a
 * run whose pass 0 never ran, with a dependency-wait limit of `polls`, so its
 * own wait runs out and its blocks stop; which = 3 does the same with the
 * persistent multi-pass 2D kernel (a Jacobi run whose first pass is skipped). The next pskel_sync(stream) reports
 * PSKEL_ERR_DEVICE (and clears it); the context stays usable. */
PSKEL_API pskel_status pskel_selftest_bounded_wait(int32_t which, uint32_t polls, void* stream);

/* pskel_iterate3d without any allocation by the library. It has no
 * counterpart in the reference: it serves callers that cannot let a library
 * call cudaMalloc, such as a host application that owns all device memory
 * through its own pool, or a latency-critical loop that cannot absorb
 * cudaMalloc's implicit synchronisation. The residual scratch and the device
 * error word live in file-scope device arrays of fixed size, held by every GPU
 * that loads the library until the process exits: at most 16384 fp64 partial
 * sums (time_steps x CTAs of one pass); larger schedules are rejected with
 * PSKEL_ERR_UNSUPPORTED (lower schedule.ctas or time_steps). The first call on
 * a device looks up the arrays' device addresses; make that first call before
 * any stream capture. All calls on a device share its arrays and the arrays
 * keep the last call's contents: calls that overlap on the GPU (for example on
 * two streams of one device) race. Every pass rewrites all the partials it
 * reads, and a reported error word is cleared, so nothing else needs clearing. The
 * caller passes the grids and the residual output, as for pskel_iterate3d.
 * Synchronous: it waits for `stream` and reports kernel-side errors. */
PSKEL_API pskel_status pskel_iterate3d_noalloc(const pskel_stencil* st, void* in, void* out, int64_t width,
                                               int64_t height, int64_t depth, int64_t iterations,
                                               const pskel_schedule* sched, int64_t residual_every,
                                               double* residuals, void* stream);

#ifdef __cplusplus
}
#endif

#endif /* PSKEL_GB300_H */
