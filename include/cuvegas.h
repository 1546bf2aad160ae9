/*
 * cuvegas.h -- C ABI of the GB300-native VEGAS+ integrator (libcuvegas.so).
 *
 * Plain pointers, sizes and status codes; no C++ or PyTorch types.  One
 * process, one GPU.  Each entry point names the reference interface it
 * replaces (paths relative to the emiliantolo/cuvegas project root).
 *
 * Threading: a cvg_context and everything created from it may be used by one
 * host thread at a time.  Errors never terminate the process (the reference
 * calls exit(), src/commons/common.cuh:39-45); they return a status and leave
 * a message readable with cvg_last_error() on the calling thread.
 */
#ifndef CUVEGAS_H
#define CUVEGAS_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef enum {
    CVG_OK = 0,
    CVG_ERR_INVALID = 1,    /* bad argument or size                         */
    CVG_ERR_CUDA = 2,       /* CUDA runtime error                           */
    CVG_ERR_COMPILE = 3,    /* NVRTC could not compile the integrand source */
    CVG_ERR_NOMEM = 4,      /* device or host allocation failed             */
    CVG_ERR_KERNEL = 5,     /* a kernel reported an inconsistent state      */
    CVG_ERR_STATE = 6       /* call out of order (e.g. past max_it)         */
} cvg_status;

enum { CVG_PREC_FP64 = 0, CVG_PREC_FP32 = 1 };

/* Integrand source conventions (cvg_compile_integrand `abi`). */
enum {
    CVG_ABI_NATIVE = 0,     /* T integrand(T* x) [, const T* theta]; T = double or float   */
    CVG_ABI_NUMBA = 1       /* int integrand(double* ret, double* x): the device ABI the
                               reference links (vegas_cuda_extension/cuda_kernel.cu:7) */
};

/* cvg_params.flags */
enum {
    CVG_FLAG_GRAPH = 1,     /* capture one iteration as a CUDA graph and replay it       */
    CVG_FLAG_NO_ADAPT = 2,  /* keep grid and nh fixed (evaluation with a trained map)    */
    CVG_FLAG_TIME_FILL = 4  /* time every fill launch with CUDA events (eager iterations)  */
};

/* Run parameters.  Meanings follow the reference: src/config.cuh:7-26 and
 * vegas_cuda/src/vegas_cuda_extension/python_wrapper.py:9. */
typedef struct {
    int64_t tot_eval;        /* total evaluations over all iterations (tot_eval / n_evals)    */
    int32_t max_it;          /* iterations                                                   */
    int32_t skip;            /* iterations left out of the weighted mean                     */
    int64_t max_batch_size;  /* accepted for compatibility; the fill is persistent           */
    int32_t n_intervals;     /* bins per dimension of the adaptive grid (nbins)              */
    int32_t n_strat;         /* strata per dimension; 0 = (int)pow(N_it/4, 1/dim)            */
    int32_t n_dim;           /* dimension (must equal the compiled integrand's)              */
    int32_t precision;       /* CVG_PREC_FP64 (plain) or CVG_PREC_FP32 (compensated)         */
    double alpha;            /* grid damping                                                 */
    double beta;             /* stratification damping                                       */
    uint64_t seed;           /* Philox key                                                   */
    double gpu_thr;          /* accepted for compatibility; no CPU mapping fallback exists   */
    int32_t flags;           /* CVG_FLAG_*                                                   */
    int32_t block;           /* fill threads per CTA; 0 = tuned default                      */
    int32_t spt;             /* fill samples per thread; 0 = tuned default                   */
    uint32_t instance;       /* Philox stream id (independent integrals)                     */
} cvg_params;

/* Result record.  First fields mirror the 14-tuple of the reference's
 * integrate_cuda (vegas_cuda/src/vegas_cuda_extension/cuda_wrapper.cu:869). */
typedef struct {
    double result;           /* weighted mean over iterations >= skip                        */
    double error;            /* 1/sqrt(sum 1/sigma^2)                                        */
    int32_t n_strat;
    int32_t n_intervals;
    int64_t n_cubes;
    int64_t tot_nevals;      /* integrand evaluations over all iterations                    */
    double tot_time_ms;      /* wall time of the call                                        */
    double avg_it_time_ms;   /* iteration-loop wall time / iterations                        */
    uint64_t seed;
    double gpu_thr;
    double chi2_dof;         /* chi^2 per degree of freedom of the iteration estimates       */
    int32_t n_it_used;
    int32_t n_it_done;
    int32_t precision;
    int32_t pad;
} cvg_result;

typedef struct cvg_context_s *cvg_context;
typedef struct cvg_integrand_s *cvg_integrand;
typedef struct cvg_run_s *cvg_run;

/* Message of the last failing call on this thread ("" if none). */
const char *cvg_last_error(void);
/* Library version string. */
const char *cvg_version(void);

/* Context on `device` (replaces the per-call device setup of
 * cuda_wrapper.cu:292-329).  `stream` may be NULL (the context creates one)
 * or a cudaStream_t owned by the caller. */
cvg_status cvg_context_create(int device, void *stream, cvg_context *out);
cvg_status cvg_context_destroy(cvg_context ctx);
/* Free the device arenas the context keeps from destroyed runs and batches
 * for reuse (the cache holds up to CVG_ARENA_CACHE_MB, default 1/8 of the
 * device; no counterpart in the reference, which allocates and frees every
 * buffer inside each call, cuda_wrapper.cu:392-451, 779-851). */
cvg_status cvg_context_trim(cvg_context ctx);

/* JIT-compile an integrand from CUDA C++ source (replaces numba PTX + the
 * cuLink step, python_wrapper.py:48-61 and cuda_wrapper.cu:221-286).  The
 * source defines `integrand` per `abi`; `n_params` > 0 means it also takes a
 * `const T* theta`; `has_grad` means it defines
 * `void integrand_grad(T* x, const T* theta, T* g)` (dF/dtheta).  Kernels are
 * compiled lazily per (precision, tile shape) and cached. */
cvg_status cvg_compile_integrand(cvg_context ctx, const char *source, int32_t n_dim,
                                 int32_t abi, int32_t n_params, int32_t has_grad,
                                 cvg_integrand *out);
/* Integrand given as PTX (numba's ABI, the device ABI the reference links:
 * a function `integrand` with `int integrand(double* ret, double* x)`,
 * vegas_cuda/src/vegas_cuda_extension/cuda_kernel.cu:7 and python_wrapper.py:48-59,
 * e.g. numba.cuda.compile(..., abi="numba", abi_info={"abi_name": "integrand"})).
 * `source` (may be NULL) is CUDA C++ compiled with the fill; when given it
 * must declare or wrap `extern "C" __device__ int integrand(double*, double*)`.
 * Each fill module is compiled relocatable and linked with the PTX (nvJitLink).
 * FP64 form only. */
cvg_status cvg_compile_integrand_ptx(cvg_context ctx, const char *source, const char *ptx,
                                     int32_t n_dim, cvg_integrand *out);
cvg_status cvg_integrand_release(cvg_integrand f);

/* Whole integration, the drop-in for integrate_cuda
 * (cuda_wrapper.cu:290-872): host parameters in, host result out.
 * `theta` (host, n_params doubles) may be NULL when n_params == 0.
 * it_res / it_sig2 (host, max_it doubles each) may be NULL. */
cvg_status cvg_integrate(cvg_context ctx, cvg_integrand f, const cvg_params *p,
                         const double *theta, cvg_result *out, double *it_res,
                         double *it_sig2);

/* ---- step-level API (persistent device state; tests, benchmarks, autograd) ---- */

cvg_status cvg_run_create(cvg_context ctx, cvg_integrand f, const cvg_params *p,
                          const double *theta, cvg_run *out);
cvg_status cvg_run_destroy(cvg_run r);
/* Enqueue n full iterations (fill, reallocation, refinement) on the context
 * stream; no host synchronisation. */
cvg_status cvg_run_iterate(cvg_run r, int32_t n);
/* Stages of one iteration, for step-by-step checks. */
enum { CVG_STAGE_FILL = 1, CVG_STAGE_REALLOC = 2, CVG_STAGE_REFINE = 4 };
cvg_status cvg_run_step(cvg_run r, int32_t stages);
/* Synchronise and summarise the iterations done so far. */
cvg_status cvg_run_result(cvg_run r, cvg_result *out, double *it_res, double *it_sig2);
cvg_status cvg_run_sync(cvg_run r);

/* Buffers readable / writable through cvg_run_get / cvg_run_set (host side). */
enum {
    CVG_BUF_X_EDGES = 0,     /* double [dim][N+1]        get/set                  */
    CVG_BUF_NH = 1,          /* uint32 [n_cubes]         get/set (set rebuilds the prefix) */
    CVG_BUF_NH_SUM = 2,      /* uint64 [n_cubes+1]       get                      */
    CVG_BUF_JF = 3,          /* double [n_cubes]         get/set                  */
    CVG_BUF_JF2 = 4,         /* double [n_cubes]         get/set                  */
    CVG_BUF_WEIGHTS = 5,     /* double [dim][N]          get/set                  */
    CVG_BUF_COUNTS = 6,      /* uint32 [dim][N]          get/set                  */
    CVG_BUF_DH = 7,          /* double [n_cubes]         get (FP32 form: kept as float,
                                widened on the way out)                               */
    CVG_BUF_THETA = 8,       /* double [n_params]        get/set                  */
    CVG_BUF_ITERATION = 9,   /* uint32 [1]               get/set (set: the loop continues from
                                this iteration; Philox counter word 2)                  */
    CVG_BUF_UNIFORMS = 10,   /* float  [S][dim]          set: replay these uniforms in
                                the next fills instead of Philox (parity tests); 0 bytes
                                switches back                                         */
    CVG_BUF_STATS = 11,      /* double [3][max_it]       get/set: I_it, sigma2_it, samples_it */
    CVG_BUF_SCALE_EXP = 12,  /* int32  [1]               get/set: FP32 form carries f*jac
                                scaled by 2^-k (k chosen by a pilot, then updated each
                                iteration) so (f*jac)^2 stays in float range             */
    CVG_BUF_BIN_EXP = 13,    /* int32  [dim*N+1]         get/set: FP32 form, binary exponent of
                                each bin's expected per-sample (f*jac)^2 for the next fill
                                (unscaled; set by the pilot, then by each refinement); the
                                last entry is the k of the last fill                      */
    CVG_BUF_HIST_STATE = 14, /* uint32 [2]               get/set: FP32 form, [0] 1 = the next
                                fill keeps its bin sums in fixed point (chosen after each
                                iteration from [1], the rare updates the fill counted)    */
    CVG_BUF_TILE_CUBE = 15   /* uint32 [max_tiles]       get: the hypercube of each fill tile's
                                first sample (tiles of tile_samples; entries past the next
                                fill's last tile are stale)                                */
};
cvg_status cvg_run_get(cvg_run r, int32_t buf, void *host, size_t bytes);
cvg_status cvg_run_set(cvg_run r, int32_t buf, const void *host, size_t bytes);

/* ---- sample split of one integral across ranks (one GPU per rank) ----
 * Replaces the reference's multi-GPU iteration (src/main.cu:591-654 and
 * vegas_cuda/src/vegas_cuda_extension/cuda_wrapper.cu:646-706): each GPU
 * fills its share of the iteration's samples, the per-cube and per-bin sums
 * are added across GPUs, and every GPU then holds the same sums.  Here each
 * rank creates the same run (same parameters, seed and instance) and calls
 * cvg_run_set_shard(r, rank, world): its fills then cover tiles
 * [T*rank/world, T*(rank+1)/world) of the iteration's T tiles, a contiguous
 * range of the samples in hypercube order.  The Philox counter names each
 * sample by (sample-in-cube, cube, iteration), so the union of the ranks'
 * fills is exactly the one-rank fill.  Per iteration: cvg_run_step(FILL);
 * sum JF, JF2, WEIGHTS and COUNTS (and, in the FP32 form, HIST_STATE word
 * [1]) over the ranks with any all-reduce (NCCL on the device views below,
 * or host copies); cvg_run_step(REALLOC | REFINE), which every rank then
 * computes identically (the reference broadcasts rank 0's grid instead,
 * src/main.cu:531-541).  The gradient pass always covers every sample.
 * Set the shard before the first graph iteration. */
cvg_status cvg_run_set_shard(cvg_run r, int32_t shard, int32_t shards);
/* Device address and size of one of the run's buffers (CVG_BUF_X_EDGES,
 * NH_SUM, JF, JF2, WEIGHTS, COUNTS, HIST_STATE), for collectives issued by
 * the caller on the context's stream.  The address stays valid until
 * cvg_run_destroy.  No counterpart in the reference (its buffers are local
 * to integrate_cuda). */
cvg_status cvg_run_buffer(cvg_run r, int32_t buf, void **device_ptr, size_t *bytes);

/* Sizes of the run: n_cubes, n_strat, samples of the next fill, tile shape. */
typedef struct {
    int64_t n_eval_it, n_cubes, next_samples, max_tiles;
    int32_t n_strat, n_intervals, n_dim, block, spt, grid, edges_smem, hist_smem;
    double v_cubes;
    int64_t fill_smem_bytes;
    int32_t tile_samples;  /* samples per fill tile: 32*spt (warp tiles) or block*spt */
    int32_t warp_tiles;    /* 1: each warp claims its own tiles; 0: the CTA shares one */
} cvg_run_info;
cvg_status cvg_run_info_get(cvg_run r, cvg_run_info *out);

/* Backward: dI_it/dtheta of one iteration with that iteration's grid and nh
 * (the current state of the run) held fixed and the same Philox samples as
 * its fill (iteration counter `it`).  grad: host, n_params doubles. */
cvg_status cvg_run_grad(cvg_run r, uint32_t it, double *grad);

/* Compile the fill kernel (and the gradient kernel when has_grad) for
 * `source` with NVRTC only -- no GPU needed -- for build checks.  `arch` such
 * as "sm_103a"; `log` (may be NULL) receives the NVRTC log. */
cvg_status cvg_compile_check(const char *source, int32_t n_dim, int32_t abi, int32_t n_params,
                             int32_t has_grad, int32_t precision, const char *arch, char *log,
                             size_t log_len);

/* Device timing of the last fill launch (CUDA events on the launch stream). */
cvg_status cvg_run_last_fill_ms(cvg_run r, float *ms);
/* Durations (ms) of the fill launches timed since the previous call
 * (CVG_FLAG_TIME_FILL); synchronises.  At most `cap` values; *n = count. */
cvg_status cvg_run_fill_times(cvg_run r, float *ms, int32_t cap, int32_t *n);

/* ---- batched integration ---- */

typedef struct cvg_batch_s *cvg_batch;

/* One integral of a batch. */
typedef struct {
    int32_t n_dim;        /* 1..16                                                  */
    int32_t n_strat;      /* 0 = (int)pow(evals per iteration / 4, 1/n_dim)         */
    int64_t tot_eval;     /* evaluations over all iterations (common max_it)        */
    uint32_t instance;    /* Philox stream id: equal to a single run with the same id */
    int32_t pad;
} cvg_instance;

/* Many independent integrals of one integrand family (one source; parameters
 * per instance) with different dimensions and evaluation counts, advanced
 * together: per iteration one persistent fill launch for the whole batch,
 * batched grid refinement and batched reallocation; with CVG_FLAG_GRAPH the
 * iteration is one CUDA-graph launch.  No counterpart in the reference (it
 * integrates one function per call, cuda_wrapper.cu:290).
 * params_per_dim[d] (d = 0..16) = parameters of the dimension-d integrand;
 * theta = the instances' parameters back to back.  `common` supplies max_it,
 * skip, n_intervals, alpha, beta, seed, precision, flags, block, spt. */
cvg_status cvg_batch_create(cvg_context ctx, const char *source, int32_t abi, int32_t n,
                            const cvg_instance *inst, const int32_t *params_per_dim,
                            const double *theta, const cvg_params *common, cvg_batch *out);
cvg_status cvg_batch_destroy(cvg_batch b);
/* Enqueue n iterations of every instance (no host synchronisation). */
cvg_status cvg_batch_iterate(cvg_batch b, int32_t n);
/* Synchronise; out[n], it_res / it_sig2 [n][max_it] (may be NULL). */
cvg_status cvg_batch_results(cvg_batch b, cvg_result *out, double *it_res, double *it_sig2);
/* Launch shape and the samples of the next batched fill (synchronises). */
cvg_status cvg_batch_info_get(cvg_batch b, int32_t *block, int32_t *spt, int32_t *grid,
                              int64_t *fill_smem_bytes, int64_t *next_samples);
/* Device time of the last timed batched fill (eager iterations). */
cvg_status cvg_batch_last_fill_ms(cvg_batch b, float *ms);
/* NVRTC-only compile of the batched kernels for the given dimensions (no GPU
 * needed), for build checks; `log` (may be NULL) receives the NVRTC log. */
cvg_status cvg_batch_compile_check(const char *source, int32_t n_dims, const int32_t *dims,
                                   const int32_t *params_per_dim, int32_t precision,
                                   int32_t block, const char *arch, char *log, size_t log_len);

/* ---- reallocation without allocation ----
 * For callers that cannot call cudaMalloc (code running inside another
 * framework's memory pool, or with all device memory reserved up front).
 * No counterpart in the reference: it allocates inside every call.
 *
 * Runs the same reallocation kernels as the iteration loop on caller-owned
 * device buffers: JF/JF2 [n_cubes] (the fill's per-hypercube sums; read, then
 * cleared to zero), nh_sum [n_cubes+1] (in: the exclusive prefix of the
 * current per-cube sample counts; out: the reallocated prefix), est [3]
 * (out: I, sigma^2 and samples of the iteration), and optionally tile_cube
 * [max_tiles] (out: the cube of each tile's first sample, tiles of
 * tile_samples; NULL skips it).  All temporaries live in one statically
 * allocated __device__ array (about 3 MiB per GPU that loads the library,
 * held until exit): n_cubes may not exceed CVG_NOALLOC_MAX_CUBES; larger
 * calls are rejected, and so are n_eval_it < 1 and n_eval_it + 2*n_cubes at
 * or above 2^31 - 2^20 (the bound of cvg_run_create).  Calls share that
 * array, so calls that overlap on the GPU race.  The first call on a device
 * looks up the array's address; make that first call before any stream
 * capture.  Calls no cudaMalloc or cudaFree.  precision: CVG_PREC_FP64
 * (reference arithmetic) or CVG_PREC_FP32 (compensated FP32 per cube, on the
 * sums scaled by a power of two worked out on the device from JF2, so sums of
 * any magnitude in double range are taken).  The call waits for its kernels
 * (it synchronises `stream`) and returns CVG_ERR_KERNEL when they report a
 * non-finite estimate or variance, or an inconsistent state.  stream may be
 * NULL. */
#define CVG_NOALLOC_MAX_CUBES 262144
cvg_status cvg_realloc_noalloc(double *JF, double *JF2, uint64_t *nh_sum, uint32_t n_cubes,
                               double v_cubes, double beta, int64_t n_eval_it, int32_t precision,
                               double *est, uint32_t *tile_cube, uint64_t max_tiles,
                               int32_t tile_samples, void *stream);

/* Throughput microbenchmark of this device: kind 0 = FP32 FMA, 1 = FP64 FMA
 * (TFLOP/s, 2 flops per FMA), 2 = device-memory copy (GB/s, read+write),
 * 3..6 = shared-memory atomic adds to random words of a 4096-word table,
 * float / u32 / u64 / double (G atomics/s), 7 = INT32 multiply-add (T ops/s),
 * 8 = ex2.approx (T ops/s), 9 = Philox4x32-10 (T calls/s), 10/11 = the fill's
 * per-bin histogram update with a float atomic / with the u32 fixed-point
 * atomic, each with its count atomic (G updates/s). */
cvg_status cvg_measure_peak(cvg_context ctx, int32_t kind, double *out);

#ifdef __cplusplus
}
#endif
#endif
