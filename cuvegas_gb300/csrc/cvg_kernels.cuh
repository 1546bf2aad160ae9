// cvg_kernels.cuh -- argument blocks and launch wrappers of the precompiled
// reallocation (K3) and grid-refinement (K4) kernels.
#ifndef CVG_KERNELS_CUH
#define CVG_KERNELS_CUH

#include <cuda_runtime.h>
#include "cvg_common.cuh"

// Per-iteration statistics kept on the device (no host sync per iteration).
// stats[0..max_it)        : I_it   (sum of per-cube estimates)
// stats[max_it..2*max_it) : sigma2_it (sum of per-cube variances / nh)
// stats[2*max_it..3*max_it): samples of iteration it
// acc                     : running sums of the weighted mean
struct cvg_acc_dev {
    double sw;        // sum 1/sigma2
    double swr;       // sum I/sigma2
    double swr2;      // sum I^2/sigma2
    double dh_sum;    // sum of damped cube variances of the last iteration
    double nh_scale;  // n_eval_it / dh_sum (FP32 form's reallocation)
    cvg_u64 used;     // iterations in the mean
    cvg_u64 tot_nevals;
    cvg_u64 last_nevals;
};

struct cvg_realloc_args {
    cvg_u64 *nh_sum;        // [n_cubes+1], read (old), rewritten (new)
    double *JF, *JF2;       // [n_cubes], read then zeroed
    double *dh;             // [n_cubes]
    cvg_u32 *nh_new;        // [n_cubes]
    double *partials;       // [n_blocks][4]
    cvg_u64 *bsums;         // [n_blocks]
    cvg_u32 *tile_cube;     // [max_tiles]
    double *stats;          // [2*max_it]
    cvg_acc_dev *acc;
    cvg_u32 *iteration;
    cvg_u32 *status;
    int *scale_exp;         // FP32 form: scale exponent k of the fill (updated here); may be null
    cvg_u32 *done;          // [2] block tickets (zero between launches): the last block of
                            // the results / count kernels also runs the finish / scan step
    cvg_u64 max_tiles;
    cvg_i64 n_eval_it;
    double v_cubes;
    double beta;
    cvg_u32 n_cubes;
    int tile_samples;
    int skip;
    int max_it;
    int fast_pow;           // 1: FP32 form (compensated FP32 per cube, FP64 sums); d_h is
                            //    then (var)^beta without the cube-volume factor V^(2 beta)
    int adapt;              // 0: keep nh (no reallocation), still accumulate results
    cvg_u32 *hist_state;    // FP32 form: the fill's histogram form (see cvg_fill_args), chosen
                            // here for the next fill; or null
    int dim;
    int rare_shift;         // fixed point stays while rare updates <= dim*samples / 2^rare_shift
    int hist_min_it;        // first iteration that may use fixed point again after iteration 0
    cvg_u64 *lb;            // [n_blocks] look-back words of the one-pass allocation, or null
                            // (three-kernel path); zero before the first launch
    cvg_u32 *lb_ctl;        // [2]: block ticket (zero between launches), launch epoch
    int small_chunks;       // 1: up to CVG_REALLOC_SMALL_CUBES hypercubes, the results kernel
                            // takes 2 per thread (partials must hold 4x the blocks)
    int lb_spin_limit;      // polls of a look-back word before the wait gives up and sets
                            // CVG_KSTAT_TIMEOUT; 0 = the default (2^22)
    cvg_u32 lb_withhold;    // failure test only: 1 + the chunk whose look-back word is never
                            // published (its successors' waits then run out); 0 = none
    double *exp_dq;         // batched FP32 form: sum over hypercubes of d_h * (JF2/n) 2^-2k,
                            // 2^-64 (the results blocks add, the finish reads and clears), or null
    int *exp_shift;         // batched FP32 form: the next fill's exponent shift (cvg_fill_args),
                            // set by the finish; or null
};

struct cvg_refine_args {
    double *x_edges;        // [dim][N+1]
    float *x_edges32;       // [dim][N+1]
    double *weights;        // [dim][N], read then zeroed
    cvg_u32 *counts;        // [dim][N], read then zeroed
    int *bin_exp;           // FP32 form: [dim][N+...] per-bin exponents for the next fill
                            // (written), [dim*N] = scale exponent of the fill (read); or null
    double alpha;
    int dim;
    int n_intervals;
    int adapt;              // 0: only clear the histograms
};

enum { CVG_REALLOC_CHUNK = 2048, CVG_REFINE_BLOCK = 1024, CVG_REFINE_MAX_N = 4096,
       CVG_REALLOC_SMALL_CUBES = 1 << 19 };

// Device tables of a batch of instances (one launch covers all of them).
struct cvg_realloc_batch {
    const cvg_realloc_args *A;    // [n]
    const unsigned *blk_base;     // [n+1] prefix of reallocation blocks
    const unsigned *blk_inst;     // [total_blocks] instance of each block
    unsigned total_blocks;
    int n;
};
struct cvg_refine_batch {
    const cvg_refine_args *R;     // [n]
    const unsigned *dim_base;     // [n+1] prefix of dimensions
    unsigned total_dims;
    int n;
    int keep_grid;                // 1: every instance as with adapt = 0
};

__host__ __device__ inline unsigned cvg_realloc_blocks(cvg_u32 n_cubes)
{
    return (unsigned)((n_cubes + CVG_REALLOC_CHUNK - 1) / CVG_REALLOC_CHUNK);
}

// Launch the reallocation chain (results, finish, count, scan, apply).
cudaError_t cvg_launch_realloc(const cvg_realloc_args &a, cudaStream_t s);
// Scale exponent k of the FP32 reallocation from caller-given per-cube sums:
// 2^k near the rms of f*jac, i.e. 2^(2k) ~ sum JF2 / total samples (the rule
// k3_finish applies after every iteration).  ss (one double) and ticket (one
// word) must be zero; both are left zero.
cudaError_t cvg_launch_scale_from_sums(const double *JF2, const cvg_u64 *nh_sum, cvg_u32 n_cubes,
                                       double *ss, cvg_u32 *ticket, int *scale_exp, cudaStream_t s);
// Launch the refinement (one CTA per dimension).
cudaError_t cvg_launch_refine(const cvg_refine_args &a, cudaStream_t s);
// Tile map + prefix from an explicit nh (state import / initialisation).
cudaError_t cvg_launch_set_nh(const cvg_realloc_args &a, const cvg_u32 *nh, cudaStream_t s);
// FP32 copy of the grid.
cudaError_t cvg_launch_grid32(const double *x, float *x32, int n, cudaStream_t s);
// Peak-throughput microbenchmarks (FP32 / FP64 FMA chains, device copy).
cudaError_t cvg_launch_fma_bench(int kind, int blocks, int iters, double *sink, cudaStream_t s);
cudaError_t cvg_launch_copy_bench(const float4 *src, float4 *dst, size_t n, cudaStream_t s);
cudaError_t cvg_launch_smem_atomic_bench(int kind, int blocks, int iters, double *sink,
                                         cudaStream_t s);
// mode 0: float atomic + count, 1: u32 fixed point with carry + count (gw: 4096 doubles)
cudaError_t cvg_launch_hist_update_bench(int mode, int blocks, int iters, double *gw, cudaStream_t s);
// kind 0: INT32 multiply-add, 1: ex2.approx, 2: Philox4x32-10 (4 calls per iteration)
cudaError_t cvg_launch_pipe_bench(int kind, int blocks, int iters, double *sink, cudaStream_t s);
// Fill n words with a value.
cudaError_t cvg_launch_fill_u32(cvg_u32 *p, cvg_u32 v, cvg_u64 n, cudaStream_t s);

// Batched reallocation (+ the tile numbering of the next batched fill).
// Work split of the next batched fill, written after each reallocation.
struct cvg_batch_sched {
    cvg_u64 *tile_base;           // [n+1] first global tile of each instance
    cvg_u64 *cost_base;           // [n+1] cost-weighted prefix of the tiles
    cvg_u64 *range_start;         // [n_ranges+1] first tile of each CTA's range
    cvg_u32 *range_inst;          // [n_ranges] instance of range_start (or one before it)
    cvg_u64 *claim;               // [n_ranges] claim counters, zeroed here
    int n_ranges;
};
cudaError_t cvg_launch_realloc_batch(const cvg_realloc_batch &B, int adapt, bool fast,
                                     const cvg_batch_sched &S, cudaStream_t s);
cudaError_t cvg_launch_set_nh_batch(const cvg_realloc_batch &B, const cvg_batch_sched &S,
                                    cudaStream_t s);
cudaError_t cvg_launch_refine_batch(const cvg_refine_batch &B, int n_intervals, cudaStream_t s);

// Set the calling thread's cvg_last_error() message (host code of the library).
void cvg_internal_set_error(const char *msg);

#endif
