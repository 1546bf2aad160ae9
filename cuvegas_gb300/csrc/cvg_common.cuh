// cvg_common.cuh -- types and device helpers shared by the NVRTC-compiled
// fill kernels, the precompiled reallocation/refinement kernels and the host
// driver.  Self-contained (no includes) so NVRTC can compile it as-is.
#ifndef CVG_COMMON_CUH
#define CVG_COMMON_CUH

typedef unsigned int cvg_u32;
typedef unsigned long long cvg_u64;
typedef long long cvg_i64;

#if defined(__CUDACC__) || defined(__CUDACC_RTC__)
#define CVG_HD __host__ __device__ __forceinline__
#define CVG_D __device__ __forceinline__
#else
#define CVG_HD inline
#endif

// Status bits written by kernels into the run's status word.
#define CVG_KSTAT_BAD_TILE 1u      // tile map inconsistent with nh_sum
#define CVG_KSTAT_NONFINITE 2u     // a non-finite per-cube estimate was seen
#define CVG_KSTAT_TIMEOUT 4u       // a bounded wait ran out (the results are not valid)
// Samples a CTA adds to its shared-memory bin histograms between flushes
// (bin counts stay below 2^24)
#define CVG_HIST_MAX_RUN 0x00FFF000u

// Philox4x32-10 key schedule of one seed: round r uses (k0 + r*0x9E3779B9,
// k1 + r*0xBB67AE85).  Kept in the kernel arguments (constant bank), so the
// rounds read their key words directly instead of recomputing them per call.
struct cvg_philox_keys { cvg_u32 k[2][10]; };
CVG_HD void cvg_philox_schedule(cvg_u64 seed, cvg_philox_keys &ks)
{
    for (int r = 0; r < 10; ++r) {
        ks.k[0][r] = (cvg_u32)seed + (cvg_u32)r * 0x9E3779B9u;
        ks.k[1][r] = (cvg_u32)(seed >> 32) + (cvg_u32)r * 0xBB67AE85u;
    }
}

// Arguments of one fill launch.  Layout is shared between host and device;
// only fixed-width scalar types and pointers.
struct cvg_fill_args {
    const double *x_edges;        // [dim][N+1] FP64 grid
    const float *x_edges32;       // [dim][N+1] FP32 copy of the grid
    const cvg_u64 *nh_sum;        // [n_cubes+1] exclusive prefix of samples per cube
    const cvg_u32 *tile_cube;     // [max_tiles] cube holding the first sample of each tile
    const cvg_u32 *iteration;     // device iteration counter (Philox counter word 2)
    const float *ubuf;            // replay uniforms [S][dim] (test path), else null
    const double *theta;          // integrand parameters [n_params], or null
    double *JF;                   // [n_cubes] sum of f*jac per cube
    double *JF2;                  // [n_cubes] sum of (f*jac)^2 per cube
    double *weights;              // [dim][N] sum of (f*jac)^2 per bin
    cvg_u32 *counts;              // [dim][N] samples per bin
    double *grad;                 // [n_params] dI/dtheta accumulator (gradient pass)
    cvg_u32 *status;              // error bits
    cvg_u32 *tile_ctl;            // warp tiles: [0] next tile to claim, [1] CTAs done (zero
                                  // between launches: the last CTA of a launch resets both)
    int *scale_exp;               // FP32 form: f*jac is scaled by 2^-scale_exp (may be null)
    double *scale_ss;             // FP32-form pilot: sum of (f*jac)^2 over its samples
    cvg_u32 *hist_state;          // FP32 form: [0] 1 = fixed-point bin sums in this fill,
                                  // [1] rare updates the fill counts (or null)
    int *bin_exp;                 // FP32 form: [dim][N] binary exponent of each bin's expected
                                  // per-sample (f*jac)^2 (unscaled); [dim*N] = the scale
                                  // exponent k of the last fill (null for FP64)
    const int *exp_shift;         // batched FP32 fills: bits added to every bin's exponent, the
                                  // predicted rise of the per-sample (f*jac)^2 after the last
                                  // reallocation (null: none)
    cvg_u64 max_tiles;            // capacity of tile_cube
    cvg_u64 seed;                 // Philox key
    cvg_u32 instance;             // Philox counter word 3, bits 8..31
    cvg_u32 n_cubes;
    int n_strat;
    int n_intervals;
    int tile_samples;             // samples per tile: 32 * spt (warp tiles) or blockDim.x * spt
    int spt;                      // consecutive samples per thread
    int n_params;
    cvg_u32 shard;                // sample split across ranks: this fill covers tiles
    cvg_u32 shards;               // [n_tiles*shard/shards, n_tiles*(shard+1)/shards) of the
                                  // iteration (shards 0 or 1: all tiles)
    int pad0;
    double v_cubes;               // volume of one hypercube
    cvg_philox_keys keys;         // key schedule of seed
};

// Arguments of one batched fill launch.
struct cvg_batch_args {
    const cvg_fill_args *inst;    // [n_inst]
    const int *dims;              // [n_inst]
    const cvg_u64 *tile_base;     // [n_inst + 1] first global tile of each instance
    const cvg_u64 *range_start;   // [n_ranges + 1] first global tile of each CTA's range
    const cvg_u32 *range_inst;    // [n_ranges] an instance at or before range_start's tile
    cvg_u64 *claim;               // [n_ranges] tiles claimed from each range (zero at launch)
    int n_inst;
    int n_ranges;                 // = gridDim.x of the fill
    cvg_u32 max_claim;            // tiles one claim may take (its samples < CVG_HIST_MAX_RUN)
    cvg_philox_keys keys;         // key schedule of the common seed
};

CVG_HD cvg_u64 cvg_align16(cvg_u64 x) { return (x + 15ull) & ~15ull; }

// Single-instance fills give each warp its own tiles of 32 * spt samples
// (no block-wide barrier between tiles; warps claim tiles from a counter);
// the batched fill keeps block-wide tiles.
#ifndef CVG_FILL_WARP_TILES
#define CVG_FILL_WARP_TILES 1
#endif

// Dynamic shared memory of one fill launch; the kernel carves it in the same
// order: theta | bin sums | grid | bin counts | cube starts | reduce scratch.
// groups: tiles in flight per CTA (block / 32 with warp tiles, else 1), each
// with its own cube-start buffer.
CVG_HD cvg_u64 cvg_fill_smem_bytes(int dim, int n_intervals, int tsz, int edges_smem,
                                   int hist_smem, int grad, int tile_samples, int n_params,
                                   int block, int groups = 1)
{
    cvg_u64 b = cvg_align16((cvg_u64)n_params * tsz);
    const int h = hist_smem && !grad;
    if (h) b += cvg_align16((cvg_u64)dim * n_intervals * tsz);
    if (edges_smem) b += cvg_align16((cvg_u64)dim * (n_intervals + 1) * tsz);
    if (h) b += cvg_align16((cvg_u64)dim * n_intervals * 4);
    b += cvg_align16((cvg_u64)groups * (tile_samples / 2 + 4) * 4);
    if (grad) b += cvg_align16((cvg_u64)(block / 32) * n_params * 8);
    return b;
}

// ---------------------------------------------------------------------------
// Philox4x32-10 (Salmon et al., SC'11): 10 rounds of two 32x32->64-bit
// multiplies with multipliers 0xD2511F53 / 0xCD9E8D57 and a Weyl key schedule
// (0x9E3779B9, 0xBB67AE85).  Counter = (sample-in-cube, cube, iteration,
// dim-block | instance << 8); key = seed.
// ---------------------------------------------------------------------------
#if defined(__CUDACC__) || defined(__CUDACC_RTC__)
struct cvg_u32x4 { cvg_u32 x, y, z, w; };

CVG_D cvg_u32x4 cvg_philox(cvg_u32 c0, cvg_u32 c1, cvg_u32 c2, cvg_u32 c3, cvg_u32 k0,
                           cvg_u32 k1)
{
#pragma unroll
    for (int r = 0; r < 10; ++r) {
        if (r > 0) { k0 += 0x9E3779B9u; k1 += 0xBB67AE85u; }
        // one 32x32->64 multiply per word pair (high and low halves together)
        const cvg_u64 p0 = (cvg_u64)0xD2511F53u * c0;
        const cvg_u64 p1 = (cvg_u64)0xCD9E8D57u * c2;
        const cvg_u32 n0 = (cvg_u32)(p1 >> 32) ^ c1 ^ k0;
        const cvg_u32 n2 = (cvg_u32)(p0 >> 32) ^ c3 ^ k1;
        c0 = n0; c1 = (cvg_u32)p1; c2 = n2; c3 = (cvg_u32)p0;
    }
    cvg_u32x4 o; o.x = c0; o.y = c1; o.z = c2; o.w = c3;
    return o;
}
// The same with the key schedule precomputed (cvg_philox_schedule).
CVG_D cvg_u32x4 cvg_philox_ks(cvg_u32 c0, cvg_u32 c1, cvg_u32 c2, cvg_u32 c3,
                              const cvg_philox_keys &ks)
{
#pragma unroll
    for (int r = 0; r < 10; ++r) {
        const cvg_u64 p0 = (cvg_u64)0xD2511F53u * c0;
        const cvg_u64 p1 = (cvg_u64)0xCD9E8D57u * c2;
        const cvg_u32 n0 = (cvg_u32)(p1 >> 32) ^ c1 ^ ks.k[0][r];
        const cvg_u32 n2 = (cvg_u32)(p0 >> 32) ^ c3 ^ ks.k[1][r];
        c0 = n0; c1 = (cvg_u32)p1; c2 = n2; c3 = (cvg_u32)p0;
    }
    cvg_u32x4 o; o.x = c0; o.y = c1; o.z = c2; o.w = c3;
    return o;
}

// 32 random bits -> uniform in (0,1).
//  float : (2*(r>>9)+1) * 2^-24, built by exponent splicing (no int->float convert)
//  double: (r + 0.5) * 2^-32, built the same way; both exact.
template <typename T> CVG_D T cvg_uniform(cvg_u32 r);
// FP32: the top 23 bits as the significand of t in [1, 2) (the same bits the
// FP64 uniform starts with, so both forms draw nearly the same points),
// u = t - (1 - 2^-24) = m 2^-23 + 2^-24 (exact), in (0, 1).
CVG_D float cvg_uniform_t(cvg_u32 r) { return __uint_as_float((r >> 9) + 0x3F800000u); }
template <> CVG_D float cvg_uniform<float>(cvg_u32 r)
{
    return cvg_uniform_t(r) - 0.99999994039535522461f;
}
template <> CVG_D double cvg_uniform<double>(cvg_u32 r)
{
    return __hiloint2double((int)(0x3FF00000u | (r >> 12)), (int)(r << 20)) -
           0.99999999988358467817;  // 1 - 2^-33
}

// Packed FP32 pairs (PTX .f32x2, sm_100 and later): one instruction applies
// the same IEEE operation, with the same rounding, to two floats, so two
// dimensions of the FP32 map issue as one instruction stream.  Each half of
// a result equals the scalar operation's result.
typedef unsigned long long cvg_f32x2;
CVG_D cvg_f32x2 cvg_pack2(float lo, float hi)
{
    cvg_f32x2 r;
    asm("mov.b64 %0, {%1, %2};" : "=l"(r) : "f"(lo), "f"(hi));
    return r;
}
CVG_D void cvg_unpack2(cvg_f32x2 r, float &lo, float &hi)
{
    asm("mov.b64 {%0, %1}, %2;" : "=f"(lo), "=f"(hi) : "l"(r));
}
CVG_D cvg_f32x2 cvg_fma2(cvg_f32x2 a, cvg_f32x2 b, cvg_f32x2 c)
{
    cvg_f32x2 d;
    asm("fma.rn.f32x2 %0, %1, %2, %3;" : "=l"(d) : "l"(a), "l"(b), "l"(c));
    return d;
}
CVG_D cvg_f32x2 cvg_add2_rd(cvg_f32x2 a, cvg_f32x2 b)
{
    cvg_f32x2 d;
    asm("add.rm.f32x2 %0, %1, %2;" : "=l"(d) : "l"(a), "l"(b));
    return d;
}
CVG_D cvg_f32x2 cvg_add2(cvg_f32x2 a, cvg_f32x2 b)
{
    cvg_f32x2 d;
    asm("add.rn.f32x2 %0, %1, %2;" : "=l"(d) : "l"(a), "l"(b));
    return d;
}
CVG_D cvg_f32x2 cvg_sub2(cvg_f32x2 a, cvg_f32x2 b)
{
    cvg_f32x2 d;
    asm("sub.rn.f32x2 %0, %1, %2;" : "=l"(d) : "l"(a), "l"(b));
    return d;
}
CVG_D cvg_f32x2 cvg_mul2(cvg_f32x2 a, cvg_f32x2 b)
{
    cvg_f32x2 d;
    asm("mul.rn.f32x2 %0, %1, %2;" : "=l"(d) : "l"(a), "l"(b));
    return d;
}
#endif  // device

#endif  // CVG_COMMON_CUH
