// cvg_kernels.cu -- precompiled FP64 kernels of the VEGAS+ iteration that do
// not depend on the integrand:
//   K3  hypercube reallocation (beta):  results -> finish -> count -> scan -> apply
//   K4  grid refinement (alpha):        one CTA per dimension
//
// K3 replaces results, updateNh, the DeviceReduce sums and the ExclusiveSum of
// the reference (src/main.cu:81-104, 173-187, 677-683, 579) and writes the
// tile map the fill uses instead of the evals[] list (src/main.cu:248-262).
// K4 replaces normalizeWeights, smoothWeights, the per-dim reduces and scans,
// setMap, updateXEdges and updateDxEdges (src/main.cu:106-145, 189-246,
// 667-694) and the histogram reset (src/main.cu:147-158).
#include "cvg_kernels.cuh"

#include <climits>
#include <cooperative_groups.h>
namespace cg = cooperative_groups;

namespace {

constexpr int RB = 256;                       // reallocation block
constexpr int RIPT = CVG_REALLOC_CHUNK / RB;  // cubes per thread

// Deterministic block sum: fixed per-thread order, fixed shuffle tree, fixed
// order over warps.  `scratch` holds blockDim/32 doubles per value.
template <int NV>
__device__ __forceinline__ void block_sum(double (&v)[NV], double *scratch)
{
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
#pragma unroll
    for (int i = 0; i < NV; ++i) {
        double x = v[i];
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) x += __shfl_down_sync(0xffffffffu, x, o);
        if (lane == 0) scratch[i * 32 + warp] = x;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
#pragma unroll
        for (int i = 0; i < NV; ++i) {
            double s = 0.0;
            for (int w = 0; w < nw; ++w) s += scratch[i * 32 + w];
            scratch[i * 32] = s;
        }
    }
    __syncthreads();
#pragma unroll
    for (int i = 0; i < NV; ++i) v[i] = scratch[i * 32];
    __syncthreads();
}

// Exclusive block scan of one u64 per thread; returns the block total.
__device__ __forceinline__ cvg_u64 block_exscan_u64(cvg_u64 &v, cvg_u64 *scratch)
{
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
    cvg_u64 x = v;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const cvg_u64 y = __shfl_up_sync(0xffffffffu, x, o);
        if (lane >= o) x += y;
    }
    if (lane == 31) scratch[warp] = x;
    __syncthreads();
    if (threadIdx.x == 0) {
        cvg_u64 s = 0;
        for (int w = 0; w < nw; ++w) { const cvg_u64 t = scratch[w]; scratch[w] = s; s += t; }
        scratch[32] = s;
    }
    __syncthreads();
    const cvg_u64 total = scratch[32];
    v = x - v + scratch[warp];
    __syncthreads();
    return total;
}

// ---- FP32-form helpers: no FP64-pipe instruction per hypercube ----

// float -> double by bit splicing: exact for normal numbers; zero and
// denormals give signed zero, inf/nan stay inf/nan (no FP64-pipe instruction)
__device__ __forceinline__ double f2d_bits(float f)
{
    const unsigned u = __float_as_uint(f);
    const unsigned e = (u >> 23) & 0xFFu;
    const unsigned sign = u & 0x80000000u;
    if (e == 0u) return __hiloint2double((int)sign, 0);
    if (e == 0xFFu) return __hiloint2double((int)(sign | 0x7FF00000u | ((u & 0x7FFFFFu) >> 3)), 0);
    return __hiloint2double((int)(sign | ((e + 896u) << 20) | ((u & 0x7FFFFFu) >> 3)), (int)(u << 29));
}

// x * 2^shift -> (hi, lo) floats holding the top 48 significand bits, integer
// ops only; magnitudes outside the float range become 0 or inf.
__device__ __forceinline__ void df_split(double x, float &hi, float &lo, int shift = 0)
{
    const int h = __double2hiint(x);
    const unsigned l = (unsigned)__double2loint(x);
    const unsigned sign = (unsigned)h & 0x80000000u;
    const int e = ((h >> 20) & 0x7FF) - 1023 + shift;   // x * 2^shift
    if (((h & 0x7FFFFFFF) | (int)l) == 0 || e < -125 || ((h >> 20) & 0x7FF) == 0) {   // zero, tiny
        hi = __uint_as_float(sign); lo = 0.f; return;
    }
    if (e > 127) { hi = __uint_as_float(sign | 0x7F800000u); lo = 0.f; return; }   // inf
    hi = __uint_as_float(sign | ((unsigned)(e + 127) << 23) | (((unsigned)h & 0xFFFFFu) << 3) |
                         (l >> 29));
    const unsigned rem = l & 0x1FFFFFFFu;
    if (rem == 0u || e < -74) { lo = 0.f; return; }
    const float sc = __uint_as_float((unsigned)(e + 75) << 23);   // 2^(e-52)
    lo = __uint_as_float(sign | __float_as_uint((float)rem * sc));
}

// double -> float (truncation), integer ops only
__device__ __forceinline__ float d2f_bits(double x)
{
    float hi, lo;
    df_split(x, hi, lo);
    return hi;
}

struct dfloat { float h, l; };

__device__ __forceinline__ dfloat df_add(dfloat a, dfloat b)
{
    const float s = a.h + b.h;
    const float bb = s - a.h;
    const float err = (a.h - (s - bb)) + (b.h - bb);
    const float t = err + a.l + b.l;
    dfloat r;
    r.h = s + t;
    r.l = t - (r.h - s);
    return r;
}

// Ticket of a finished block: true in the last of `nb` blocks (which then
// resets the counter).  Writes of every block are visible to the last one.
__device__ __forceinline__ bool last_block(cvg_u32 *ctr, unsigned nb)
{
    __shared__ bool last;
    __threadfence();
    __syncthreads();
    if (threadIdx.x == 0) {
        const cvg_u32 t = atomicAdd(ctr, 1u);
        last = (t == nb - 1);
        if (last) *ctr = 0u;
    }
    __syncthreads();
    if (last) __threadfence();
    return last;
}

// R hypercubes per thread (RIPT, or 2 for runs with few hypercubes, where
// the per-thread chain of 8 would leave the launch latency-bound)
template <int R = RIPT>
__device__ __forceinline__ void k3_results_dev(const cvg_realloc_args &a, const unsigned blk)
{
    __shared__ double scratch[3 * 32];
    const cvg_u32 base = blk * (cvg_u32)(RB * R);
    double v[3] = {0.0, 0.0, 0.0};   // dh, I, sigma2
    const double vc = a.v_cubes;
    for (int k = 0; k < R; ++k) {
        const cvg_u32 c = base + k * RB + threadIdx.x;
        if (c >= a.n_cubes) break;
        const int neval = (int)(a.nh_sum[c + 1] - a.nh_sum[c]);
        const double jf = a.JF[c], jf2 = a.JF2[c];
        a.JF[c] = 0.0;
        a.JF2[c] = 0.0;
        // src/main.cu:88-102, same operation order
        const double Ih = jf / neval * vc;
        const double Sig2 = (jf2 / neval * vc * vc) - (Ih * Ih);
        v[1] += Ih;
        v[2] += Sig2 / neval;
        double t = vc * vc * jf2 / neval - pow(vc * jf / neval, 2);
        if (t < 0) t = 0;
        const double dh = pow(t, a.beta);
        a.dh[c] = dh;
        v[0] += dh;
    }
    block_sum<3>(v, scratch);
    if (threadIdx.x == 0) {
        a.partials[4 * blk + 0] = v[0];
        a.partials[4 * blk + 1] = v[1];
        a.partials[4 * blk + 2] = v[2];
        a.partials[4 * blk + 3] = 0.0;
    }
}

__device__ void k3_finish_dev(const cvg_realloc_args &a, unsigned nb);
__device__ void k3_scan_dev(const cvg_realloc_args &a, unsigned nb);

template <int R>
__global__ void __launch_bounds__(RB) k3_results(cvg_realloc_args a)
{
    k3_results_dev<R>(a, blockIdx.x);
    if (last_block(&a.done[0], gridDim.x)) k3_finish_dev(a, gridDim.x);
}


// FP32 form of k3_results.  Per cube, with m = JF/n and q = JF2/n held as
// double-floats (48-bit significands): I_h / V = m, sigma2_h / V^2 = q - m^2,
// d_h = (q - m^2)^beta (the constant V^(2 beta) cancels in the allocation).
// Sums are compensated in FP32 per thread, FP64 across warps and blocks;
// k3_finish multiplies by V and V^2.
template <int R = RIPT, bool XQ = false>
__device__ __forceinline__ void k3_results_f32_dev(const cvg_realloc_args &a, const unsigned blk)
{
    __shared__ double wsum[4][RB / 32];
    __shared__ float wdq[XQ ? RB / 32 : 1];
    const cvg_u32 base = blk * (cvg_u32)(RB * R);
    // XQ (batched runs): sum of d_h * q (2^-64) for the next fill's exponent shift
    const bool xq = XQ && a.exp_dq != nullptr;
    float sdq = 0.f;
    const float beta = (float)a.beta;
    const int kx = a.scale_exp ? *a.scale_exp : 0;   // work on JF*2^-k, JF2*2^-2k
    dfloat sm = {0.f, 0.f};
    float sv = 0.f, kv = 0.f, sd = 0.f, kd = 0.f;   // Kahan sums of var/n and d_h
    float sq = 0.f;                                  // sum of JF2*2^-2k (next scale)
    const cvg_u64 *__restrict__ nhs = a.nh_sum;
    double *__restrict__ JF = a.JF;
    double *__restrict__ JF2 = a.JF2;
    float *__restrict__ DH = reinterpret_cast<float *>(a.dh);   // FP32 form: d_h as float
    // issue every load of this thread's cubes before any store
    cvg_u64 s0[R], s1[R];
    double j1[R], j2[R];
#pragma unroll
    for (int k = 0; k < R; ++k) {
        const cvg_u32 c = base + k * RB + threadIdx.x;
        const bool in = c < a.n_cubes;
        s0[k] = in ? nhs[c] : 0ull;
        s1[k] = in ? nhs[c + 1] : 1ull;
        j1[k] = in ? JF[c] : 0.0;
        j2[k] = in ? JF2[c] : 0.0;
    }
#pragma unroll
    for (int k = 0; k < R; ++k) {
        const cvg_u32 c = base + k * RB + threadIdx.x;
        if (c >= a.n_cubes) break;
        JF[c] = 0.0;
        JF2[c] = 0.0;
        const int neval = (int)(s1[k] - s0[k]);
        float jh, jl, qh, ql;
        df_split(j1[k], jh, jl, -kx);
        df_split(j2[k], qh, ql, -2 * kx);
        sq += qh;
        const float fn = (float)neval;
        const float inv = 1.0f / fn;
        // m = JF/n, q = JF2/n as double-floats
        float mh = jh * inv;
        float ml = (fmaf(-mh, fn, jh) + jl) * inv;
        float qq = qh * inv;
        float qlo = (fmaf(-qq, fn, qh) + ql) * inv;
        // var = q - m^2 (the leading difference is exact when it cancels)
        const float p = mh * mh;
        const float pe = fmaf(mh, mh, -p) + 2.0f * mh * ml;
        float var = (qq - p) + (qlo - pe);
        var = var > 0.f ? var : 0.f;
        dfloat mv = {mh, ml};
        sm = df_add(sm, mv);
        {
            const float y = var * inv - kv, t = sv + y;
            kv = (t - sv) - y; sv = t;
        }
        const float dh = var > 0.f ? exp2f(beta * log2f(var)) : 0.f;
        {
            const float y = dh - kd, t = sd + y;
            kd = (t - sd) - y; sd = t;
        }
        if (xq) sdq = fmaf(dh * 0x1p-32f, qq * 0x1p-32f, sdq);
        DH[c] = dh;
    }
    // warp reduction in FP32 (double-float for the estimate)
    float v = sv - kv, d = sd - kd;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        dfloat other = {__shfl_down_sync(0xffffffffu, sm.h, o), __shfl_down_sync(0xffffffffu, sm.l, o)};
        sm = df_add(sm, other);
        v += __shfl_down_sync(0xffffffffu, v, o);
        d += __shfl_down_sync(0xffffffffu, d, o);
        sq += __shfl_down_sync(0xffffffffu, sq, o);
        if (xq) sdq += __shfl_down_sync(0xffffffffu, sdq, o);
    }
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    if (lane == 0) {
        if (xq) wdq[warp] = sdq;
        wsum[0][warp] = f2d_bits(d);
        wsum[1][warp] = f2d_bits(sm.h) + f2d_bits(sm.l);
        wsum[2][warp] = f2d_bits(v);
        wsum[3][warp] = f2d_bits(sq);
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        double t0 = 0.0, t1 = 0.0, t2 = 0.0, t3 = 0.0;
        for (int w = 0; w < RB / 32; ++w) {
            t0 += wsum[0][w]; t1 += wsum[1][w]; t2 += wsum[2][w]; t3 += wsum[3][w];
        }
        a.partials[4 * blk + 0] = t0;
        a.partials[4 * blk + 1] = t1;
        a.partials[4 * blk + 2] = t2;
        a.partials[4 * blk + 3] = t3;
        if (xq) {
            double t4 = 0.0;
            for (int w = 0; w < RB / 32; ++w) t4 += f2d_bits(wdq[w]);
            atomicAdd(a.exp_dq, t4);
        }
    }
}

// 4 blocks per SM (64 registers, no spills): more loads in flight than the
// 76-register build's 3 (C2 step 1.955 -> 1.938 ms); 5 or more spill
template <int R>
__global__ void __launch_bounds__(RB, 4) k3_results_f32(cvg_realloc_args a)
{
    k3_results_f32_dev<R>(a, blockIdx.x);
    if (last_block(&a.done[0], gridDim.x)) k3_finish_dev(a, gridDim.x);
}


__device__ void k3_finish_dev(const cvg_realloc_args &a, unsigned nb)
{
    __shared__ double scratch[4 * 32];
    double v[4] = {0.0, 0.0, 0.0, 0.0};
    for (unsigned i = threadIdx.x; i < nb; i += blockDim.x) {
        v[0] += a.partials[4 * i + 0];
        v[1] += a.partials[4 * i + 1];
        v[2] += a.partials[4 * i + 2];
        v[3] += a.partials[4 * i + 3];
    }
    block_sum<4>(v, scratch);
    if (threadIdx.x == 0) {
        // every load of the loop state first, then the arithmetic, then the
        // stores: one round trip to memory instead of one per field (this step
        // is on the critical path of small iterations)
        cvg_acc_dev *acc = a.acc;
        const cvg_u32 it = *a.iteration;
        const int kx = (a.fast_pow && a.scale_exp) ? *a.scale_exp : 0;
        const cvg_u64 S = a.nh_sum[a.n_cubes];
        const double sw = acc->sw, swr = acc->swr, swr2 = acc->swr2;
        const cvg_u64 used = acc->used, tot = acc->tot_nevals;
        const cvg_u32 rare_n = a.hist_state ? a.hist_state[1] : 0u;
        const double dq = a.exp_dq ? *a.exp_dq : 0.0;

        double r = v[1], s = v[2];
        int knew = kx;
        if (a.fast_pow) {   // FP32 form sums m 2^-k and var 2^-2k / n without the cube volume
            r = ldexp(r, kx) * a.v_cubes;
            s = ldexp(s, 2 * kx) * (a.v_cubes * a.v_cubes);
            if (a.scale_exp) {   // next scale: 2^k ~ rms of f*jac
                const double ms = v[3] / (double)S;
                if (ms > 0.0 && isfinite(ms)) {
                    int e = 0;
                    frexp(ms, &e);
                    knew = kx + e / 2;
                    knew = knew < -100 ? -100 : (knew > 100 ? 100 : knew);
                }
            }
        }
        const bool in_mean = (int)it >= a.skip;   // src/main.cu:680, 698-713
        // FP32 form: fixed-point bin sums in the next fill only from the third
        // iteration on (the first reallocation of a peaked integrand moves
        // the samples far from what the exponent table predicts) and only
        // while rare updates stayed below 1 in 1024
        const bool fixed_next = (int)it + 1 >= a.hist_min_it &&
                                ldexp((double)rare_n, a.rare_shift) <= (double)S * (double)a.dim;

        if (a.fast_pow && a.scale_exp) *a.scale_exp = knew;
        if (a.exp_dq && a.exp_shift) {
            // batched FP32 form: the next fill samples hypercube c about
            // n_eval d_h/sum(d_h) times, so its mean per-sample (f*jac)^2 is
            // near sum(d_h q)/sum(d_h), against sum(JF2)/S in this fill (q =
            // JF2/n of c, both in 2^-2k units); the exponent table (per-bin
            // means of this fill) is raised by that ratio's whole bits
            // (without adaptation the allocation does not follow d_h: no shift)
            const double enew = ldexp(dq, 64) / v[0], eold = v[3] / (double)S;
            int sh = 0;
            if (a.adapt && enew > 0.0 && eold > 0.0 && isfinite(enew) && isfinite(eold)) {
                int e = 0;
                frexp(enew / eold, &e);
                sh = e - 1 < 0 ? 0 : (e - 1 > 40 ? 40 : e - 1);
            }
            *a.exp_shift = sh;
            *a.exp_dq = 0.0;
        }
        if ((int)it < a.max_it) {
            a.stats[it] = r;
            a.stats[a.max_it + it] = s;
            a.stats[2 * a.max_it + it] = (double)S;
        }
        acc->dh_sum = v[0];
        acc->nh_scale = (double)a.n_eval_it / v[0];
        acc->tot_nevals = tot + S;
        acc->last_nevals = S;
        if (in_mean) {
            acc->sw = sw + 1.0 / s;
            acc->swr = swr + r / s;
            acc->swr2 = swr2 + r * r / s;
            acc->used = used + 1;
        }
        if (!isfinite(r) || !isfinite(s)) atomicOr(a.status, CVG_KSTAT_NONFINITE);
        if (a.hist_state) {
            a.hist_state[0] = fixed_next ? 1u : 0u;
            a.hist_state[1] = 0u;
        }
        *a.iteration = it + 1;
    }
}




// mode 0: nh from the damped variances (updateNh, src/main.cu:173-187)
// mode 1: nh_new already holds the counts (initialisation / state import)
// mode 2: FP32 form, nh = floor(d_h * n_eval_it / sum d_h) in FP32
// mode 0: n_h from the FP64 d_h (reference conversion); 1: n_h given in
// nh_new; 2: n_h from the FP32 form's float d_h, scaled.
template <int MODE>
__device__ __forceinline__ void k3_count_mode(const cvg_realloc_args &a, const unsigned blk)
{
    __shared__ cvg_u64 wtot[RB / 32];
    const cvg_u32 base = blk * CVG_REALLOC_CHUNK;
    double dsum = 0.0, n_it = 0.0;
    float scale = 0.f;
    if (MODE == 0) { dsum = a.acc->dh_sum; n_it = (double)a.n_eval_it; }
    if (MODE == 2) scale = d2f_bits(a.acc->nh_scale) * 0.99999905f;   // round the total down
    cvg_u64 tot = 0;
    double dhv[MODE == 0 ? RIPT : 1];
    float dhf[MODE == 2 ? RIPT : 1];
    const float *dh32 = reinterpret_cast<const float *>(a.dh);
#pragma unroll
    for (int k = 0; k < RIPT; ++k) {   // issue the loads first
        const cvg_u32 c = base + k * RB + threadIdx.x;
        if (MODE == 0) dhv[k] = c < a.n_cubes ? a.dh[c] : 0.0;
        if (MODE == 2) dhf[k] = c < a.n_cubes ? dh32[c] : 0.f;
    }
#pragma unroll
    for (int k = 0; k < RIPT; ++k) {
        const cvg_u32 c = base + k * RB + threadIdx.x;
        if (c >= a.n_cubes) break;
        cvg_u32 nh;
        if (MODE == 0) {
            const double f = dhv[k] / dsum;
            const double x = f * n_it;
            // (int) conversion of the reference: NaN -> 0, saturating above
            int ns = (x >= 0.0 && x < 2147483647.0) ? (int)x : (x >= 2147483647.0 ? 2147483647 : 0);
            nh = ns < 2 ? 2u : (cvg_u32)ns;
            a.nh_new[c] = nh;
        } else if (MODE == 2) {
            const float x = dhf[k] * scale;
            const int ns = (x >= 0.f && x < 2147483520.f) ? (int)x : (x >= 2147483520.f ? 2147483520 : 0);
            nh = ns < 2 ? 2u : (cvg_u32)ns;
            a.nh_new[c] = nh;
        } else {
            nh = a.nh_new[c];
        }
        tot += nh;
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) tot += __shfl_down_sync(0xffffffffu, tot, o);
    if ((threadIdx.x & 31) == 0) wtot[threadIdx.x >> 5] = tot;
    __syncthreads();
    if (threadIdx.x == 0) {
        cvg_u64 t = 0;
        for (int w = 0; w < RB / 32; ++w) t += wtot[w];
        a.bsums[blk] = t;
    }
}

__device__ __forceinline__ void k3_count_dev(const cvg_realloc_args &a, int mode, const unsigned blk)
{
    if (mode == 0) k3_count_mode<0>(a, blk);
    else if (mode == 1) k3_count_mode<1>(a, blk);
    else k3_count_mode<2>(a, blk);
}

__global__ void __launch_bounds__(RB) k3_count(cvg_realloc_args a, int mode)
{
    k3_count_dev(a, mode, blockIdx.x);
    const unsigned nb = cvg_realloc_blocks(a.n_cubes);
    if (last_block(&a.done[1], nb)) k3_scan_dev(a, nb);
}


__device__ void k3_scan_dev(const cvg_realloc_args &a, unsigned nb)
{
    __shared__ cvg_u64 scratch[33];
    const unsigned per = (nb + blockDim.x - 1) / blockDim.x;
    const unsigned b0 = threadIdx.x * per;
    cvg_u64 local = 0;
    for (unsigned i = 0; i < per; ++i)
        if (b0 + i < nb) local += a.bsums[b0 + i];
    cvg_u64 off = local;
    const cvg_u64 total = block_exscan_u64(off, scratch);
    for (unsigned i = 0; i < per; ++i)
        if (b0 + i < nb) { const cvg_u64 t = a.bsums[b0 + i]; a.bsums[b0 + i] = off; off += t; }
    if (threadIdx.x == 0) a.bsums[nb] = total;
}

// Prefixes st[] of this thread's RIPT hypercubes (sh[] holds their n_h, off is
// the first one's prefix) and the tile map: tile t (samples [t*TS, (t+1)*TS))
// records the hypercube holding its first sample.  One division per thread;
// the tile index then only advances (t*TS >= off at every hypercube).
__device__ __forceinline__ void k3_prefix_tiles(const cvg_realloc_args &a, const cvg_u32 *sh,
                                                cvg_u64 *st, cvg_u64 off, cvg_u32 base, cvg_u32 cnt)
{
    const cvg_u64 TS = (cvg_u64)a.tile_samples;
    cvg_u64 t = (off + TS - 1) / TS;
    cvg_u64 ts = t * TS;
#pragma unroll 1
    for (int k = 0; k < RIPT; ++k) {
        const int i = threadIdx.x * RIPT + k;
        const cvg_u64 n = sh[i];
        st[i] = off;
        if ((cvg_u32)i < cnt)
            for (; ts < off + n && t < a.max_tiles; ++t, ts += TS) a.tile_cube[t] = base + i;
        off += n;
    }
}

__device__ __forceinline__ void k3_apply_dev(const cvg_realloc_args &a, unsigned nb, const unsigned blk)
{
    __shared__ cvg_u32 sh[CVG_REALLOC_CHUNK];
    __shared__ cvg_u64 st[CVG_REALLOC_CHUNK];
    __shared__ cvg_u64 scratch[33];
    const cvg_u32 base = blk * CVG_REALLOC_CHUNK;
    const cvg_u32 cnt = min((cvg_u32)CVG_REALLOC_CHUNK, a.n_cubes - base);
    for (int i = threadIdx.x; i < CVG_REALLOC_CHUNK; i += RB)
        sh[i] = (cvg_u32)i < cnt ? a.nh_new[base + i] : 0u;
    __syncthreads();
    cvg_u64 local = 0;
#pragma unroll
    for (int k = 0; k < RIPT; ++k) local += sh[threadIdx.x * RIPT + k];
    cvg_u64 off = local;
    block_exscan_u64(off, scratch);
    off += a.bsums[blk];
    k3_prefix_tiles(a, sh, st, off, base, cnt);
    __syncthreads();
    for (int i = threadIdx.x; i < (int)cnt; i += RB) a.nh_sum[base + i] = st[i];
    if (blk == nb - 1 && threadIdx.x == 0) a.nh_sum[a.n_cubes] = a.bsums[nb];
}

__global__ void __launch_bounds__(RB) k3_apply(cvg_realloc_args a, unsigned nb) { k3_apply_dev(a, nb, blockIdx.x); }

// ---------------------------------------------------------------------------
// One-pass allocation (count + scan + apply): each block computes n_h for its
// chunk of hypercubes, publishes the chunk's sum, and finds the sum of all
// chunks before it by decoupled look-back over the blocks' published words;
// then it writes the exclusive prefixes (nh_sum) and the tile map.  Blocks
// take chunk indices in the order they start (a ticket), so every block a
// block waits on has started before it; the waits are bounded anyway (a
// timeout sets CVG_KSTAT_TIMEOUT).  A look-back word packs the launch epoch
// (bits 34..63), a flag (1 = chunk sum, 2 = inclusive prefix) and a 32-bit
// value, so the words need no clearing between launches.
// ---------------------------------------------------------------------------
constexpr cvg_u64 LB_AGG = 1ull << 32, LB_PRE = 2ull << 32;
constexpr int LB_SPIN_LIMIT = 1 << 22;

__device__ __forceinline__ cvg_u64 lb_word(cvg_u32 epoch, cvg_u64 flag, cvg_u64 value)
{
    return ((cvg_u64)epoch << 34) | flag | (value & 0xFFFFFFFFull);
}
// Epochs run 1 .. 2^30 - 1 (0 marks a word never written).
__device__ __forceinline__ cvg_u32 lb_next_epoch(cvg_u32 e) { return e % 0x3FFFFFFFu + 1u; }

template <int MODE>
__device__ __forceinline__ void k3_alloc_dev(const cvg_realloc_args &a, unsigned nb)
{
    __shared__ cvg_u64 scratch[33];
    __shared__ unsigned s_blk;
    __shared__ cvg_u32 s_epoch;
    __shared__ cvg_u64 s_excl;
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    if (tid == 0) {
        s_epoch = lb_next_epoch(*(volatile cvg_u32 *)&a.lb_ctl[1]);   // read before the ticket
        __threadfence();
        s_blk = atomicAdd(&a.lb_ctl[0], 1u);
    }
    __syncthreads();
    const unsigned blk = s_blk;
    const cvg_u32 epoch = s_epoch;
    const cvg_u32 base = blk * CVG_REALLOC_CHUNK;
    const cvg_u32 cnt = min((cvg_u32)CVG_REALLOC_CHUNK, a.n_cubes - base);

    // n_h of this thread's RIPT consecutive hypercubes, in registers (as k3_count)
    double dsum = 0.0, n_it = 0.0;
    float scale = 0.f;
    if (MODE == 0) { dsum = a.acc->dh_sum; n_it = (double)a.n_eval_it; }
    if (MODE == 2) scale = d2f_bits(a.acc->nh_scale) * 0.99999905f;
    const float *dh32 = reinterpret_cast<const float *>(a.dh);
    const int i0 = tid * RIPT;
    const cvg_u32 c0 = base + (cvg_u32)i0;
    static_assert(RIPT == 8, "k3_alloc loads 8 hypercubes per thread");
    cvg_u32 nh[RIPT];
    const bool full = (cvg_u32)i0 + RIPT <= cnt;
    if (MODE == 2 && full) {   // 32 contiguous bytes per thread
        const float4 v0 = *reinterpret_cast<const float4 *>(dh32 + c0);
        const float4 v1 = *reinterpret_cast<const float4 *>(dh32 + c0 + 4);
        const float x[8] = {v0.x, v0.y, v0.z, v0.w, v1.x, v1.y, v1.z, v1.w};
#pragma unroll
        for (int k = 0; k < RIPT; ++k) {
            const float y = x[k] * scale;
            const int ns = (y >= 0.f && y < 2147483520.f) ? (int)y : (y >= 2147483520.f ? 2147483520 : 0);
            nh[k] = ns < 2 ? 2u : (cvg_u32)ns;
        }
    } else {
#pragma unroll
        for (int k = 0; k < RIPT; ++k) {
            const cvg_u32 c = c0 + k;
            cvg_u32 v = 0u;
            if ((cvg_u32)(i0 + k) < cnt) {
                if (MODE == 0) {
                    const double x = a.dh[c] / dsum * n_it;
                    int ns = (x >= 0.0 && x < 2147483647.0) ? (int)x : (x >= 2147483647.0 ? 2147483647 : 0);
                    v = ns < 2 ? 2u : (cvg_u32)ns;
                } else if (MODE == 2) {
                    const float y = dh32[c] * scale;
                    const int ns = (y >= 0.f && y < 2147483520.f) ? (int)y : (y >= 2147483520.f ? 2147483520 : 0);
                    v = ns < 2 ? 2u : (cvg_u32)ns;
                } else {
                    v = a.nh_new[c];
                }
            }
            nh[k] = v;
        }
    }
    cvg_u64 local = 0;
#pragma unroll
    for (int k = 0; k < RIPT; ++k) local += nh[k];
    cvg_u64 off = local;
    const cvg_u64 agg = block_exscan_u64(off, scratch);

    // decoupled look-back by warp 0, 32 predecessors at a time
    const int spin_limit = a.lb_spin_limit > 0 ? a.lb_spin_limit : LB_SPIN_LIMIT;
    const bool publish = blk + 1u != a.lb_withhold;   // false only in the failure test
    if (warp == 0) {
        cvg_u64 excl = 0;
        bool timeout = false;
        if (blk == 0) {
            if (lane == 0 && publish) atomicExch((unsigned long long *)&a.lb[0], lb_word(epoch, LB_PRE, agg));
        } else {
            if (lane == 0 && publish)
                atomicExch((unsigned long long *)&a.lb[blk], lb_word(epoch, LB_AGG, agg));
            int j = (int)blk - 1;
            while (true) {
                const int idx = j - lane;
                cvg_u64 w = 0;
                int spins = 0;
                bool ready;
                do {
                    w = idx >= 0 ? *(volatile cvg_u64 *)&a.lb[idx] : lb_word(epoch, LB_PRE, 0);
                    ready = (cvg_u32)(w >> 34) == epoch;
                } while (!__all_sync(0xffffffffu, ready) && ++spins < spin_limit);
                if (spins >= spin_limit) { timeout = true; break; }
                const unsigned pm = __ballot_sync(0xffffffffu, (w & LB_PRE) != 0);
                const int lp = pm ? __ffs(pm) - 1 : 31;
                cvg_u64 v = lane <= lp ? (w & 0xFFFFFFFFull) : 0ull;
#pragma unroll
                for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
                excl += v;
                if (pm) break;
                j -= 32;
            }
            if (lane == 0) {
                if (timeout) atomicOr(a.status, CVG_KSTAT_TIMEOUT);
                if (publish)
                    atomicExch((unsigned long long *)&a.lb[blk], lb_word(epoch, LB_PRE, excl + agg));
            }
        }
        if (lane == 0) s_excl = excl;
    }
    __syncthreads();
    off += s_excl;

    // prefixes and tile map from registers (as k3_apply): one division per
    // thread, the tile index then only advances
    const cvg_u64 TS = (cvg_u64)a.tile_samples;
    cvg_u64 t = (off + TS - 1) / TS;
    cvg_u64 ts = t * TS;
    cvg_u64 pre[RIPT];
#pragma unroll
    for (int k = 0; k < RIPT; ++k) {
        pre[k] = off;
        for (; ts < off + nh[k] && t < a.max_tiles; ++t, ts += TS) a.tile_cube[t] = c0 + k;
        off += nh[k];
    }
    if (full) {   // 64 contiguous bytes per thread
#pragma unroll
        for (int k = 0; k < RIPT; k += 2)
            *reinterpret_cast<ulonglong2 *>(a.nh_sum + c0 + k) = make_ulonglong2(pre[k], pre[k + 1]);
    } else {
#pragma unroll
        for (int k = 0; k < RIPT; ++k)
            if ((cvg_u32)(i0 + k) < cnt) a.nh_sum[c0 + k] = pre[k];
    }
    if (blk == nb - 1 && tid == 0) {
        // every block has taken its ticket: reset it; the next launch's epoch
        a.nh_sum[a.n_cubes] = s_excl + agg;
        a.lb_ctl[0] = 0u;
        a.lb_ctl[1] = epoch;
    }
}

// 8 CTAs per SM (32 registers; a few bytes spill): more blocks in their
// look-back at once (C2: 76.9 -> 69.6 us against 6 CTAs at 40 registers)
template <int MODE>
__global__ void __launch_bounds__(RB, 8) k3_alloc(cvg_realloc_args a, unsigned nb)
{
    k3_alloc_dev<MODE>(a, nb);
}


// ---------------------------------------------------------------------------
// K4: grid refinement, FP64.  One thread-block cluster of CL CTAs per
// dimension: CTA r owns bins [r*B, (r+1)*B).  Partial sums and scan offsets
// are exchanged through distributed shared memory, so the FP64 pow/log of
// the damping run on CL SMs per dimension instead of one.
// ---------------------------------------------------------------------------
constexpr int CL = 8;      // CTAs per cluster (portable size)
constexpr int KB = 128;    // threads per CTA

// Dynamic shared memory of one K4 CTA: doubles w[B+2] sw[B] cs[B] fsw[N]
// fcs[N] xo[N+1] fw[N], then ints fdv[N] eb[B] dv[B].
__host__ __device__ inline size_t k4_smem_bytes(int N)
{
    const size_t B = (size_t)((N + CL - 1) / CL);
    return sizeof(double) * (3 * B + 4 * (size_t)N + 3) + sizeof(int) * ((size_t)N + 2 * B) + 16;
}

// Binary exponent of a positive finite double (denormals: -1023), else INT_MIN.
__device__ __forceinline__ int k4_exponent(double v)
{
    if (!(v > 0.0) || !isfinite(v)) return INT_MIN;
    return (int)((__double_as_longlong(v) >> 52) & 0x7FF) - 1023;
}

__device__ __forceinline__ double cl_sum(cg::cluster_group &cl, double *slot)
{
    double t = 0.0;
    for (int q = 0; q < CL; ++q) t += *cl.map_shared_rank(slot, q);   // same order everywhere
    return t;
}

__device__ __forceinline__ void k4_refine_dev(const cvg_refine_args &a, const int d)
{
    extern __shared__ __align__(16) double ks[];
    __shared__ double part[4];
    __shared__ double wscr[KB / 32];
    __shared__ int iscr[KB / 32];
    __shared__ int emin_slot;
    cg::cluster_group cl = cg::this_cluster();
    const int r = (int)cl.block_rank();
    const int N = a.n_intervals, tid = threadIdx.x;
    const int B = (N + CL - 1) / CL;
    const int i0 = min(N, r * B), i1 = min(N, i0 + B), nb = i1 - i0;
    // smem: w[B+2] (with halo) | sw[B] | cs[B] | fsw[N] | fcs[N] | xo[N+1] | fw[N] | fdv[N] |
    // eb[B] | dv[B]
    double *w = ks, *sw = w + B + 2, *cs = sw + B, *fsw = cs + B, *fcs = fsw + N, *xo = fcs + N;
    double *fw = xo + N + 1;
    int *fdv = (int *)(fw + N), *eb = fdv + N, *dv = eb + B;
    // FP32 form: per-bin exponents of the expected per-sample (f*jac)^2 of the
    // next fill (see the fill's histogram update); eb holds this CTA's bins
    const bool ex = a.bin_exp != nullptr;
    double *xe = a.x_edges + (size_t)d * (N + 1);
    float *xe32 = a.x_edges32 + (size_t)d * (N + 1);

    auto block_total = [&](double v) -> double {   // fixed-order block sum
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
        if ((tid & 31) == 0) wscr[tid >> 5] = v;
        __syncthreads();
        double t = 0.0;
        for (int q = 0; q < KB / 32; ++q) t += wscr[q];
        __syncthreads();
        return t;
    };

    // normalizeWeights (src/main.cu:106-118) for own bins and one halo bin
    // each side; the old grid row is kept in shared memory.
    double p1 = 0.0;
    for (int i = i0 - 1 + tid; i <= i1; i += KB) {
        if (i < 0 || i >= N) continue;
        const size_t g = (size_t)d * N + i;
        const double wi = a.weights[g];
        const cvg_u32 cn = a.counts[g];
        const double x = cn != 0u ? wi / (double)cn : wi;
        w[i - i0 + 1] = x;
        if (i >= i0 && i < i1) p1 += x;
    }
    for (int i = tid; i <= N; i += KB) xo[i] = xe[i];
    p1 = block_total(p1);
    if (tid == 0) part[0] = p1;
    cl.sync();
    const double dsum = cl_sum(cl, &part[0]);          // d_sum (src/main.cu:668-670)
    for (int i = i0 + tid; i < i1; i += KB) {          // resetWeights (src/main.cu:147-158)
        a.weights[(size_t)d * N + i] = 0.0;
        a.counts[(size_t)d * N + i] = 0u;
    }
    bool ok = a.adapt && dsum > 0.0 && isfinite(dsum);

    if (ok) {
        // smoothWeights (src/main.cu:120-145).  The FP32 form (ex) multiplies
        // by 1/(8 d_sum) instead of dividing per bin (FP64 divisions are the
        // costly part of this kernel; a one-rounding difference in the
        // smoothed weight is far inside that form's tolerance); the FP64 form
        // keeps the reference's division.
        const double r8 = ex ? 1.0 / (8.0 * dsum) : 0.0;
        double p2 = 0.0;
        for (int i = i0 + tid; i < i1; i += KB) {
            const double wm = i > 0 ? w[i - i0] : 0.0, wc = w[i - i0 + 1];
            const double wp = i < N - 1 ? w[i - i0 + 2] : 0.0;
            double t;
            const double num = i == 0 ? 7.0 * wc + wp
                             : (i == N - 1 ? wm + 7.0 * wc : wm + 6.0 * wc + wp);
            t = ex ? num * r8 : num / (8.0 * dsum);
            if (t != 0) {
                // ((t-1)/ln t)^alpha; alpha = 0.5 (the default) as a square
                // root, correctly rounded and several times cheaper than pow
                // on this GPU's FP64 pipe
                const double v = (t - 1.0) / log(t);
                t = a.alpha == 0.5 ? sqrt(v) : pow(v, a.alpha);
            }
            sw[i - i0] = t;
            p2 += t;
        }
        __syncthreads();
        // inclusive scan of own bins: each thread a contiguous run
        const int per = (nb + KB - 1) / KB;
        const int j0 = tid * per;
        double loc = 0.0;
        for (int k = 0; k < per && j0 + k < nb; ++k) loc += sw[j0 + k];
        double x = loc;
        const int lane = tid & 31, warp = tid >> 5;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const double y = __shfl_up_sync(0xffffffffu, x, o);
            if (lane >= o) x += y;
        }
        if (lane == 31) wscr[warp] = x;
        __syncthreads();
        double woff = 0.0;
        for (int q = 0; q < warp; ++q) woff += wscr[q];
        double run = x - loc + woff;
        for (int k = 0; k < per && j0 + k < nb; ++k) { run += sw[j0 + k]; cs[j0 + k] = run; }
        __syncthreads();
        p2 = block_total(p2);
        if (tid == 0) { part[1] = p2; part[2] = nb > 0 ? cs[nb - 1] : 0.0; }
        cl.sync();
        const double ssum = cl_sum(cl, &part[1]);      // summed_weights (src/main.cu:673-675)
        double pre = 0.0;
        for (int q = 0; q < r; ++q) pre += *cl.map_shared_rank(&part[2], q);
        ok = ssum > 0.0 && isfinite(ssum);
        const double delta = ssum / N;
        // the cumulative sum and setMap's div (src/main.cu:189-209) of this
        // CTA's own bins; the cluster gathers both below (one FP64 division
        // per bin in the cluster, not per bin in every CTA)
        for (int j = tid; j < nb; j += KB) {
            cs[j] += pre;
            if (ok) dv[j] = (int)(cs[j] / delta);
        }
        cl.sync();
        if (ok) {
            // gather sw and the scan of every bin of this dimension
            for (int q = 0; q < CL; ++q) {
                const int q0 = min(N, q * B), q1 = min(N, q0 + B);
                const double *rsw = cl.map_shared_rank(sw, q), *rcs = cl.map_shared_rank(cs, q);
                const double *rw = cl.map_shared_rank(w, q);
                const int *rdv = cl.map_shared_rank(dv, q);
                for (int j = tid; j < q1 - q0; j += KB) {
                    fsw[q0 + j] = rsw[j];
                    fcs[q0 + j] = rcs[j];
                    fdv[q0 + j] = rdv[j];
                    if (ex) fw[q0 + j] = rw[j + 1];
                }
            }
            __syncthreads();
            // updateXEdges (src/main.cu:211-230): new edge k+1 lies in old
            // interval o = min{ i : div_i > k }, the interval setMap assigns to k
            for (int k = i0 + tid; k < min(i1, N - 1); k += KB) {
                int lo = 0, hi = N - 1;
                while (lo < hi) {
                    const int mid = (lo + hi) >> 1;
                    if (fdv[mid] > k) hi = mid; else lo = mid + 1;
                }
                const int o = lo;
                const double acc = (k + 1) * delta - (o > 0 ? fcs[o - 1] : 0.0);
                if (ex) {
                    // FP32 form: one reciprocal of the old bin's weight for
                    // the edge and the exponent
                    const double rw = 1.0 / fsw[o];
                    const double xn = fma(acc * rw, xo[o + 1] - xo[o], xo[o]);
                    xe[k + 1] = xn;
                    xe32[k + 1] = (float)xn;
                    // new bin k ends in old bin o, where it is delta/fsw[o] of
                    // o's width wide: its samples' (f*jac)^2 scale by that
                    // ratio squared
                    const double rr = fsw[o] > 0.0 ? delta * rw : 1.0;
                    eb[k - i0] = k4_exponent(fw[o] * rr * rr);
                } else {
                    const double xn = fma(acc / fsw[o], xo[o + 1] - xo[o], xo[o]);
                    xe[k + 1] = xn;
                    xe32[k + 1] = (float)xn;
                }
            }
            if (ex && i1 == N && i0 < N && tid == 0) {
                const double rr = fsw[N - 1] > 0.0 ? delta / fsw[N - 1] : 1.0;
                eb[N - 1 - i0] = k4_exponent(fw[N - 1] * rr * rr);
            }
            if (r == 0 && tid == 0) xe32[0] = (float)xo[0];
            if (i1 == N && i0 < N && tid == 0) xe32[N] = (float)xo[N];
        }
    }
    if (!ok && nb > 0) {
        for (int i = i0 + tid; i <= (i1 == N ? N : i1 - 1); i += KB) xe32[i] = (float)xo[i];
        if (ex)
            for (int i = i0 + tid; i < i1; i += KB) eb[i - i0] = k4_exponent(w[i - i0 + 1]);
    }
    if (ex) {
        // bins without an estimate (no samples, zero weight) take the
        // dimension's smallest exponent; stored unscaled (+2k of the fill)
        __syncthreads();
        int mn = INT_MAX;
        for (int i = tid; i < nb; i += KB)
            if (eb[i] != INT_MIN) mn = min(mn, eb[i]);
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) mn = min(mn, __shfl_down_sync(0xffffffffu, mn, o));
        if ((tid & 31) == 0) iscr[tid >> 5] = mn;
        __syncthreads();
        if (tid == 0) {
            int m = INT_MAX;
            for (int q = 0; q < KB / 32; ++q) m = min(m, iscr[q]);
            emin_slot = m;
        }
        cl.sync();
        int cmn = INT_MAX;
        for (int q = 0; q < CL; ++q) cmn = min(cmn, *cl.map_shared_rank(&emin_slot, q));
        if (cmn == INT_MAX) cmn = 0;
        const int kused = a.bin_exp[a.dim * N];
        for (int i = tid; i < nb; i += KB) {
            const int e = eb[i] != INT_MIN ? eb[i] : cmn;
            a.bin_exp[(size_t)d * N + i0 + i] = e + 2 * kused;
        }
    }
    cl.sync();   // keep shared memory alive until every CTA has read it
}

__global__ void __cluster_dims__(CL, 1, 1) __launch_bounds__(KB) k4_refine(cvg_refine_args a)
{
    k4_refine_dev(a, blockIdx.x / CL);
}

// ---------------------------------------------------------------------------
// Batched forms: one launch covers the blocks (or clusters) of every
// instance.  A reallocation block finds its instance in a block-to-instance
// table; a refinement cluster by binary search over the prefix of
// dimensions per instance.
// ---------------------------------------------------------------------------
__device__ __forceinline__ int find_inst(const unsigned *base, int n, unsigned b)
{
    int lo = 0, hi = n - 1;
    while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if (base[mid] <= b) lo = mid; else hi = mid - 1;
    }
    return lo;
}

// one form per launch (the batch's precision), 4 blocks per SM as k3_results_f32
template <bool FAST>
__global__ void __launch_bounds__(RB, 4) k3_results_b(cvg_realloc_batch B)
{
    const int i = (int)B.blk_inst[blockIdx.x];
    const cvg_realloc_args &a = B.A[i];
    if (FAST) k3_results_f32_dev<RIPT, true>(a, blockIdx.x - B.blk_base[i]);
    else k3_results_dev(a, blockIdx.x - B.blk_base[i]);
    const unsigned nb = B.blk_base[i + 1] - B.blk_base[i];
    if (last_block(&a.done[0], nb)) k3_finish_dev(a, nb);
}



// One-pass allocation of every instance: a block's chunk within its
// instance comes from the instance's ticket, so the blocks an instance's
// look-back waits on have started before it.
template <int MODE>
__global__ void __launch_bounds__(RB, 8) k3_alloc_b(cvg_realloc_batch B)
{
    const int i = (int)B.blk_inst[blockIdx.x];
    const cvg_realloc_args &a = B.A[i];
    if (!a.adapt && MODE != 1) return;
    k3_alloc_dev<MODE>(a, B.blk_base[i + 1] - B.blk_base[i]);
}

__global__ void __cluster_dims__(CL, 1, 1) __launch_bounds__(KB) k4_refine_b(cvg_refine_batch B)
{
    const unsigned cid = blockIdx.x / CL;
    const int i = find_inst(B.dim_base, B.n, cid);
    if (B.keep_grid) {
        cvg_refine_args a = B.R[i];
        a.adapt = 0;
        k4_refine_dev(a, (int)(cid - B.dim_base[i]));
    } else {
        k4_refine_dev(B.R[i], (int)(cid - B.dim_base[i]));
    }
}

// Estimated cost of one tile of a dimension-D instance in the batched fill:
// its time per sample, measured on product-peak instances of d = 2..12, grows
// by about 1/20 of the d = 2 time per added dimension.  The fill's claims
// correct what this estimate misses.
__device__ __forceinline__ cvg_u64 cvg_batch_tile_cost(int dim) { return (cvg_u64)dim + 20u; }

// Work split of the next batched fill.  tile_base[i] = first global tile of
// instance i, tile_base[n] = total (tiles per instance clamped to the
// capacity of its tile map); cost_base the same prefix over tile costs.  The
// cost-weighted tile sequence is cut into n_ranges equal parts: range r
// starts at the first tile whose cost prefix is >= C*r/n_ranges, so the
// ranges are contiguous, ordered and cover every tile once.  One CTA of the
// fill owns each range; the claim counters start at zero.
__global__ void __launch_bounds__(1024) k_tile_base(cvg_realloc_batch B, cvg_batch_sched S)
{
    __shared__ cvg_u64 wt[32], wc[32];
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5, nw = blockDim.x >> 5;
    cvg_u64 carry_t = 0, carry_c = 0;
    for (int b0 = 0; b0 < B.n; b0 += blockDim.x) {
        const int i = b0 + threadIdx.x;
        cvg_u64 nt = 0, nc = 0;
        if (i < B.n) {
            const cvg_realloc_args &a = B.A[i];
            const cvg_u64 Sm = a.nh_sum[a.n_cubes], TS = (cvg_u64)a.tile_samples;
            nt = (Sm + TS - 1) / TS;
            if (nt > a.max_tiles) nt = a.max_tiles;
            nc = nt * cvg_batch_tile_cost(a.dim);
        }
        // block-wide inclusive scan of (nt, nc)
        cvg_u64 st = nt, sc = nc;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const cvg_u64 ut = __shfl_up_sync(0xffffffffu, st, o), uc = __shfl_up_sync(0xffffffffu, sc, o);
            if (lane >= o) { st += ut; sc += uc; }
        }
        if (lane == 31) { wt[w] = st; wc[w] = sc; }
        __syncthreads();
        if (w == 0) {
            cvg_u64 xt = lane < nw ? wt[lane] : 0, xc = lane < nw ? wc[lane] : 0;
#pragma unroll
            for (int o = 1; o < 32; o <<= 1) {
                const cvg_u64 ut = __shfl_up_sync(0xffffffffu, xt, o), uc = __shfl_up_sync(0xffffffffu, xc, o);
                if (lane >= o) { xt += ut; xc += uc; }
            }
            if (lane < nw) { wt[lane] = xt; wc[lane] = xc; }
        }
        __syncthreads();
        const cvg_u64 pt = carry_t + (w ? wt[w - 1] : 0) + st - nt;
        const cvg_u64 pc = carry_c + (w ? wc[w - 1] : 0) + sc - nc;
        if (i < B.n) { S.tile_base[i] = pt; S.cost_base[i] = pc; }
        carry_t += wt[nw - 1];
        carry_c += wc[nw - 1];
        __syncthreads();   // wt / wc are rewritten by the next chunk
    }
    if (threadIdx.x == 0) { S.tile_base[B.n] = carry_t; S.cost_base[B.n] = carry_c; }
    __syncthreads();
    const cvg_u64 C = carry_c, R = (cvg_u64)S.n_ranges;
    for (int r = threadIdx.x; r <= S.n_ranges; r += blockDim.x) {
        if (r == S.n_ranges) { S.range_start[r] = carry_t; break; }
        // c = floor(C * r / R) without overflow
        const cvg_u64 c = (C / R) * (cvg_u64)r + (C % R) * (cvg_u64)r / R;
        int lo = 0, hi = B.n - 1;                  // last instance with cost_base <= c
        while (lo < hi) {
            const int mid = (lo + hi + 1) >> 1;
            if (S.cost_base[mid] <= c) lo = mid; else hi = mid - 1;
        }
        const cvg_u64 wc1 = cvg_batch_tile_cost(B.A[lo].dim);
        const cvg_u64 lt = (c - S.cost_base[lo] + wc1 - 1) / wc1;
        S.range_start[r] = S.tile_base[lo] + lt;
        S.range_inst[r] = (cvg_u32)lo;
        S.claim[r] = 0;
    }
}

__global__ void grid32(const double *x, float *x32, int n)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) x32[i] = (float)x[i];
}

__global__ void fill_u32(cvg_u32 *p, cvg_u32 v, cvg_u64 n)
{
    for (cvg_u64 i = blockIdx.x * (cvg_u64)blockDim.x + threadIdx.x; i < n;
         i += (cvg_u64)gridDim.x * blockDim.x)
        p[i] = v;
}

// 8 independent FMA chains per thread; result kept live through `sink`.
template <typename T>
__global__ void __launch_bounds__(256) fma_bench(int iters, double *sink)
{
    T a[8];
    const T m = (T)0.999999, c = (T)1e-7;
#pragma unroll
    for (int i = 0; i < 8; ++i) a[i] = (T)(threadIdx.x + i);
    for (int k = 0; k < iters; ++k) {
#pragma unroll
        for (int i = 0; i < 8; ++i) a[i] = a[i] * m + c;
    }
    T s = (T)0;
#pragma unroll
    for (int i = 0; i < 8; ++i) s += a[i];
    if (s == (T)-1.2345) sink[0] = (double)s;
}

// Pipe throughput microbenchmarks for the fill's roofline (8 independent
// chains per thread, 256 threads, 8 CTAs per SM).
// INT32 multiply-add (the sampler's and the bin arithmetic's integer work).
__global__ void __launch_bounds__(256) int_bench(int iters, double *sink)
{
    cvg_u32 a[8];
#pragma unroll
    for (int i = 0; i < 8; ++i) a[i] = threadIdx.x * 7u + (cvg_u32)i;
    const cvg_u32 m = 0x9E3779B1u, c = blockIdx.x | 1u;
    for (int k = 0; k < iters; ++k) {
#pragma unroll
        for (int i = 0; i < 8; ++i) a[i] = a[i] * m + c;
    }
    cvg_u32 s = 0;
#pragma unroll
    for (int i = 0; i < 8; ++i) s ^= a[i];
    if (s == 0x12345678u) sink[0] = (double)s;
}
// Special-function unit: ex2.approx (the integrands' exp).
__global__ void __launch_bounds__(256) sfu_bench(int iters, double *sink)
{
    float a[8];
#pragma unroll
    for (int i = 0; i < 8; ++i) a[i] = 0.001f * (float)(threadIdx.x + i);
    for (int k = 0; k < iters; ++k) {
#pragma unroll
        for (int i = 0; i < 8; ++i) {
            float r;
            asm volatile("ex2.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(a[i]));
            a[i] = r - 1.0f;
        }
    }
    float s = 0.f;
#pragma unroll
    for (int i = 0; i < 8; ++i) s += a[i];
    if (s == -1.2345f) sink[0] = (double)s;
}
// Philox4x32-10 calls (the sampler: one call per 4 dimensions of a sample).
__global__ void __launch_bounds__(256) philox_bench(int iters, double *sink)
{
    cvg_u32 acc = 0;
    const cvg_u32 t = blockIdx.x * blockDim.x + threadIdx.x;
    for (int k = 0; k < iters; ++k) {
#pragma unroll
        for (int i = 0; i < 4; ++i) {
            const cvg_u32x4 r = cvg_philox((cvg_u32)k, t, (cvg_u32)i, 7u, 0x1234u, 0x5678u);
            acc ^= r.x ^ r.y ^ r.z ^ r.w;
        }
    }
    if (acc == 0x12345678u) sink[0] = (double)acc;
}

// Shared-memory atomic throughput: every thread adds to random words of a
// 4096-word table (the access pattern of the fill's bin histograms).
template <typename V>
__global__ void __launch_bounds__(512) smem_atomic_bench(int iters, double *sink)
{
    __shared__ V tab[4096];
    for (int i = threadIdx.x; i < 4096; i += blockDim.x) tab[i] = (V)0;
    __syncthreads();
    cvg_u32 x = threadIdx.x * 2654435761u + blockIdx.x * 40503u + 1u;
    for (int k = 0; k < iters; ++k) {
        x ^= x << 13; x ^= x >> 17; x ^= x << 5;
        atomicAdd(&tab[x & 4095u], (V)1);
    }
    __syncthreads();
    if (threadIdx.x == 0 && (double)tab[7] == -1.0) sink[0] = 1.0;
}

__global__ void copy_bench(const float4 *__restrict__ src, float4 *__restrict__ dst, size_t n)
{
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n;
         i += (size_t)gridDim.x * blockDim.x)
        dst[i] = src[i];
}

}  // namespace

cudaError_t cvg_launch_fma_bench(int kind, int blocks, int iters, double *sink, cudaStream_t s)
{
    if (kind == 0) fma_bench<float><<<blocks, 256, 0, s>>>(iters, sink);
    else fma_bench<double><<<blocks, 256, 0, s>>>(iters, sink);
    return cudaGetLastError();
}

cudaError_t cvg_launch_pipe_bench(int kind, int blocks, int iters, double *sink, cudaStream_t s)
{
    if (kind == 0) int_bench<<<blocks, 256, 0, s>>>(iters, sink);
    else if (kind == 1) sfu_bench<<<blocks, 256, 0, s>>>(iters, sink);
    else philox_bench<<<blocks, 256, 0, s>>>(iters, sink);
    return cudaGetLastError();
}

// The fill's per-(dimension, bin) histogram update in its two forms: MODE 0
// = float atomicAdd of the weight + u32 count; MODE 1 = u32 fixed-point add
// whose wrap carries into a global FP64 word + u32 count.  Lanes of a warp
// draw bins from a 128-bin window, as samples of one stratum do.
template <int MODE>
__global__ void __launch_bounds__(512) hist_update_bench(int iters, double *gw)
{
    __shared__ cvg_u32 lo[4096];
    __shared__ cvg_u32 cn[4096];
    for (int i = threadIdx.x; i < 4096; i += blockDim.x) { lo[i] = 0u; cn[i] = 0u; }
    __syncthreads();
    cvg_u32 x = threadIdx.x * 2654435761u + blockIdx.x * 40503u + 1u;
    const cvg_u32 base = ((threadIdx.x >> 5) * 128u) & 4095u;
    for (int it = 0; it < iters; ++it) {
        x ^= x << 13; x ^= x >> 17; x ^= x << 5;
        const cvg_u32 i = (base + (x & 127u) + (cvg_u32)it * 512u) & 4095u;
        const float w = __uint_as_float(0x3F800000u | (x >> 9)) - 0.5f;   // [0.5, 1.5)
        if (MODE == 0) {
            atomicAdd(reinterpret_cast<float *>(&lo[i]), w);
        } else {
            const cvg_u32 q = __float_as_uint(__fadd_rn(w * 65536.f, 8388608.f)) - 0x4B000000u;
            const cvg_u32 o = atomicAdd(&lo[i], q);
            if (o + q < o) atomicAdd(&gw[i], 65536.0);
        }
        atomicAdd(&cn[i], 1u);
    }
    __syncthreads();
    if (threadIdx.x == 0 && lo[5] == 0xFFFFFFFFu && cn[3] == 7u) gw[0] = -1.0;
}

cudaError_t cvg_launch_hist_update_bench(int mode, int blocks, int iters, double *gw, cudaStream_t s)
{
    if (mode == 0) hist_update_bench<0><<<blocks, 512, 0, s>>>(iters, gw);
    else hist_update_bench<1><<<blocks, 512, 0, s>>>(iters, gw);
    return cudaGetLastError();
}

cudaError_t cvg_launch_smem_atomic_bench(int kind, int blocks, int iters, double *sink,
                                         cudaStream_t s)
{
    if (kind == 0) smem_atomic_bench<float><<<blocks, 512, 0, s>>>(iters, sink);
    else if (kind == 1) smem_atomic_bench<cvg_u32><<<blocks, 512, 0, s>>>(iters, sink);
    else if (kind == 2) smem_atomic_bench<cvg_u64><<<blocks, 512, 0, s>>>(iters, sink);
    else smem_atomic_bench<double><<<blocks, 512, 0, s>>>(iters, sink);
    return cudaGetLastError();
}

cudaError_t cvg_launch_copy_bench(const float4 *src, float4 *dst, size_t n, cudaStream_t s)
{
    copy_bench<<<152 * 8, 512, 0, s>>>(src, dst, n);
    return cudaGetLastError();
}

cudaError_t cvg_launch_realloc(const cvg_realloc_args &a, cudaStream_t s)
{
    const unsigned nb = cvg_realloc_blocks(a.n_cubes);
    // + finish in the last block.  Runs with few hypercubes take 2 per thread
    // (4x the blocks): the results kernel is then latency-bound, not
    // bandwidth-bound (d=4, 1e6 evaluations, 234k hypercubes)
    if (a.small_chunks && a.n_cubes <= CVG_REALLOC_SMALL_CUBES) {
        const unsigned nb2 = (a.n_cubes + RB * 2 - 1) / (RB * 2);
        if (a.fast_pow) k3_results_f32<2><<<nb2, RB, 0, s>>>(a);
        else k3_results<2><<<nb2, RB, 0, s>>>(a);
    } else if (a.fast_pow) {
        k3_results_f32<RIPT><<<nb, RB, 0, s>>>(a);
    } else {
        k3_results<RIPT><<<nb, RB, 0, s>>>(a);
    }
    if (a.adapt) {
        if (a.lb) {   // one pass: count, scan and apply
            if (a.fast_pow) k3_alloc<2><<<nb, RB, 0, s>>>(a, nb);
            else k3_alloc<0><<<nb, RB, 0, s>>>(a, nb);
        } else {
            k3_count<<<nb, RB, 0, s>>>(a, a.fast_pow ? 2 : 0);    // + scan in the last block
            k3_apply<<<nb, RB, 0, s>>>(a, nb);
        }
    }
    return cudaGetLastError();
}

// Sum of JF2 over all hypercubes (FP64, one atomic per block); the last block
// turns it into the FP32 reallocation's scale exponent: 2^(2k) ~ the mean of
// (f*jac)^2 over the iteration's samples, as k3_finish_dev sets it after each
// iteration of the loop.
__global__ void __launch_bounds__(RB) k3_scale_from_sums(const double *JF2, const cvg_u64 *nh_sum,
                                                        cvg_u32 n_cubes, double *ss,
                                                        cvg_u32 *ticket, int *scale_exp)
{
    __shared__ double scratch[32];
    double v[1] = {0.0};
    for (cvg_u64 c = (cvg_u64)blockIdx.x * RB + threadIdx.x; c < n_cubes; c += (cvg_u64)gridDim.x * RB)
        v[0] += JF2[c];
    block_sum<1>(v, scratch);
    if (threadIdx.x == 0) atomicAdd(ss, v[0]);
    if (last_block(ticket, gridDim.x) && threadIdx.x == 0) {
        const double S = (double)nh_sum[n_cubes];
        const double ms = S > 0.0 ? *(volatile double *)ss / S : 0.0;
        int k = 0;
        if (ms > 0.0 && isfinite(ms)) {
            int e = 0;
            frexp(ms, &e);
            k = e / 2;
            k = k < -100 ? -100 : (k > 100 ? 100 : k);
        }
        *scale_exp = k;
        *ss = 0.0;
    }
}

cudaError_t cvg_launch_scale_from_sums(const double *JF2, const cvg_u64 *nh_sum, cvg_u32 n_cubes,
                                       double *ss, cvg_u32 *ticket, int *scale_exp, cudaStream_t s)
{
    const unsigned nb = cvg_realloc_blocks(n_cubes);
    k3_scale_from_sums<<<nb < 304u ? nb : 304u, RB, 0, s>>>(JF2, nh_sum, n_cubes, ss, ticket,
                                                          scale_exp);
    return cudaGetLastError();
}

cudaError_t cvg_launch_set_nh(const cvg_realloc_args &a_in, const cvg_u32 *nh, cudaStream_t s)
{
    cvg_realloc_args a = a_in;
    a.lb_withhold = 0;   // the failure test's withheld word applies to reallocations only
    const unsigned nb = cvg_realloc_blocks(a.n_cubes);
    if (nh != a.nh_new) {
        cudaError_t e = cudaMemcpyAsync(a.nh_new, nh, sizeof(cvg_u32) * a.n_cubes,
                                        cudaMemcpyDefault, s);
        if (e != cudaSuccess) return e;
    }
    if (a.lb) {
        k3_alloc<1><<<nb, RB, 0, s>>>(a, nb);
    } else {
        k3_count<<<nb, RB, 0, s>>>(a, 1);
        k3_apply<<<nb, RB, 0, s>>>(a, nb);
    }
    return cudaGetLastError();
}

cudaError_t cvg_launch_refine(const cvg_refine_args &a, cudaStream_t s)
{
    const size_t smem = k4_smem_bytes(a.n_intervals);
    if (smem > 48 * 1024) {
        cudaError_t e = cudaFuncSetAttribute(k4_refine, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                             (int)smem);
        if (e != cudaSuccess) return e;
    }
    k4_refine<<<a.dim * CL, KB, smem, s>>>(a);
    return cudaGetLastError();
}

cudaError_t cvg_launch_grid32(const double *x, float *x32, int n, cudaStream_t s)
{
    grid32<<<(n + 255) / 256, 256, 0, s>>>(x, x32, n);
    return cudaGetLastError();
}

cudaError_t cvg_launch_fill_u32(cvg_u32 *p, cvg_u32 v, cvg_u64 n, cudaStream_t s)
{
    if (n == 0) return cudaSuccess;
    cvg_u64 blocks = (n + 255) / 256;
    if (blocks > 4096) blocks = 4096;
    fill_u32<<<(unsigned)blocks, 256, 0, s>>>(p, v, n);
    return cudaGetLastError();
}

cudaError_t cvg_launch_realloc_batch(const cvg_realloc_batch &B, int adapt, bool fast,
                                     const cvg_batch_sched &S, cudaStream_t s)
{
    if (fast) k3_results_b<true><<<B.total_blocks, RB, 0, s>>>(B);    // + finish per instance
    else k3_results_b<false><<<B.total_blocks, RB, 0, s>>>(B);
    if (adapt) {
        if (fast) k3_alloc_b<2><<<B.total_blocks, RB, 0, s>>>(B);
        else k3_alloc_b<0><<<B.total_blocks, RB, 0, s>>>(B);
    }
    k_tile_base<<<1, 1024, 0, s>>>(B, S);
    return cudaGetLastError();
}

cudaError_t cvg_launch_set_nh_batch(const cvg_realloc_batch &B, const cvg_batch_sched &S,
                                    cudaStream_t s)
{
    k3_alloc_b<1><<<B.total_blocks, RB, 0, s>>>(B);
    k_tile_base<<<1, 1024, 0, s>>>(B, S);
    return cudaGetLastError();
}

cudaError_t cvg_launch_refine_batch(const cvg_refine_batch &B, int n_intervals, cudaStream_t s)
{
    const size_t smem = k4_smem_bytes(n_intervals);
    if (smem > 48 * 1024) {
        cudaError_t e = cudaFuncSetAttribute(k4_refine_b, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                             (int)smem);
        if (e != cudaSuccess) return e;
    }
    k4_refine_b<<<B.total_dims * CL, KB, smem, s>>>(B);
    return cudaGetLastError();
}
