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

// d^beta for d > 0 through FP32 log2/exp2 with the binary exponent kept exact
// (relative error ~1e-6; used for the FP32 form's allocation only).
__device__ __forceinline__ double fast_pow_pos(double t, double beta)
{
    if (!(t > 0.0)) return 0.0;
    if (!(t < 1.0e300)) return pow(t, beta);
    int scale = 0;
    if (t < 1.0e-290) { t *= 18446744073709551616.0; scale = -64; }   // 2^64
    const int hi = __double2hiint(t), lo = __double2loint(t);
    const int e = ((hi >> 20) & 0x7ff) - 1023 + scale;
    const float m = __int_as_float(0x3F800000 | ((hi & 0xFFFFF) << 3) | ((unsigned)lo >> 29));
    const double y = beta * (double)e + (double)((float)beta * log2f(m));
    const double k = floor(y);
    const float f = exp2f((float)(y - k));           // in [1, 2)
    return ldexp((double)f, (int)k);
}

__global__ void __launch_bounds__(RB) k3_results(cvg_realloc_args a)
{
    __shared__ double scratch[3 * 32];
    const cvg_u32 base = blockIdx.x * CVG_REALLOC_CHUNK;
    double v[3] = {0.0, 0.0, 0.0};   // dh, I, sigma2
    const double vc = a.v_cubes;
    for (int k = 0; k < RIPT; ++k) {
        const cvg_u32 c = base + k * RB + threadIdx.x;
        if (c >= a.n_cubes) break;
        const int neval = (int)(a.nh_sum[c + 1] - a.nh_sum[c]);
        const double jf = a.JF[c], jf2 = a.JF2[c];
        a.JF[c] = 0.0;
        a.JF2[c] = 0.0;
        double dh;
        if (!a.fast_pow) {
            // src/main.cu:88-102, same operation order
            const double Ih = jf / neval * vc;
            const double Sig2 = (jf2 / neval * vc * vc) - (Ih * Ih);
            v[1] += Ih;
            v[2] += Sig2 / neval;
            const double m = vc * jf / neval;
            double t = vc * vc * jf2 / neval - m * m;
            if (t < 0) t = 0;
            dh = pow(t, a.beta);
        } else {
            const double inv = 1.0 / (double)neval;
            const double Ih = jf * inv * vc;
            const double Sig2 = jf2 * inv * vc * vc - Ih * Ih;
            v[1] += Ih;
            v[2] += Sig2 * inv;
            double t = Sig2;
            if (t < 0) t = 0;
            dh = fast_pow_pos(t, a.beta);
        }
        a.dh[c] = dh;
        v[0] += dh;
    }
    block_sum<3>(v, scratch);
    if (threadIdx.x == 0) {
        a.partials[3 * blockIdx.x + 0] = v[0];
        a.partials[3 * blockIdx.x + 1] = v[1];
        a.partials[3 * blockIdx.x + 2] = v[2];
    }
}

__global__ void __launch_bounds__(1024) k3_finish(cvg_realloc_args a, unsigned nb)
{
    __shared__ double scratch[3 * 32];
    double v[3] = {0.0, 0.0, 0.0};
    for (unsigned i = threadIdx.x; i < nb; i += blockDim.x) {
        v[0] += a.partials[3 * i + 0];
        v[1] += a.partials[3 * i + 1];
        v[2] += a.partials[3 * i + 2];
    }
    block_sum<3>(v, scratch);
    if (threadIdx.x == 0) {
        const cvg_u32 it = *a.iteration;
        const double r = v[1], s = v[2];
        if ((int)it < a.max_it) {
            a.stats[it] = r;
            a.stats[a.max_it + it] = s;
            a.stats[2 * a.max_it + it] = (double)a.nh_sum[a.n_cubes];
        }
        cvg_acc_dev *acc = a.acc;
        acc->dh_sum = v[0];
        const cvg_u64 S = a.nh_sum[a.n_cubes];
        acc->tot_nevals += S;
        acc->last_nevals = S;
        if ((int)it >= a.skip) {   // src/main.cu:680, 698-713
            acc->sw += 1.0 / s;
            acc->swr += r / s;
            acc->swr2 += r * r / s;
            acc->used += 1;
        }
        if (!isfinite(r) || !isfinite(s)) atomicOr(a.status, CVG_KSTAT_NONFINITE);
        *a.iteration = it + 1;
    }
}

// mode 0: nh from the damped variances (updateNh, src/main.cu:173-187)
// mode 1: nh_new already holds the counts (initialisation / state import)
__global__ void __launch_bounds__(RB) k3_count(cvg_realloc_args a, int mode)
{
    __shared__ double scratch[32];
    const cvg_u32 base = blockIdx.x * CVG_REALLOC_CHUNK;
    const double dsum = a.acc->dh_sum;
    const double n_it = (double)a.n_eval_it;
    double tot = 0.0;   // counts are exact in double (< 2^53)
    for (int k = 0; k < RIPT; ++k) {
        const cvg_u32 c = base + k * RB + threadIdx.x;
        if (c >= a.n_cubes) break;
        cvg_u32 nh;
        if (mode == 0) {
            const double f = a.dh[c] / dsum;
            const double x = f * n_it;
            // (int) conversion of the reference: NaN -> 0, saturating above
            int ns = (x >= 0.0 && x < 2147483647.0) ? (int)x : (x >= 2147483647.0 ? 2147483647 : 0);
            nh = ns < 2 ? 2u : (cvg_u32)ns;
            a.nh_new[c] = nh;
        } else {
            nh = a.nh_new[c];
        }
        tot += (double)nh;
    }
    double v[1] = {tot};
    block_sum<1>(v, scratch);
    if (threadIdx.x == 0) a.bsums[blockIdx.x] = (cvg_u64)v[0];
}

__global__ void __launch_bounds__(1024) k3_scan(cvg_realloc_args a, unsigned nb)
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

__global__ void __launch_bounds__(RB) k3_apply(cvg_realloc_args a, unsigned nb)
{
    __shared__ cvg_u32 sh[CVG_REALLOC_CHUNK];
    __shared__ cvg_u64 st[CVG_REALLOC_CHUNK];
    __shared__ cvg_u64 scratch[33];
    const cvg_u32 base = blockIdx.x * CVG_REALLOC_CHUNK;
    const cvg_u32 cnt = min((cvg_u32)CVG_REALLOC_CHUNK, a.n_cubes - base);
    for (int i = threadIdx.x; i < CVG_REALLOC_CHUNK; i += RB)
        sh[i] = (cvg_u32)i < cnt ? a.nh_new[base + i] : 0u;
    __syncthreads();
    cvg_u64 local = 0;
#pragma unroll
    for (int k = 0; k < RIPT; ++k) local += sh[threadIdx.x * RIPT + k];
    cvg_u64 off = local;
    block_exscan_u64(off, scratch);
    off += a.bsums[blockIdx.x];
    const cvg_u64 TS = (cvg_u64)a.tile_samples;
#pragma unroll 1
    for (int k = 0; k < RIPT; ++k) {
        const int i = threadIdx.x * RIPT + k;
        const cvg_u64 n = sh[i];
        st[i] = off;
        if ((cvg_u32)i < cnt) {
            const cvg_u32 c = base + i;
            for (cvg_u64 t = (off + TS - 1) / TS; t * TS < off + n && t < a.max_tiles; ++t)
                a.tile_cube[t] = c;
        }
        off += n;
    }
    __syncthreads();
    for (int i = threadIdx.x; i < (int)cnt; i += RB) a.nh_sum[base + i] = st[i];
    if (blockIdx.x == nb - 1 && threadIdx.x == 0) a.nh_sum[a.n_cubes] = a.bsums[nb];
}

// ---------------------------------------------------------------------------
// K4: grid refinement, one CTA per dimension, FP64.
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(CVG_REFINE_BLOCK) k4_refine(cvg_refine_args a)
{
    extern __shared__ __align__(16) double ks[];
    __shared__ double scratch[32];
    const int N = a.n_intervals, d = blockIdx.x, tid = threadIdx.x, bs = blockDim.x;
    double *w = ks, *sw = ks + N, *cs = ks + 2 * N, *xo = ks + 3 * N;
    int *dv = (int *)(xo + N + 1);
    double *xe = a.x_edges + (size_t)d * (N + 1);
    float *xe32 = a.x_edges32 + (size_t)d * (N + 1);

    // normalizeWeights (src/main.cu:106-118) + resetWeights (147-158)
    double part = 0.0;
    for (int i = tid; i < N; i += bs) {
        const size_t g = (size_t)d * N + i;
        const double wi = a.weights[g];
        const cvg_u32 cn = a.counts[g];
        const double x = cn != 0u ? wi / (double)cn : wi;
        w[i] = x;
        part += x;
        a.weights[g] = 0.0;
        a.counts[g] = 0u;
    }
    for (int i = tid; i <= N; i += bs) xo[i] = xe[i];
    double v[1] = {part};
    block_sum<1>(v, scratch);          // d_sum (src/main.cu:668-670)
    const double dsum = v[0];
    bool ok = a.adapt && dsum > 0.0 && isfinite(dsum);

    if (ok) {
        // smoothWeights (src/main.cu:120-145)
        double p2 = 0.0;
        for (int i = tid; i < N; i += bs) {
            double t;
            if (i == 0) t = (7.0 * w[0] + w[1]) / (8.0 * dsum);
            else if (i == N - 1) t = (w[i - 1] + 7.0 * w[i]) / (8.0 * dsum);
            else t = (w[i - 1] + 6.0 * w[i] + w[i + 1]) / (8.0 * dsum);
            if (t != 0) t = pow((t - 1.0) / log(t), a.alpha);
            sw[i] = t;
            p2 += t;
        }
        v[0] = p2;
        block_sum<1>(v, scratch);      // summed_weights (src/main.cu:673-675)
        const double ssum = v[0];
        ok = ssum > 0.0 && isfinite(ssum);
        if (ok) {
            // inclusive scan (src/main.cu:688-690): each thread a contiguous run
            const int per = (N + bs - 1) / bs;
            const int i0 = tid * per;
            double loc = 0.0;
            for (int k = 0; k < per && i0 + k < N; ++k) loc += sw[i0 + k];
            // exclusive scan of the per-thread totals (doubles)
            const int lane = tid & 31, warp = tid >> 5, nw = bs >> 5;
            double x = loc;
#pragma unroll
            for (int o = 1; o < 32; o <<= 1) {
                const double y = __shfl_up_sync(0xffffffffu, x, o);
                if (lane >= o) x += y;
            }
            if (lane == 31) scratch[warp] = x;
            __syncthreads();
            if (tid == 0) {
                double s = 0.0;
                for (int q = 0; q < nw; ++q) { const double t = scratch[q]; scratch[q] = s; s += t; }
            }
            __syncthreads();
            double run = x - loc + scratch[warp];
            for (int k = 0; k < per && i0 + k < N; ++k) { run += sw[i0 + k]; cs[i0 + k] = run; }
            __syncthreads();
            const double delta = ssum / N;
            for (int i = tid; i < N; i += bs) dv[i] = (int)(cs[i] / delta);   // setMap div
            __syncthreads();
            // updateXEdges (src/main.cu:211-230): new edge k+1 lies in the old
            // interval o = min{ i : div_i > k }, the interval setMap assigns to k.
            for (int k = tid; k < N - 1; k += bs) {
                int lo = 0, hi = N - 1;
                while (lo < hi) {
                    const int mid = (lo + hi) >> 1;
                    if (dv[mid] > k) hi = mid; else lo = mid + 1;
                }
                const int o = lo;
                const double acc = (k + 1) * delta - (o > 0 ? cs[o - 1] : 0.0);
                const double xn = fma(acc / sw[o], xo[o + 1] - xo[o], xo[o]);
                xe[k + 1] = xn;
                xe32[k + 1] = (float)xn;
            }
        }
    }
    if (!ok)
        for (int i = tid; i <= N; i += bs) xe32[i] = (float)xo[i];
    else if (tid == 0) { xe32[0] = (float)xo[0]; xe32[N] = (float)xo[N]; }
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

cudaError_t cvg_launch_copy_bench(const float4 *src, float4 *dst, size_t n, cudaStream_t s)
{
    copy_bench<<<152 * 8, 512, 0, s>>>(src, dst, n);
    return cudaGetLastError();
}

cudaError_t cvg_launch_realloc(const cvg_realloc_args &a, cudaStream_t s)
{
    const unsigned nb = cvg_realloc_blocks(a.n_cubes);
    k3_results<<<nb, RB, 0, s>>>(a);
    k3_finish<<<1, 1024, 0, s>>>(a, nb);
    if (a.adapt) {
        k3_count<<<nb, RB, 0, s>>>(a, 0);
        k3_scan<<<1, 1024, 0, s>>>(a, nb);
        k3_apply<<<nb, RB, 0, s>>>(a, nb);
    }
    return cudaGetLastError();
}

cudaError_t cvg_launch_set_nh(const cvg_realloc_args &a, const cvg_u32 *nh, cudaStream_t s)
{
    const unsigned nb = cvg_realloc_blocks(a.n_cubes);
    if (nh != a.nh_new) {
        cudaError_t e = cudaMemcpyAsync(a.nh_new, nh, sizeof(cvg_u32) * a.n_cubes,
                                        cudaMemcpyDefault, s);
        if (e != cudaSuccess) return e;
    }
    k3_count<<<nb, RB, 0, s>>>(a, 1);
    k3_scan<<<1, 1024, 0, s>>>(a, nb);
    k3_apply<<<nb, RB, 0, s>>>(a, nb);
    return cudaGetLastError();
}

cudaError_t cvg_launch_refine(const cvg_refine_args &a, cudaStream_t s)
{
    const size_t smem = sizeof(double) * (4 * (size_t)a.n_intervals + 1) +
                        sizeof(int) * (size_t)a.n_intervals + 16;
    if (smem > 48 * 1024) {
        cudaError_t e = cudaFuncSetAttribute(k4_refine, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                             (int)smem);
        if (e != cudaSuccess) return e;
    }
    k4_refine<<<a.dim, CVG_REFINE_BLOCK, smem, s>>>(a);
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
