// cvg_fill.cuh -- the fused VEGAS+ fill: counter-based sampling, map through
// the adaptive grid, integrand, per-hypercube and per-bin accumulation.
//
// Replaces vegasFill of the reference (src/main.cu:20-79 and
// vegas_cuda/src/vegas_cuda_extension/cuda_kernel.cu:14-76) together with the
// evals[] expansion it depends on (mapCubes, src/main.cu:248-262), the curand
// state it carries (setup_kernel, src/main.cu:12-18) and the accumulator
// resets (src/main.cu:147-171).
//
// Work decomposition.  Samples of one iteration are numbered s = 0..S-1 in
// cube order (cube c owns [nh_sum[c], nh_sum[c+1])), exactly the order of the
// reference's evals[] array.  A persistent grid walks fixed-size tiles of
// tile_samples consecutive samples, each taken by one warp (warp tiles,
// claimed from a launch-wide counter) or by the whole CTA (block tiles, for
// small iterations); thread t of a tile owns spt consecutive
// samples, so a thread stays inside one cube for a run of samples and keeps
// Sum f*jac and Sum (f*jac)^2 of that run in registers (compensated in FP32).
// A run that starts and ends inside the thread's slice covers its whole cube
// and is stored; a run touching either end of the slice may be shared with a
// neighbour and is added with an FP64 atomic.  Per-bin Sum (f*jac)^2 and
// counts go to shared-memory histograms, added to the global FP64/u32
// histograms once per CTA at the end.
//
// The FP32 form issues no FP64-pipe instruction per sample: bins are found
// without float/int conversions and run sums are widened to FP64 by bit
// splicing before the (L2-executed) FP64 atomics.
//
// Expects cvg_common.cuh before inclusion.  The integrand comes in as a type
// F with static members  T f(T* x, const T* th)  and
// void df(T* x, const T* th, T* g)  (gradient w.r.t. theta; gradient pass).
#ifndef CVG_FILL_CUH
#define CVG_FILL_CUH

template <typename T> struct cvg_grid_src;
template <> struct cvg_grid_src<float> {
    static CVG_D const float *get(const cvg_fill_args &a) { return a.x_edges32; }
};
template <> struct cvg_grid_src<double> {
    static CVG_D const double *get(const cvg_fill_args &a) { return a.x_edges; }
};

// Running sum.  FP32: Kahan-compensated; FP64: plain.
template <typename T> struct cvg_acc;
template <> struct cvg_acc<float> {
    float s, k;
    CVG_D void reset() { s = 0.f; k = 0.f; }
    CVG_D void add(float x) { const float y = x - k; const float t = s + y; k = (t - s) - y; s = t; }
    CVG_D double value() const { return (double)s - (double)k; }
    CVG_D float value_t() const { return s - k; }
};
template <> struct cvg_acc<double> {
    double s;
    CVG_D void reset() { s = 0.0; }
    CVG_D void add(double x) { s += x; }
    CVG_D double value() const { return s; }
    CVG_D double value_t() const { return s; }
};

CVG_D float cvg_fma(float a, float b, float c) { return fmaf(a, b, c); }
CVG_D double cvg_fma(double a, double b, double c) { return fma(a, b, c); }

// float -> double by bit splicing (no FP64-pipe instruction): exact for
// normal numbers; zero and denormals give signed zero, inf/nan stay inf/nan.
CVG_D double cvg_f2d(float f)
{
    const cvg_u32 u = __float_as_uint(f);
    const cvg_u32 e = (u >> 23) & 0xFFu;
    const cvg_u32 sign = u & 0x80000000u;
    if (e == 0u) return __hiloint2double((int)sign, 0);
    if (e == 0xFFu) return __hiloint2double((int)(sign | 0x7FF00000u | ((u & 0x7FFFFFu) >> 3)), 0);
    const cvg_u32 hi = sign | ((e + 896u) << 20) | ((u & 0x7FFFFFu) >> 3);
    return __hiloint2double((int)hi, (int)(u << 29));
}
CVG_D double cvg_to_double(float f) { return cvg_f2d(f); }
CVG_D double cvg_to_double(double f) { return f; }

// f * 2^k widened to double by bit splicing (FP32 form: undoes the 2^-k
// scaling of f*jac; k = 0 for FP64).  Overflow gives inf, underflow zero.
CVG_D double cvg_to_double_scaled(float f, int k)
{
    const cvg_u32 u = __float_as_uint(f);
    const int e = (int)((u >> 23) & 0xFFu);
    const cvg_u32 sign = u & 0x80000000u;
    if (e == 0) return __hiloint2double((int)sign, 0);
    if (e == 0xFF) return __hiloint2double((int)(sign | 0x7FF00000u | ((u & 0x7FFFFFu) >> 3)), 0);
    const int E = e + 896 + k;
    if (E <= 0) return __hiloint2double((int)sign, 0);
    if (E >= 2047) return __hiloint2double((int)(sign | 0x7FF00000u), 0);
    return __hiloint2double((int)(sign | ((cvg_u32)E << 20) | ((u & 0x7FFFFFu) >> 3)), (int)(u << 29));
}
CVG_D double cvg_to_double_scaled(double f, int) { return f; }

// 2^-k as T (FP32 form scale of f*jac; 1 for FP64)
CVG_D float cvg_scale_pow2(float, int k)
{
    k = k < -126 ? -126 : (k > 126 ? 126 : k);
    return __int_as_float((127 - k) << 23);
}
CVG_D double cvg_scale_pow2(double, int) { return 1.0; }

// Bin of z = y*N (0 <= z <= N) and the fraction inside it:
// b = min(floor(z), N-1), frac = z - b (src/main.cu:49-52).  The FP32 form
// floors by a round-down add of 2^23 (no float/int conversion instruction).
CVG_D int cvg_bin(float z, int N, float fNm1, float &frac)
{
    const float C = 8388608.0f;
    const float bf = fminf(fmaxf(__fadd_rd(z, C) - C, 0.0f), fNm1);
    frac = z - bf;
    return __float_as_int(bf + C) - 0x4B000000;
}
// Same for z known to be positive (Philox samples): no lower clamp.  The
// clamp is taken on C + floor(z) against C + N - 1 (both exact), whose bits
// are also the bin index.
CVG_D int cvg_bin_pos(float z, float fNm1, float &frac)
{
    const float C = 8388608.0f;
    const float cb = fminf(__fadd_rd(z, C), C + fNm1);
    frac = z - (cb - C);
    return __float_as_int(cb) - 0x4B000000;
}

// FP32 map of one dimension from a Philox word r (src/main.cu:43-52, z = y*N
// formed from the uniform's significand t: z = t*zs + czs): bin b, mapped x
// and the Jacobian factor N*dx.  Gd is the dimension's edge table.
CVG_D void cvg_map_t(cvg_u32 r, float zs, float czs, float fN, float fNm1, const float *Gd,
                     float &x, int &b, float &jd)
{
    float frac;
    const float z = fmaf(cvg_uniform_t(r), zs, czs);
    b = cvg_bin_pos(z, fNm1, frac);
    const float e0 = Gd[b];
    const float dx = Gd[b + 1] - e0;
    x = fmaf(dx, frac, e0);
    jd = fN * dx;
}
// The same for two dimensions (Philox words ra, rb; edge tables Ga, Gb) in
// packed pairs: every result is bit-identical to two cvg_map_t calls.
CVG_D void cvg_map_t2(cvg_u32 ra, cvg_u32 rb, cvg_f32x2 zs2, cvg_f32x2 czs2, cvg_f32x2 fN2,
                      float fNm1, const float *Ga, const float *Gb, float &xa, float &xb,
                      int &ba, int &bb, float &ja, float &jb)
{
    const float C = 8388608.0f;
    const cvg_f32x2 C2 = cvg_pack2(C, C);
    const cvg_f32x2 z = cvg_fma2(cvg_pack2(cvg_uniform_t(ra), cvg_uniform_t(rb)), zs2, czs2);
    float ca, cb;
    cvg_unpack2(cvg_add2_rd(z, C2), ca, cb);
    ca = fminf(ca, C + fNm1);
    cb = fminf(cb, C + fNm1);
    const cvg_f32x2 frac = cvg_sub2(z, cvg_sub2(cvg_pack2(ca, cb), C2));
    ba = __float_as_int(ca) - 0x4B000000;
    bb = __float_as_int(cb) - 0x4B000000;
    const float e0a = Ga[ba], e0b = Gb[bb];
    const cvg_f32x2 e0 = cvg_pack2(e0a, e0b);
    const cvg_f32x2 dx = cvg_sub2(cvg_pack2(Ga[ba + 1], Gb[bb + 1]), e0);
    cvg_unpack2(cvg_fma2(dx, frac, e0), xa, xb);
    cvg_unpack2(cvg_mul2(fN2, dx), ja, jb);
}
CVG_D int cvg_bin(double z, int N, double, double &frac)
{
    int b = (int)z;
    b = b < N - 1 ? b : N - 1;
    b = b > 0 ? b : 0;
    frac = z - (double)b;
    return b;
}

// Per-bin histogram update in shared memory.
//
// FP32 form: shared-memory float atomics are not a single native operation
// on this GPU (measured: float adds to shared memory run at a quarter of the
// u32 rate), so the bin's Sum (f*jac)^2 is kept in fixed point in a u32 word
// and updated with the native integer atomic.  Each bin has its own scale:
// the top 8 bits of its count word hold a signed exponent e (set when the
// histogram is cleared; counts stay below 2^24 between flushes), and a weight
// w is added as round(w * 2^(16-e)) units.  e comes from the bin's expected
// per-sample weight, so every bin -- also one whose weights are 1e-12 of the
// core's -- is resolved to about 2^-16 of its typical sample.  A word that
// wraps adds its 2^32 units to the global FP64 sum; a weight at or above
// 2^(e+7) (or non-finite) goes to the global FP64 sum directly.
// FP64 form: FP64 atomics, sums in the reference's precision.
// The FP32 map runs dimension pairs as packed f32x2 instructions
// (CVG_FILL_PAIRS; the batched fill, which holds every dimension's variant in
// one kernel, keeps one dimension at a time).
#ifndef CVG_FILL_PAIRS
#define CVG_FILL_PAIRS 1
#endif
// The fixed-point histogram updates of a sample go in groups of
// CVG_HIST_GROUP dimensions (then 4, 2, 1): count atomics together, scale
// arithmetic in f32x2 pairs, rare updates of all dimensions behind one branch
// per sample.  Measured on GB300 (fill ms, d=8 Gaussian 1e8 / d=16 corner
// 1e9): scalar updates, a branch each 2.02 / 38.2; pairs, a branch per update
// 1.94 / 33.9; groups of 4, a branch per group - / 30.95; one branch per
// sample in groups of 4 1.875 / 30.52, of 8 1.869 / 29.57, of 16 - / 29.92.
#ifndef CVG_HIST_GROUP
#define CVG_HIST_GROUP 8
#endif
#define CVG_HIST_CNT_MASK 0x00FFFFFFu
// Fixed-point bin sums are used by the FP32 form up to this dimension;
// above it the shared-memory float atomics are kept.
#ifndef CVG_HIST_FIX_MAX_DIM
#define CVG_HIST_FIX_MAX_DIM 16
#endif
template <int D, typename T> CVG_D constexpr bool cvg_hist_fixed()
{
    return sizeof(T) == 4 && D <= CVG_HIST_FIX_MAX_DIM;
}

// Float-form update of bin i (shared-memory float atomic and count).
CVG_D void cvg_hist_add_float(float *hw, cvg_u32 *hc, int i, float w)
{
    atomicAdd(hw + i, w);
    atomicAdd(hc + i, 1u);
}
CVG_D void cvg_hist_add_float(double *hw, cvg_u32 *hc, int i, double w)
{
    atomicAdd(hw + i, w);
    atomicAdd(hc + i, 1u);
}
// 2^(16-e) for a bin exponent e in [-100, 100]: the float bits (143 - e) << 23
// formed as one integer multiply-add (FMA pipe) instead of an add and a shift
// (ALU, the fill's busiest pipe): measured 1.5 % off the d=8 fill.
CVG_D float cvg_pow2_16me(int e)
{
    int b;
    asm("mad.lo.s32 %0, %1, -8388608, 1199570944;" : "=r"(b) : "r"(e));
    return __int_as_float(b);
}
// Fixed-point update of bin i, with no branch and no select: adds
// u = round(w * 2^(16-e)) units to the bin's word.  Two cases are rare and are
// settled after all of a sample's updates, behind one branch (cvg_hist_rare):
//  * the weight does not fit (w >= 2^(e+7), or not finite): its u is >= 2^23
//    (for a non-finite w some large value); it is added all the same, OR-ed
//    into `big`, and the rare step takes it back out of the word;
//  * the word wraps: the carry out of the 32-bit add is shifted into `wraps`
//    by a carry chain (wraps = 2*wraps + carry), so after a sample's D
//    updates bit D-1-d says that dimension d's word wrapped (2^32 units more
//    go to the global FP64 sum).
// Every add and every take-back has its carry or borrow accounted for, so
// the global sum plus the word's final value is exactly the sum of the
// units that fitted: the same result as adding only those.  The rare step
// recomputes u from the bin's exponent (the top byte of its count word,
// fixed between flushes) by the same float operations.
CVG_D void cvg_hist_add_fix(float *hw, cvg_u32 *hc, int i, float w, cvg_u32 &wraps, cvg_u32 &big)
{
    const int e = (int)atomicAdd(hc + i, 1u) >> 24;          // this bin's scale exponent
    const float s = w * cvg_pow2_16me(e);                     // w * 2^(16-e)
    const cvg_u32 u = __float_as_uint(__fadd_rn(s, 8388608.0f)) - 0x4B000000u;
    const cvg_u32 o = atomicAdd(reinterpret_cast<cvg_u32 *>(hw) + i, u);
    asm("{\n\t.reg .u32 t;\n\tadd.cc.u32 t, %1, %2;\n\taddc.u32 %0, %0, %0;\n\t}"
        : "+r"(wraps) : "r"(o), "r"(u));
    big |= u;
}
// G updates (G even; bins i[0..G), one weight w), as cvg_hist_add_fix: all
// count atomics first, then the scale arithmetic in pairs, then the value
// atomics, so that G shared-memory round trips overlap.
template <int G>
CVG_D void cvg_hist_group(float *hw, cvg_u32 *hc, const int *i, float w, cvg_u32 &wraps,
                          cvg_u32 &big)
{
    const float C = 8388608.0f;
    int e[G];
    float q[G];
#pragma unroll
    for (int k = 0; k < G; ++k) e[k] = (int)atomicAdd(hc + i[k], 1u) >> 24;
#pragma unroll
    for (int k = 0; k < G; k += 2) {
        const cvg_f32x2 s2 = cvg_mul2(cvg_pack2(w, w),
                                      cvg_pack2(cvg_pow2_16me(e[k]), cvg_pow2_16me(e[k + 1])));
        cvg_unpack2(cvg_add2(s2, cvg_pack2(C, C)), q[k], q[k + 1]);
    }
#pragma unroll
    for (int k = 0; k < G; ++k) {
        const cvg_u32 u = __float_as_uint(q[k]) - 0x4B000000u;
        const cvg_u32 o = atomicAdd(reinterpret_cast<cvg_u32 *>(hw) + i[k], u);
        asm("{\n\t.reg .u32 t;\n\tadd.cc.u32 t, %1, %2;\n\taddc.u32 %0, %0, %0;\n\t}"
            : "+r"(wraps) : "r"(o), "r"(u));
        big |= u;
    }
}
// Dimensions d0..d0+G-1 of one sample (bins bin[], weight w) through
// cvg_hist_group.
template <int G>
CVG_D void cvg_fill_hist_group(float *hw, cvg_u32 *hc, int d0, int N, const int *bin, float w,
                               cvg_u32 &wraps, cvg_u32 &big)
{
    int i[G];
#pragma unroll
    for (int k = 0; k < G; ++k) i[k] = (d0 + k) * N + bin[d0 + k];
    cvg_hist_group<G>(hw, hc, i, w, wraps, big);
}
// The rare updates of one sample (see cvg_hist_add_fix): for each dimension
// whose word wrapped, 2^32 units (2^(16+e)) go to the global FP64 sum; for
// each whose units did not fit, the units are taken back out of the word
// (a borrow takes 2^32 units back from the global sum) and the weight itself
// goes to the global sum.  Returns the number of rare updates.
template <int D>
CVG_D cvg_u32 cvg_hist_rare(float *hw, const cvg_u32 *hc, double *gw, int N, const int *bin,
                            float w, cvg_u32 wraps)
{
    cvg_u32 n = 0;
#pragma unroll   // bin[] stays in registers (a loop indexing it would move it to the stack)
    for (int d = 0; d < D; ++d) {
        const int i = d * N + bin[d];
        const int e = (int)hc[i] >> 24;
        const double unit32 = __hiloint2double((1039 + e) << 20, 0);   // 2^32 units = 2^(16+e)
        bool rare = false;
        if ((wraps >> (D - 1 - d)) & 1u) {
            atomicAdd(gw + i, unit32);
            rare = true;
        }
        const cvg_u32 u = __float_as_uint(__fadd_rn(w * cvg_pow2_16me(e), 8388608.0f)) - 0x4B000000u;
        if (u >= 0x800000u) {
            const cvg_u32 o = atomicSub(reinterpret_cast<cvg_u32 *>(hw) + i, u);
            if (o < u) atomicAdd(gw + i, -unit32);
            atomicAdd(gw + i, cvg_f2d(w));
            rare = true;
        }
        n += rare ? 1u : 0u;
    }
    return n;
}
// Bin sum and count of a shared-memory histogram entry, in the units of the
// global histogram.
template <bool FIX>
CVG_D double cvg_hist_value(const float *hw, const cvg_u32 *hc, int i)
{
    if (!FIX) return cvg_f2d(hw[i]);
    // lo * 2^(e-16), exactly: (2^52 + lo) * 2^(e-68) - 2^(e-16), one FP64 add
    const int e = ((int)hc[i] >> 24) - 16;
    const cvg_u32 lo = reinterpret_cast<const cvg_u32 *>(hw)[i];
    return __hiloint2double((1075 + e) << 20, (int)lo) - __hiloint2double((1075 + e) << 20, 0);
}
template <bool FIX>
CVG_D double cvg_hist_value(const double *hw, const cvg_u32 *, int i) { return hw[i]; }
template <bool FIX> CVG_D cvg_u32 cvg_hist_count(cvg_u32 w) { return FIX ? (w & CVG_HIST_CNT_MASK) : w; }
// Cleared count word of bin i: with fixed point it carries the bin's scale
// exponent (unscaled exponent from the table minus 2k for the f*jac scaling).
template <bool FIX>
CVG_D cvg_u32 cvg_hist_word(const cvg_fill_args &a, int i, int kx, int shift)
{
    if (!FIX) return 0u;
    int e = a.bin_exp ? a.bin_exp[i] - 2 * kx + shift : 0;
    e = e < -100 ? -100 : (e > 100 ? 100 : e);
    return (cvg_u32)e << 24;
}

// Add a thread's run sums of cube c to the global per-cube sums.  When every
// lane of a full, converged warp holds a single run of the same cube (a
// hypercube with hundreds of samples or more, as the reallocation produces
// for peaked integrands), the warp first combines its runs -- in
// double-float for the FP32 form -- so one atomic pair replaces 32 on the
// same two addresses.
CVG_D void cvg_two_sum(float a, float b, float &s, float &e)
{
    s = a + b;
    const float bb = s - a;
    e = (a - (s - bb)) + (b - bb);
}
CVG_D void cvg_df_acc(float &h, float &l, float oh, float ol)
{
    float s, e;
    cvg_two_sum(h, oh, s, e);
    e += l + ol;
    h = s + e;
    l = e - (h - s);
}
CVG_D void cvg_run_to_global(const cvg_fill_args &a, cvg_u32 c, const cvg_acc<float> &a1,
                             const cvg_acc<float> &a2, int kx, bool whole)
{
    const unsigned m = __activemask();
    bool same = false;
    if (m == 0xffffffffu) {   // every lane executes both collectives
        const cvg_u32 c0 = __shfl_sync(m, c, 0);
        same = __all_sync(m, whole && c == c0);
    }
    if (same) {
        float h1 = a1.s, l1 = -a1.k, h2 = a2.s, l2 = -a2.k;
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) {
            const float oh1 = __shfl_xor_sync(m, h1, o), ol1 = __shfl_xor_sync(m, l1, o);
            const float oh2 = __shfl_xor_sync(m, h2, o), ol2 = __shfl_xor_sync(m, l2, o);
            cvg_df_acc(h1, l1, oh1, ol1);
            cvg_df_acc(h2, l2, oh2, ol2);
        }
        if ((threadIdx.x & 31) == 0) {
            atomicAdd(&a.JF[c], cvg_to_double_scaled(h1, kx) + cvg_to_double_scaled(l1, kx));
            atomicAdd(&a.JF2[c], cvg_to_double_scaled(h2, 2 * kx) + cvg_to_double_scaled(l2, 2 * kx));
        }
        return;
    }
    atomicAdd(&a.JF[c], cvg_to_double_scaled(a1.value_t(), kx));
    atomicAdd(&a.JF2[c], cvg_to_double_scaled(a2.value_t(), 2 * kx));
}
CVG_D void cvg_run_to_global(const cvg_fill_args &a, cvg_u32 c, const cvg_acc<double> &a1,
                             const cvg_acc<double> &a2, int, bool whole)
{
    const unsigned m = __activemask();
    double v1 = a1.value(), v2 = a2.value();
    bool same = false;
    if (m == 0xffffffffu) {   // every lane executes both collectives
        const cvg_u32 c0 = __shfl_sync(m, c, 0);
        same = __all_sync(m, whole && c == c0);
    }
    if (same) {
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) {
            v1 += __shfl_xor_sync(m, v1, o);
            v2 += __shfl_xor_sync(m, v2, o);
        }
        if ((threadIdx.x & 31) == 0) { atomicAdd(&a.JF[c], v1); atomicAdd(&a.JF2[c], v2); }
        return;
    }
    atomicAdd(&a.JF[c], v1);
    atomicAdd(&a.JF2[c], v2);
}

// Digits of the current cube in base n_strat.  With D >= 4 every digit is
// below 256 (n_strat^D < 2^32 hypercubes), so four share a register.
template <int D, bool PACK = (D >= 4)>
struct cvg_coords {
    int v[D];
    CVG_D void clear() {}
    CVG_D int get(int d) const { return v[d]; }
    CVG_D void set(int d, int x) { v[d] = x; }
};
template <int D>
struct cvg_coords<D, true> {
    cvg_u32 w[(D + 3) / 4];
    CVG_D void clear()
    {
#pragma unroll
        for (int k = 0; k < (D + 3) / 4; ++k) w[k] = 0u;
    }
    CVG_D int get(int d) const { return (int)((w[d >> 2] >> (8 * (d & 3))) & 0xFFu); }
    CVG_D void set(int d, int x)
    {
        const int sh = 8 * (d & 3);
        w[d >> 2] = (w[d >> 2] & ~(0xFFu << sh)) | ((cvg_u32)x << sh);
    }
};

// Stratum offsets coord_d * dy - sh of cube c (digit d of c in base n_strat,
// least significant first: src/main.cu:43-47); cvg_cube_next steps to cube
// c+1 like an odometer.  sh = 0 gives the reference's coord * dy.
template <int D, typename T>
CVG_D void cvg_cube_offsets(cvg_u32 c, cvg_u32 ns, T dy, T sh, cvg_coords<D> &co, T *cdy)
{
    co.clear();
#pragma unroll
    for (int d = 0; d < D; ++d) {
        const cvg_u32 q = c / ns;
        const int v = (int)(c - q * ns);
        co.set(d, v);
        cdy[d] = (T)v * dy - sh;
        c = q;
    }
}
template <int D, typename T>
CVG_D void cvg_cube_next(int ns, T dy, T sh, cvg_coords<D> &co, T *cdy)
{
    bool carry = true;
#pragma unroll
    for (int d = 0; d < D; ++d) {
        if (carry) {
            const int v = co.get(d) + 1;
            carry = v == ns;
            const int nv = carry ? 0 : v;
            co.set(d, nv);
            cdy[d] = (T)nv * dy - sh;
        }
    }
}

// Shared-memory views of one fill CTA, carved in the order of
// cvg_fill_smem_bytes: theta | bin sums | grid | bin counts | cube starts | scratch.
template <int D, typename T, bool ESM, bool HSM, int P, bool GRAD>
struct cvg_fill_smem {
    T *th, *hw, *E;
    cvg_u32 *hc;
    int *starts;
    double *red;
    CVG_D void carve(unsigned char *base, int N, int TS, int groups = 1)
    {
        constexpr bool H = HSM && !GRAD;
        cvg_u64 off = 0;
        th = (T *)(base + off);
        off += cvg_align16((cvg_u64)P * sizeof(T));
        hw = (T *)(base + off);
        if (H) off += cvg_align16((cvg_u64)D * N * sizeof(T));
        E = (T *)(base + off);
        if (ESM) off += cvg_align16((cvg_u64)D * (N + 1) * sizeof(T));
        hc = (cvg_u32 *)(base + off);
        if (H) off += cvg_align16((cvg_u64)D * N * 4);
        starts = (int *)(base + off);
        off += cvg_align16((cvg_u64)groups * (TS / 2 + 4) * 4);
        red = (double *)(base + off);
    }
};

// Per-instance constants of a fill CTA.
template <typename T>
struct cvg_fill_ctx {
    const T *G;
    cvg_u32 it, c3;
    int ns, N, kx;
    T dy, fN, fNm1, vc, jac0;
};

// Load theta and the grid into shared memory, clear the bin histograms and
// set the per-instance constants.  The caller synchronises afterwards.
template <int D, typename T, int BS, bool ESM, bool HSM, int P, bool GRAD, bool FIX>
CVG_D void cvg_fill_setup(const cvg_fill_args &a, const cvg_fill_smem<D, T, ESM, HSM, P, GRAD> &sm,
                          cvg_fill_ctx<T> &cx)
{
    constexpr bool H = HSM && !GRAD;
    const int N = a.n_intervals, tid = threadIdx.x;
    const T *grid = cvg_grid_src<T>::get(a);
    if (P > 0)
        for (int i = tid; i < P; i += BS) sm.th[i] = (T)a.theta[i];
    if (ESM)
        for (int i = tid; i < D * (N + 1); i += BS) sm.E[i] = grid[i];
    cx.G = ESM ? sm.E : grid;
    cx.it = *a.iteration;
    cx.c3 = a.instance << 8;
    cx.ns = a.n_strat;
    cx.N = N;
    cx.dy = (T)1 / (T)a.n_strat;
    cx.fN = (T)N;
    cx.fNm1 = (T)(N - 1);
    cx.vc = (T)a.v_cubes;
    // FP32 form: f*jac is carried as f*jac*2^-k so its square stays in range;
    // sums are widened back with the exponent shift (exact)
    cx.kx = (sizeof(T) == 4 && a.scale_exp) ? *a.scale_exp : 0;
    cx.jac0 = cvg_scale_pow2((T)0, cx.kx);
    if (H) {
        const int shift = (FIX && a.exp_shift) ? *a.exp_shift : 0;
        for (int i = tid; i < D * N; i += BS) {
            sm.hw[i] = (T)0;
            sm.hc[i] = cvg_hist_word<FIX>(a, i, cx.kx, shift);
        }
        // the refinement turns this fill's bin sums (units 2^-2k) back into
        // unscaled exponents for the next fill's table
        // (every CTA of the instance writes the same value)
        if (sizeof(T) == 4 && a.bin_exp && tid == 0) a.bin_exp[D * N] = cx.kx;
    }
}

// One tile: samples [tile*TS, min((tile+1)*TS, S)), taken by the whole CTA
// or (WT) by one warp.  Returns false (and sets a status bit) if the tile map
// is inconsistent; uniform across the block (warp).
template <bool WT> CVG_D void cvg_tile_sync()
{
    if (WT) __syncwarp(); else __syncthreads();
}
template <int D, typename T, int BS, bool ESM, bool HSM, bool REPLAY, int P, bool GRAD, class F,
          int NI, bool FIX, bool WT = false>
CVG_D bool cvg_fill_tile(const cvg_fill_args &a, const cvg_fill_smem<D, T, ESM, HSM, P, GRAD> &sm,
                         const cvg_fill_ctx<T> &cx, cvg_u64 tile, cvg_u64 n_tiles, cvg_u64 S,
                         cvg_acc<T> *gacc, cvg_u32 &nrare, const cvg_philox_keys &keys)
{
    constexpr int PP = P > 0 ? P : 1;
    constexpr int NB = (D + 3) / 4;
    constexpr bool H = HSM && !GRAD;
    constexpr int GS = WT ? 32 : BS;   // threads sharing the tile
    const int tid = WT ? (int)(threadIdx.x & 31) : (int)threadIdx.x;
    const int TS = a.tile_samples, N = NI > 0 ? NI : cx.N, ns = cx.ns;   // NI: bins fixed at compile time
    const T dy = cx.dy, fN = cx.fN, fNm1 = cx.fNm1;
    const T *G = cx.G;
    int *starts = sm.starts + (WT ? (int)(threadIdx.x >> 5) * (TS / 2 + 4) : 0);
    const cvg_u64 base = tile * (cvg_u64)TS;
    const cvg_u32 c_lo = a.tile_cube[tile];
    const cvg_u32 c_hi = (tile + 1 < n_tiles) ? a.tile_cube[tile + 1] : a.n_cubes - 1;
    if (c_hi < c_lo || c_hi >= a.n_cubes || (int)(c_hi - c_lo) > TS / 2 + 1) {
        if (tid == 0) atomicOr(a.status, CVG_KSTAT_BAD_TILE);
        return false;
    }
    const int K = (int)(c_hi - c_lo) + 2;
    for (int i = tid; i < K; i += GS)
        starts[i] = (int)((cvg_i64)a.nh_sum[c_lo + i] - (cvg_i64)base);
    cvg_tile_sync<WT>();

    const int spt = a.spt;
    const int l0 = tid * spt;
    const cvg_u64 rem = S - base;
    const int lend_tile = rem < (cvg_u64)TS ? (int)rem : TS;
    if (l0 < lend_tile) {
        int lo = 0, hi = K - 2;
        while (lo < hi) {
            const int mid = (lo + hi + 1) >> 1;
            if (starts[mid] <= l0) lo = mid; else hi = mid - 1;
        }
        int ci = lo;
        cvg_u32 c = c_lo + (cvg_u32)ci;
        int cstart = starts[ci];
        int next = starts[ci + 1];
        cvg_u32 j = (cvg_u32)(l0 - cstart);
        // FP32 form with Philox samples: z = y*N is formed directly from the
        // uniform's significand t in [1,2): z = t*(N/ns) + (coord - (1-2^-24))*(N/ns),
        // one FMA instead of shift, subtract, FMA and multiply
        constexpr bool ZF = sizeof(T) == 4 && !REPLAY;
        const T zs = ZF ? dy * fN : dy;
        const T zsh = ZF ? (T)0.99999994039535522461 * zs : (T)0;
#if CVG_FILL_PAIRS
        const cvg_f32x2 zs2 = cvg_pack2((float)zs, (float)zs), fN2 = cvg_pack2((float)fN, (float)fN);
#endif
        cvg_coords<D> coord;
        T cdy[D];
        cvg_cube_offsets<D, T>(c, (cvg_u32)ns, zs, zsh, coord, cdy);
        const int lend = min(l0 + spt, lend_tile);

        cvg_acc<T> a1, a2;
        a1.reset(); a2.reset();
        T ag[PP];
#pragma unroll
        for (int p = 0; p < PP; ++p) ag[p] = (T)0;
        int run = 0;   // samples in the current cube run

        for (int l = l0; l < lend; ++l) {
            if (l >= next) {
                // run [max(cstart, l0), next) is complete: private to this
                // thread unless its cube began before l0
                if (run > 0) {
                    if (GRAD) {
                        const T sc = cx.vc / (T)(next - cstart);
#pragma unroll
                        for (int p = 0; p < PP; ++p) { gacc[p].add(ag[p] * sc); ag[p] = (T)0; }
                    } else {
                        const double v1 = cvg_to_double_scaled(a1.value_t(), cx.kx);
                        const double v2 = cvg_to_double_scaled(a2.value_t(), 2 * cx.kx);
                        if (cstart >= l0) { a.JF[c] = v1; a.JF2[c] = v2; }
                        else { atomicAdd(&a.JF[c], v1); atomicAdd(&a.JF2[c], v2); }
                        a1.reset(); a2.reset();
                    }
                    run = 0;
                }
                if (ci < K - 2) {
                    do {  // empty cubes (never produced by the reallocation) are skipped
                        ++ci; ++c;
                        cvg_cube_next<D, T>(ns, zs, zsh, coord, cdy);
                        cstart = next;
                        next = starts[ci + 1];
                    } while (l >= next && ci < K - 2);
                }
                if (l >= next) {
                    // the prefix ends before the tile map says (only after a
                    // reallocation whose bounded wait ran out): report it and
                    // stay in the tile's last cube, so every access stays in
                    // bounds
                    atomicOr(a.status, CVG_KSTAT_BAD_TILE);
                    next = lend;
                }
                j = 0u;
            }
            ++run;
            T x[D];
            int bin[D];
            T jac = cx.jac0;
#pragma unroll
            for (int bk = 0; bk < NB; ++bk) {   // 4 dimensions per Philox call
                cvg_u32x4 r4;
                if (!REPLAY) r4 = cvg_philox_ks(j, c, cx.it, (cvg_u32)bk | cx.c3, keys);
#if CVG_FILL_PAIRS
                if constexpr (ZF) {
                    // dimension pairs in packed FP32 (same results as below)
                    const float *Gb = reinterpret_cast<const float *>(G);
#pragma unroll
                    for (int q = 0; q < 4; q += 2) {
                        const int d = 4 * bk + q;
                        if (d >= D) break;
                        const cvg_u32 ra = q == 0 ? r4.x : r4.z, rb = q == 0 ? r4.y : r4.w;
                        float ja, jb;
                        if (d + 1 < D) {
                            cvg_map_t2(ra, rb, zs2, cvg_pack2(cdy[d], cdy[d + 1]), fN2, fNm1,
                                       Gb + d * (N + 1), Gb + (d + 1) * (N + 1), x[d], x[d + 1],
                                       bin[d], bin[d + 1], ja, jb);
                            jac *= ja;
                            jac *= jb;
                        } else {
                            cvg_map_t(ra, zs, cdy[d], fN, fNm1, Gb + d * (N + 1), x[d], bin[d], ja);
                            jac *= ja;
                        }
                    }
                    continue;
                }
#endif
#pragma unroll
                for (int q = 0; q < 4; ++q) {
                    const int d = 4 * bk + q;
                    if (d >= D) break;
                    T z, frac;
                    int b;
                    if constexpr (ZF) {
                        const cvg_u32 r = q == 0 ? r4.x : q == 1 ? r4.y : q == 2 ? r4.z : r4.w;
                        z = fmaf(cvg_uniform_t(r), zs, cdy[d]);
                        b = cvg_bin_pos(z, fNm1, frac);
                    } else {
                        T u;
                        if (REPLAY) u = (T)a.ubuf[(base + (cvg_u64)l) * D + d];
                        else u = cvg_uniform<T>(q == 0 ? r4.x : q == 1 ? r4.y : q == 2 ? r4.z : r4.w);
                        const T y = cvg_fma(u, dy, cdy[d]);
                        z = y * fN;
                        b = cvg_bin(z, N, fNm1, frac);
                    }
                    const T e0 = G[d * (N + 1) + b];
                    const T e1 = G[d * (N + 1) + b + 1];
                    const T dx = e1 - e0;
                    x[d] = cvg_fma(dx, frac, e0);
                    jac *= fN * dx;
                    bin[d] = b;
                }
            }
            if (GRAD) {
                T g[PP];
                F::df(x, sm.th, g);
#pragma unroll
                for (int p = 0; p < PP; ++p) ag[p] += g[p] * jac;
            } else {
                const T jf = (T)F::f(x, sm.th) * jac;
                const T jf2 = jf * jf;
                if constexpr (H && FIX) {
                    // fixed-point bin sums in groups of dimensions (count
                    // atomics together, scale arithmetic in f32x2 pairs); the
                    // rare updates (a wrap or a large weight) of all
                    // dimensions are collected in a mask and handled behind
                    // one branch per sample.  Groups of CVG_HIST_GROUP, then
                    // of 4 and 2, then one dimension.
                    static_assert(D <= 32, "one wrap bit per dimension in 32 bits");
                    constexpr int HG = CVG_HIST_GROUP;
                    constexpr int R0 = (D / HG) * HG;
                    constexpr int R1 = R0 + ((D - R0) / 4) * 4;
                    constexpr int R2 = R1 + ((D - R1) / 2) * 2;
                    cvg_u32 wraps = 0u, big = 0u;   // in dimension order: see cvg_hist_add_fix
#pragma unroll
                    for (int d0 = 0; d0 < R0; d0 += HG)
                        cvg_fill_hist_group<HG>(sm.hw, sm.hc, d0, N, bin, jf2, wraps, big);
#pragma unroll
                    for (int d0 = R0; d0 < R1; d0 += 4)
                        cvg_fill_hist_group<4>(sm.hw, sm.hc, d0, N, bin, jf2, wraps, big);
                    if constexpr (R2 > R1)
                        cvg_fill_hist_group<2>(sm.hw, sm.hc, R1, N, bin, jf2, wraps, big);
                    if constexpr (D > R2)
                        cvg_hist_add_fix(sm.hw, sm.hc, R2 * N + bin[R2], jf2, wraps, big);
                    if (wraps | (big >> 23))
                        nrare += cvg_hist_rare<D>(sm.hw, sm.hc, a.weights, N, bin, jf2, wraps);
                } else {
#pragma unroll
                    for (int d = 0; d < D; ++d) {
                        if (H) {
                            cvg_hist_add_float(sm.hw, sm.hc, d * N + bin[d], jf2);
                        } else {
                            atomicAdd(&a.weights[d * N + bin[d]], cvg_to_double(jf2));
                            atomicAdd(&a.counts[d * N + bin[d]], 1u);
                        }
                    }
                }
                a1.add(jf);
                a2.add(jf2);
            }
            ++j;
        }
        if (run > 0) {   // last run: private only if it began here and its cube ends here
            if (GRAD) {
                const T sc = cx.vc / (T)(next - cstart);
#pragma unroll
                for (int p = 0; p < PP; ++p) gacc[p].add(ag[p] * sc);
            } else {
                if (cstart >= l0 && next == lend) {
                    a.JF[c] = cvg_to_double_scaled(a1.value_t(), cx.kx);
                    a.JF2[c] = cvg_to_double_scaled(a2.value_t(), 2 * cx.kx);
                } else {
                    cvg_run_to_global(a, c, a1, a2, cx.kx, run == lend - l0);
                }
            }
        }
    }
    cvg_tile_sync<WT>();
    return true;
}

// Add the CTA's shared-memory bin histograms to the global FP64/u32 ones;
// with reset, clear them for more samples (scale exponents kept).
template <int D, typename T, int BS, bool ESM, bool HSM, int P, bool GRAD, int NI, bool FIX>
CVG_D void cvg_fill_flush(const cvg_fill_args &a, const cvg_fill_smem<D, T, ESM, HSM, P, GRAD> &sm,
                          bool reset = false)
{
    if (!(HSM && !GRAD)) return;
    __syncthreads();
    const int N = NI > 0 ? NI : a.n_intervals;
    for (int i = threadIdx.x; i < D * N; i += BS) {
        const cvg_u32 cn = cvg_hist_count<FIX>(sm.hc[i]);
        if (cn) {
            const double w = cvg_hist_value<FIX>(sm.hw, sm.hc, i);
            if (w != 0.0) atomicAdd(&a.weights[i], w);
            atomicAdd(&a.counts[i], cn);
            if (reset) { sm.hw[i] = (T)0; sm.hc[i] -= cn; }
        }
    }
    __syncthreads();
}

// Rare histogram updates (wraps, large weights) of a CTA, added to the
// instance's count once; the reallocation's finish step reads it to choose
// the next fill's histogram form.
CVG_D void cvg_fill_count_rare(const cvg_fill_args &a, cvg_u32 nrare)
{
    if (!a.hist_state) return;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) nrare += __shfl_down_sync(0xffffffffu, nrare, o);
    if ((threadIdx.x & 31) == 0 && nrare) atomicAdd(&a.hist_state[1], nrare);
}

// FP32 form: fixed-point bin sums when the instance's state says so (the
// per-bin exponents predicted the weights well in the last fill), float
// atomics otherwise.  Uniform across the launch.
template <int D, typename T>
CVG_D bool cvg_fill_use_fixed(const cvg_fill_args &a)
{
    return cvg_hist_fixed<D, T>() && (!a.hist_state || a.hist_state[0] != 0u);
}

// Persistent single-instance fill.  Block tiles: this CTA takes tiles
// blockIdx.x, blockIdx.x + gridDim.x, ...  Warp tiles (CVG_FILL_WARP_TILES):
// each warp claims tiles of 32 * spt samples from a launch-wide counter, one
// ahead of the tile it works on, with no barrier between tiles, so the warps
// of a CTA drift into different phases (sampler, map, histogram) and the
// launch ends within one warp tile of its average.  A CTA claims at most
// CVG_HIST_MAX_RUN samples (its histogram counts stay below 2^24); the grid's
// budget (>= 152 CTAs) exceeds the 2^31 samples an iteration may hold.
template <int D, typename T, int BS, bool ESM, bool HSM, bool REPLAY, int P, bool GRAD, class F,
          int NI, bool FIX>
CVG_D void cvg_fill_run(const cvg_fill_args &a, cvg_u64 S, cvg_u64 n_tiles, cvg_u64 t0, cvg_u64 t1)
{
    extern __shared__ __align__(16) unsigned char cvg_smem[];
    constexpr int PP = P > 0 ? P : 1;
    constexpr bool WT = CVG_FILL_WARP_TILES != 0;
    const int tid = threadIdx.x;
    const int TS = a.tile_samples;
    cvg_fill_smem<D, T, ESM, HSM, P, GRAD> sm;
    // bins fixed at compile time: the views sit at constant offsets, so one
    // scaled bin index addresses both histogram words
    sm.carve(cvg_smem, NI > 0 ? NI : a.n_intervals, TS, WT ? BS / 32 : 1);
    cvg_fill_ctx<T> cx;
    cvg_fill_setup<D, T, BS, ESM, HSM, P, GRAD, FIX>(a, sm, cx);
    cvg_acc<T> gacc[PP];   // gradient pass: sum over runs of (v_cubes/nh) * run sum
#pragma unroll
    for (int p = 0; p < PP; ++p) gacc[p].reset();
    __syncthreads();

    cvg_u32 nrare = 0;
    if constexpr (WT) {
        // tile (warp number) first, then tiles n_warps, n_warps + 1, ... from the
        // counter (no burst of claims at the start)
        __shared__ cvg_u32 claimed;   // samples this CTA has claimed
        constexpr int W = BS / 32;
        if (tid == 0) claimed = (cvg_u32)(W * TS);
        __syncthreads();
        // (tile numbers fit 32 bits: an iteration holds < 2^31 samples);
        // tiles are numbered from t0, the first tile of this fill's range
        const cvg_u32 lane = tid & 31;
        const cvg_u32 n_warps = gridDim.x * W, nt = (cvg_u32)(t1 - t0);
        auto claim = [&]() -> cvg_u32 {
            cvg_u32 t = 0xFFFFFFFFu;
            if (lane == 0 && atomicAdd(&claimed, (cvg_u32)TS) + (cvg_u32)TS <= CVG_HIST_MAX_RUN)
                t = atomicAdd(&a.tile_ctl[0], 1u);
            t = __shfl_sync(0xffffffffu, t, 0);
            return t >= nt - n_warps ? 0xFFFFFFFFu : n_warps + t;
        };
        cvg_u32 tile = blockIdx.x * W + (tid >> 5);
        while (tile < nt) {
            const cvg_u32 next = n_warps < nt ? claim() : 0xFFFFFFFFu;
            if (!cvg_fill_tile<D, T, BS, ESM, HSM, REPLAY, P, GRAD, F, NI, FIX, true>(
                    a, sm, cx, t0 + tile, n_tiles, S, gacc, nrare, a.keys))
                break;
            tile = next;
        }
    } else {
        cvg_u64 since = 0;   // samples in the shared histograms since their last flush
        for (cvg_u64 tile = t0 + blockIdx.x; tile < t1; tile += gridDim.x) {
            if (since + (cvg_u64)TS > CVG_HIST_MAX_RUN) {
                cvg_fill_flush<D, T, BS, ESM, HSM, P, GRAD, NI, FIX>(a, sm, true);
                since = 0;
            }
            since += (cvg_u64)TS;
            if (!cvg_fill_tile<D, T, BS, ESM, HSM, REPLAY, P, GRAD, F, NI, FIX>(a, sm, cx, tile,
                                                                               n_tiles, S, gacc,
                                                                               nrare, a.keys))
                break;
        }
    }

    cvg_fill_flush<D, T, BS, ESM, HSM, P, GRAD, NI, FIX>(a, sm);
    if (WT && tid == 0) {   // the last CTA resets the tile counter for the next launch
        __threadfence();
        if (atomicAdd(&a.tile_ctl[1], 1u) == gridDim.x - 1) {
            a.tile_ctl[0] = 0u;
            a.tile_ctl[1] = 0u;
            __threadfence();
        }
    }
    if (FIX) cvg_fill_count_rare(a, nrare);
    if (GRAD) {
        const int lane = tid & 31, warp = tid >> 5;
#pragma unroll
        for (int p = 0; p < PP; ++p) {
            double v = ldexp(gacc[p].value(), cx.kx);
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
            if (lane == 0) sm.red[warp * PP + p] = v;
        }
        __syncthreads();
        if (tid < PP && tid < P) {
            double v = 0.0;
            for (int w = 0; w < BS / 32; ++w) v += sm.red[w * PP + tid];
            atomicAdd(&a.grad[tid], v);
        }
    }
}

template <int D, typename T, int BS, bool ESM, bool HSM, bool REPLAY, int P, bool GRAD, class F,
          int NI = 0>
CVG_D void cvg_fill_body(const cvg_fill_args &a)
{
    const cvg_u64 S = a.nh_sum[a.n_cubes];
    const int TS = a.tile_samples;
    cvg_u64 n_tiles = (S + (cvg_u64)TS - 1) / (cvg_u64)TS;
    if (n_tiles > a.max_tiles) {   // never produced by the reallocation; keep accesses in bounds
        if (blockIdx.x == 0 && threadIdx.x == 0) atomicOr(a.status, CVG_KSTAT_BAD_TILE);
        n_tiles = a.max_tiles;
    }
    // sample split across ranks: this fill's contiguous range of tiles
    cvg_u64 t0 = 0, t1 = n_tiles;
    if (a.shards > 1u) {
        t0 = n_tiles * a.shard / a.shards;
        t1 = n_tiles * (a.shard + 1u) / a.shards;
    }
    // with warp tiles every CTA takes part (the last one to finish resets the
    // tile counter)
    if (!CVG_FILL_WARP_TILES && (cvg_u64)blockIdx.x >= t1 - t0) return;
    if constexpr (cvg_hist_fixed<D, T>() && HSM && !GRAD) {
        if (cvg_fill_use_fixed<D, T>(a))
            cvg_fill_run<D, T, BS, ESM, HSM, REPLAY, P, GRAD, F, NI, true>(a, S, n_tiles, t0, t1);
        else
            cvg_fill_run<D, T, BS, ESM, HSM, REPLAY, P, GRAD, F, NI, false>(a, S, n_tiles, t0, t1);
    } else {
        cvg_fill_run<D, T, BS, ESM, HSM, REPLAY, P, GRAD, F, NI, false>(a, S, n_tiles, t0, t1);
    }
}

// ---------------------------------------------------------------------------
// Batched fill: many independent integrals (different dimensions and sample
// counts) in one persistent launch.  Tiles of all instances are numbered
// globally (tile_base[i] = first tile of instance i this iteration) and cut
// into one contiguous range per CTA, of equal estimated cost (the tile-base
// kernel weighs a tile by its instance's dimension).  A CTA claims chunks of
// tiles from its own range first, then from the others' (cvg_batch_claim), so
// CTAs that drew cheaper work take over the tail of heavier ranges.  Tiles
// are warp tiles (32 * spt samples): within a chunk each warp takes the next
// tile from a shared counter, with no block barrier until the chunk is used
// up.  While its claims stay in one instance the CTA keeps that instance's
// grid and histograms in shared memory; on a change it flushes the
// histograms and loads the next grid.  DISP::run(dim, op) calls
// op(cvg_int<D>, cvg_int<P>) for the dimensions present; DISP::fn<D> is the
// integrand of dimension D.
// ---------------------------------------------------------------------------
template <int V> struct cvg_int { static constexpr int value = V; };
template <bool V> struct cvg_bool { static constexpr bool value = V; };

// Block-wide claim of the next tiles.  Warp 0 looks at 32 ranges at a time,
// starting at the CTA's own (ranges blockIdx.x, blockIdx.x + 1, ... modulo
// n_ranges) and takes a quarter of what is left of the first range with
// tiles unclaimed (at least one tile, at most max_claim): the owner starts
// with long runs, the last claims of a range are single tiles.  The claim is left in shared
// memory, sh = {first tile t, end te, an instance at or before t, ranges
// found used up}; it stays there until the next claim.  Returns t < te
// (false once every range is used up).  Call from all threads of the block.
__device__ __noinline__ bool cvg_batch_claim(const cvg_batch_args &b, cvg_u64 *sh)
{
    if (threadIdx.x < 32) {
        const int lane = threadIdx.x;
        const int R = b.n_ranges;
        int vv = (int)sh[3];
        cvg_u64 got = 0, end = 0, gi = 0;
        while (vv < R) {
            const int o = vv + lane;
            int v = 0;
            cvg_u64 r0 = 0, len = 0, seen = 0;
            bool avail = false;
            if (o < R) {
                v = (int)blockIdx.x + o;
                if (v >= R) v -= R;
                r0 = b.range_start[v];
                len = b.range_start[v + 1] - r0;
                seen = *(volatile const cvg_u64 *)&b.claim[v];
                avail = seen < len;
            }
            const unsigned m = __ballot_sync(0xffffffffu, avail);
            if (!m) { vv += 32; continue; }
            const int src = __ffs(m) - 1;
            cvg_u64 c0 = 0, k = 0;
            if (lane == src) {
                k = (len - seen) >> 2;
                if (k > (cvg_u64)b.max_claim) k = b.max_claim;
                if (k == 0) k = 1;
                c0 = atomicAdd(&b.claim[v], k);
                if (c0 < len) {
                    got = r0 + c0;
                    end = r0 + (c0 + k < len ? c0 + k : len);
                    gi = b.range_inst[v];
                }
            }
            if (__shfl_sync(0xffffffffu, (int)(c0 < len), src)) {
                got = __shfl_sync(0xffffffffu, got, src);
                end = __shfl_sync(0xffffffffu, end, src);
                gi = __shfl_sync(0xffffffffu, gi, src);
                vv += src;                         // this range may hold more
                break;
            }
            vv += src + 1;                         // raced to its end: next range
        }
        __syncwarp();
        if (lane == 0) { sh[0] = got; sh[1] = end; sh[2] = gi; sh[3] = (cvg_u64)vv; }
    }
    __syncthreads();
    return sh[0] < sh[1];
}

template <typename T, int BS, class DISP, int NI = 0>
CVG_D void cvg_fill_batch(const cvg_batch_args &b)
{
    extern __shared__ __align__(16) unsigned char cvg_smem[];
    __shared__ cvg_u64 sh[4];
    __shared__ cvg_u32 s_tile[2];   // next tile of the chunk (counted in its instance), bad-tile flag
    if (threadIdx.x == 0) { sh[3] = 0; s_tile[1] = 0; }
    __syncwarp();
    bool more = cvg_batch_claim(b, sh);
    cvg_u64 t = sh[0];
    int i = (int)sh[2];
    const cvg_u32 lane = threadIdx.x & 31;
    while (more) {
        while (b.tile_base[i + 1] <= t) ++i;   // instance holding tile t
        const cvg_u64 t_in = t;
        const cvg_fill_args a = b.inst[i];
        DISP::run(b.dims[i], [&](auto Dc, auto Pc) {
            constexpr int D = decltype(Dc)::value, P = decltype(Pc)::value;
            using F = typename DISP::template fn<D>;
            auto session = [&](auto Fx) {
                constexpr bool FIX = decltype(Fx)::value;
                cvg_fill_smem<D, T, true, true, P, false> sm;
                sm.carve(cvg_smem, a.n_intervals, a.tile_samples, BS / 32);
                cvg_fill_ctx<T> cx;
                cvg_fill_setup<D, T, BS, true, true, P, false, FIX>(a, sm, cx);
                const cvg_u64 S = a.nh_sum[a.n_cubes];
                const cvg_u32 nt = (cvg_u32)(b.tile_base[i + 1] - b.tile_base[i]);
                // tiles of this instance counted from its first (< 2^32)
                cvg_u32 l0 = (cvg_u32)(t - b.tile_base[i]);
                cvg_u32 nrare = 0, since = 0;
                if (threadIdx.x == 0) s_tile[0] = l0;
                __syncthreads();
                while (true) {
                    const cvg_u64 tb = b.tile_base[i], te = sh[1];
                    const bool cont = te > tb + nt;    // the claim goes on in the next instance
                    const cvg_u32 lstop = cont ? nt : (cvg_u32)(te - tb);
                    // warp tiles of the chunk, one at a time from the shared counter:
                    // no barrier until the chunk is used up
                    while (true) {
                        cvg_u32 lt = 0;
                        if (lane == 0) lt = atomicAdd(&s_tile[0], 1u);
                        lt = __shfl_sync(0xffffffffu, lt, 0);
                        if (lt >= lstop) break;
                        if (!cvg_fill_tile<D, T, BS, true, true, false, P, false, F, NI, FIX, true>(
                                a, sm, cx, lt, nt, S, nullptr, nrare, b.keys)) {
                            if (lane == 0) s_tile[1] = 1u;   // inconsistent tile map (status set)
                            break;
                        }
                    }
                    since += (lstop - l0) * (cvg_u32)a.tile_samples;
                    __syncthreads();                   // every warp is done with the chunk
                    if (s_tile[1]) { more = false; break; }
                    if (cont) { t = tb + nt; break; }
                    more = cvg_batch_claim(b, sh);
                    if (!more) break;
                    t = sh[0];
                    if (t < tb || t >= tb + nt) {      // another instance: flush, reload
                        const int hint = (int)sh[2];
                        if (t < tb || hint > i) i = hint;
                        break;
                    }
                    l0 = (cvg_u32)(t - tb);
                    const cvg_u64 te2 = sh[1] < tb + nt ? sh[1] : tb + nt;
                    // counts stay below 2^24 (a claim holds at most max_claim tiles)
                    if (since + (cvg_u32)(te2 - t) * (cvg_u32)a.tile_samples > CVG_HIST_MAX_RUN) {
                        cvg_fill_flush<D, T, BS, true, true, P, false, NI, FIX>(a, sm, true);
                        since = 0;
                    }
                    if (threadIdx.x == 0) s_tile[0] = l0;
                    __syncthreads();
                }
                cvg_fill_flush<D, T, BS, true, true, P, false, NI, FIX>(a, sm);
                if (FIX) cvg_fill_count_rare(a, nrare);
            };
            // one histogram form per dimension here: a second copy of every
            // dimension's loop made the batched kernel spill
            session(cvg_bool<cvg_hist_fixed<D, T>()>{});
        });
        if (more && t == t_in) {                 // no variant for this dimension
            const cvg_u64 te = sh[1], tn = b.tile_base[i + 1];
            t = te < tn ? te : tn;
            if (t >= te) {
                more = cvg_batch_claim(b, sh);
                t = sh[0];
                i = (int)sh[2];
            }
        }
    }
}

// Pilot for the FP32 form's scales: samples uniform in [0,1)^dim mapped
// through the grid as it is now (Philox counter word 2 = 0xFFFFFFFF, so no
// iteration's samples are reused).  It takes the binary exponent of max
// |f*jac| (atomicMax into *a.scale_exp, initialised by the host) and the sum
// of (f*jac)^2 in FP64 (atomicAdd into *a.scale_ss, zeroed by the host), from
// which the host sets 2^k near the rms of f*jac, raised where needed so that
// the largest (f*jac*2^-k)^2 stays in FP32 range.  With a.bin_exp it also adds
// each sample's unscaled (f*jac)^2 and count to the global bin histograms
// (zero beforehand); the refinement kernel, run without adaptation, turns
// them into the first fill's per-bin exponents.
template <int D, typename T, int BS, int P, class F>
CVG_D void cvg_pilot_body(const cvg_fill_args &a, cvg_u32 blk)
{
    __shared__ T th[P > 0 ? P : 1];
    for (int i = threadIdx.x; i < P; i += BS) th[i] = (T)a.theta[i];
    __syncthreads();
    const cvg_u32 gid = blk * BS + threadIdx.x;
    const int N = a.n_intervals;
    const T fN = (T)N, fNm1 = (T)(N - 1);
    const T *grid = cvg_grid_src<T>::get(a);
    constexpr int NB = (D + 3) / 4;
    cvg_u32 rr[NB * 4];
#pragma unroll
    for (int b = 0; b < NB; ++b) {
        const cvg_u32x4 r4 = cvg_philox(0u, gid, 0xFFFFFFFFu, (cvg_u32)b | (a.instance << 8),
                                        (cvg_u32)a.seed, (cvg_u32)(a.seed >> 32));
        rr[4 * b + 0] = r4.x; rr[4 * b + 1] = r4.y; rr[4 * b + 2] = r4.z; rr[4 * b + 3] = r4.w;
    }
    T x[D];
    int bin[D];
    T jac = (T)1;
#pragma unroll
    for (int d = 0; d < D; ++d) {
        const T z = cvg_uniform<T>(rr[d]) * fN;
        T frac;
        const int b = cvg_bin(z, N, fNm1, frac);
        const T e0 = grid[d * (N + 1) + b], dx = grid[d * (N + 1) + b + 1] - e0;
        x[d] = cvg_fma(dx, frac, e0);
        jac *= fN * dx;
        bin[d] = b;
    }
    const T v = (T)F::f(x, th) * jac;
    const float fv = fabsf((float)v);
    int e = -200;
    double sq = 0.0;
    if (fv > 0.f && fv <= 3.4e38f) {
        e = (int)((__float_as_uint(fv) >> 23) & 0xFFu) - 127;
        const double vd = cvg_to_double(v < (T)0 ? -v : v);
        sq = vd * vd;
    } else if (!(fv <= 3.4e38f)) {
        e = 128;
    }
    if (a.bin_exp && fv <= 3.4e38f) {
#pragma unroll
        for (int d = 0; d < D; ++d) {
            atomicAdd(&a.weights[d * N + bin[d]], sq);
            atomicAdd(&a.counts[d * N + bin[d]], 1u);
        }
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        e = max(e, __shfl_down_sync(0xffffffffu, e, o));
        sq += __shfl_down_sync(0xffffffffu, sq, o);
    }
    if ((threadIdx.x & 31) == 0) {
        atomicMax(a.scale_exp, e);
        if (a.scale_ss) atomicAdd(a.scale_ss, sq);
    }
    if (a.bin_exp && blk == 0 && threadIdx.x == 0) a.bin_exp[D * N] = 0;   // sums are unscaled
}

// Batched pilot: blocks [i*PB, (i+1)*PB) evaluate instance i.
template <typename T, int PB, class DISP>
CVG_D void cvg_pilot_batch(const cvg_batch_args &b)
{
    const int i = blockIdx.x / PB;
    if (i >= b.n_inst) return;
    const cvg_fill_args a = b.inst[i];
    DISP::run(b.dims[i], [&](auto Dc, auto Pc) {
        constexpr int D = decltype(Dc)::value, P = decltype(Pc)::value;
        cvg_pilot_body<D, T, 256, P, typename DISP::template fn<D>>(a, blockIdx.x % PB);
    });
}

#endif  // CVG_FILL_CUH
