/*
 * vegas_oracle.c -- CPU FP64 restatement of the cuVegas VEGAS+ loop.
 *
 * TEST INFRASTRUCTURE ONLY: the checker for the CUDA build and the timed CPU
 * baseline.  The product never links or calls this file.
 *
 * Reference lines are cited per function (paths relative to the reference
 * project root).  Build: see oracle/build_oracle.py (gcc -O2 -fopenmp
 * -ffp-contract=off, so x86_64 and aarch64 give the same results).
 */
#include "vegas_oracle.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

/* ------------------------------------------------------------------------ */
/* Philox4x32-10, from the published description (SC'11, section 5):        */
/* two 32x32->64 multiplies per round with multipliers 0xD2511F53 and       */
/* 0xCD9E8D57, Weyl key schedule with 0x9E3779B9 / 0xBB67AE85, 10 rounds.   */
/* ------------------------------------------------------------------------ */
void orc_philox4x32_10(const uint32_t ctr[4], const uint32_t key[2], uint32_t out[4])
{
    uint32_t c0 = ctr[0], c1 = ctr[1], c2 = ctr[2], c3 = ctr[3];
    uint32_t k0 = key[0], k1 = key[1];
    for (int r = 0; r < 10; ++r) {
        if (r > 0) { k0 += 0x9E3779B9u; k1 += 0xBB67AE85u; }
        uint64_t p0 = (uint64_t)0xD2511F53u * c0;
        uint64_t p1 = (uint64_t)0xCD9E8D57u * c2;
        uint32_t hi0 = (uint32_t)(p0 >> 32), lo0 = (uint32_t)p0;
        uint32_t hi1 = (uint32_t)(p1 >> 32), lo1 = (uint32_t)p1;
        uint32_t n0 = hi1 ^ c1 ^ k0;
        uint32_t n2 = hi0 ^ c3 ^ k1;
        c0 = n0; c1 = lo1; c2 = n2; c3 = lo0;
    }
    out[0] = c0; out[1] = c1; out[2] = c2; out[3] = c3;
}

/* ------------------------------------------------------------------------ */
/* Integrands                                                                */
/* ------------------------------------------------------------------------ */

/* Reference integrand library, src/commons/functions.cu:5-111, restated:   */
/* 0 linear, 1 roosarnold, 2 morokoffcalfisch, 3 hellekalek, 4 ridge,       */
/* 5 expon, 6 cosin, 7 dirichlet, 8 gaussian, 9 sinexp, 10 one.             */
/* The float-precision quirks of the reference (fabsf in roosarnold,         */
/* sqrtf in hellekalek) are kept.                                            */
static double reflib(int idx, const double *x, int n)
{
    double f;
    switch (idx) {
    case 0: /* linear, functions.cu:5-12 */
        f = 0.0;
        for (int i = 0; i < n; i++) f += x[i];
        return f;
    case 1: { /* roosarnold, functions.cu:14-23 */
        double aux = 0.0;
        f = 1.0 / (double)n;
        for (int i = 0; i < n; i++) aux += fabsf((float)(4.0 * x[i] - 2.0));
        return f * aux;
    }
    case 2: /* morokoffcalfisch, functions.cu:25-33 */
        f = 1.0;
        for (int i = 0; i < n; i++) f *= pow(x[i], 1.0 / (double)n);
        f *= pow(1.0 + 1.0 / (double)n, n);
        return f;
    case 3: /* hellekalek, functions.cu:35-43 */
        f = 1.0;
        for (int i = 0; i < n; i++) f *= ((x[i] - 0.5) / sqrtf(12.0f));
        return f;
    case 4: { /* ridge, functions.cu:45-60 */
        const int N = 1000;
        double norm = pow(100.0 / M_PI, 2.0) / N;
        f = 0.0;
        for (int i = 0; i < N; i++) {
            double x0 = i / (N - 1.0);
            double dx2 = 0.0;
            for (int j = 0; j < n; j++) { double a = x[j] - x0; dx2 += a * a; }
            f += exp(-100.0 * dx2);
        }
        return f * norm;
    }
    case 5: /* expon, functions.cu:62-69 */
        f = 0.0;
        for (int i = 0; i < n; i++) f += x[i] * x[i];
        return exp(-f);
    case 6: /* cosin, functions.cu:71-78 */
        f = 1.0;
        for (int i = 0; i < n; i++) f *= cos(x[i]);
        return f;
    case 7: { /* dirichlet, functions.cu:80-89 (alpha = 5) */
        const double alpha = 5.0;
        const double b = pow(tgamma(alpha), n) / tgamma(alpha * n);
        f = 1.0;
        for (int i = 0; i < n; i++) f *= pow(x[i], alpha - 1.0);
        return f / b;
    }
    case 8: { /* gaussian, functions.cu:91-101 (sigma^2 = 1e-4, mu = 0.5) */
        const double sigma2 = 0.0001, mu = 0.5;
        f = 0.0;
        for (int i = 0; i < n; i++) { const double a = x[i] - mu; f += a * a; }
        return exp(-0.5 * f / sigma2) / pow(2.0 * M_PI * sigma2, n / 2.0);
    }
    case 9: /* sinexp, functions.cu:103-106 (needs n >= 2) */
        return sin(x[0]) + exp(x[1]);
    case 10: /* one, functions.cu:108-111 */
        return 1.0;
    default:
        return 0.0;
    }
}

double orc_eval(int family, const double *x, int dim, const double *th)
{
    switch (family) {
    case ORC_F_GAUSS: {
        double mu = th ? th[0] : 0.5, s = th ? th[1] : 0.1;
        double norm = 1.0 / (s * sqrt(M_PI));
        double f = 1.0;
        for (int d = 0; d < dim; d++) {
            double t = (x[d] - mu) / s;
            f *= exp(-t * t) * norm;
        }
        return f;
    }
    case ORC_F_MIXTURE: {
        double f = 0.0;
        for (int k = 0; k < 2; k++) {
            double w = th[k], s = th[2 + k];
            const double *mu = th + 4 + k * dim;
            double g = 1.0;
            for (int d = 0; d < dim; d++) {
                double t = (x[d] - mu[d]) / s;
                g *= exp(-t * t);
            }
            f += w * g;
        }
        return f;
    }
    case ORC_F_PRODPEAK: {
        const double *c = th, *u = th + dim;
        double f = 1.0;
        for (int d = 0; d < dim; d++) {
            double a = x[d] - u[d];
            f *= 1.0 / (1.0 / (c[d] * c[d]) + a * a);
        }
        return f;
    }
    case ORC_F_CORNER: {
        double s = 1.0;
        for (int d = 0; d < dim; d++) s += th[d] * x[d];
        return pow(s, -(double)(dim + 1));
    }
    case ORC_F_CONST:
        return th ? th[0] : 1.0;
    case ORC_F_REFLIB:
        return reflib((int)th[0], x, dim);
    default:
        return 0.0;
    }
}

int orc_eval_grad(int family, const double *x, int dim, const double *th, double *g)
{
    switch (family) {
    case ORC_F_MIXTURE: {
        /* theta = [w1, w2, s1, s2, mu1(dim), mu2(dim)] */
        for (int k = 0; k < 2; k++) {
            double w = th[k], s = th[2 + k];
            const double *mu = th + 4 + k * dim;
            double q = 0.0, prod = 1.0;
            for (int d = 0; d < dim; d++) {
                double t = (x[d] - mu[d]) / s;
                prod *= exp(-t * t);
                q += t * t;
            }
            g[k] = prod;                              /* dF/dw_k  */
            g[2 + k] = w * prod * 2.0 * q / s;        /* dF/ds_k  */
            for (int d = 0; d < dim; d++)             /* dF/dmu_kd */
                g[4 + k * dim + d] = w * prod * 2.0 * (x[d] - mu[d]) / (s * s);
        }
        return 4 + 2 * dim;
    }
    case ORC_F_PRODPEAK: {
        const double *c = th, *u = th + dim;
        double f = orc_eval(family, x, dim, th);
        for (int d = 0; d < dim; d++) {
            double a = x[d] - u[d];
            double den = 1.0 / (c[d] * c[d]) + a * a;
            g[d] = f * (2.0 / (c[d] * c[d] * c[d])) / den;   /* d/dc_d */
            g[dim + d] = f * (2.0 * a) / den;                  /* d/du_d */
        }
        return 2 * dim;
    }
    case ORC_F_CORNER: {
        double s = 1.0;
        for (int d = 0; d < dim; d++) s += th[d] * x[d];
        double f = pow(s, -(double)(dim + 1));
        for (int d = 0; d < dim; d++) g[d] = -(double)(dim + 1) * f / s * x[d];
        return dim;
    }
    default:
        return 0;
    }
}

/* ------------------------------------------------------------------------ */
/* Sizing: src/main.cu:304 (n_eval_it), 329-331 (n_strat, n_cubes, v_cubes), */
/* 444-445 (initial nh); python_wrapper.py:16-18 (n_strat default).          */
/* ------------------------------------------------------------------------ */
int orc_compute_sizes(int64_t tot_eval, int max_it, int dim, int n_strat_in, orc_sizes *o)
{
    if (max_it <= 0 || dim <= 0 || tot_eval <= 0) return -1;
    o->n_eval_it = tot_eval / max_it;
    int ns = n_strat_in > 0 ? n_strat_in : (int)pow((double)o->n_eval_it / 4.0, 1.0 / dim);
    if (ns < 1) return -2;
    o->n_strat = ns;
    double nc = pow((double)ns, (double)dim);
    if (nc > 4294967295.0) return -3;
    o->n_cubes = (int64_t)nc;
    o->v_cubes = pow(1.0 / ns, (double)dim);
    int64_t nh = (int64_t)(1.0 / (double)o->n_cubes * (double)o->n_eval_it);
    o->nh_init = nh < 2 ? 2 : nh;
    return 0;
}

int orc_state_init(orc_state *st, int dim, int n_intervals, const orc_sizes *sz,
                   double alpha, double beta)
{
    memset(st, 0, sizeof(*st));
    st->dim = dim; st->n_intervals = n_intervals; st->n_strat = sz->n_strat;
    st->n_cubes = sz->n_cubes; st->n_eval_it = sz->n_eval_it; st->v_cubes = sz->v_cubes;
    st->alpha = alpha; st->beta = beta;
    int N = n_intervals;
    st->x_edges = (double *)malloc(sizeof(double) * dim * (N + 1));
    st->weights = (double *)calloc((size_t)dim * N, sizeof(double));
    st->counts = (int64_t *)calloc((size_t)dim * N, sizeof(int64_t));
    st->JF = (double *)calloc((size_t)st->n_cubes, sizeof(double));
    st->JF2 = (double *)calloc((size_t)st->n_cubes, sizeof(double));
    st->dh = (double *)calloc((size_t)st->n_cubes, sizeof(double));
    st->nh = (int64_t *)malloc(sizeof(int64_t) * st->n_cubes);
    st->nh_sum = (int64_t *)malloc(sizeof(int64_t) * (st->n_cubes + 1));
    if (!st->x_edges || !st->weights || !st->counts || !st->JF || !st->JF2 || !st->dh ||
        !st->nh || !st->nh_sum) {
        orc_state_free(st);
        return -1;
    }
    /* uniform grid x_j = j/N: src/main.cu:432-441 */
    double step = 1.0 / N;
    for (int d = 0; d < dim; d++)
        for (int j = 0; j <= N; j++) st->x_edges[d * (N + 1) + j] = j * step;
    /* nh init: src/main.cu:443-448 */
    for (int64_t c = 0; c < st->n_cubes; c++) st->nh[c] = sz->nh_init;
    orc_scan_nh(st);
    return 0;
}

void orc_state_free(orc_state *st)
{
    free(st->x_edges); free(st->weights); free(st->counts); free(st->JF); free(st->JF2);
    free(st->dh); free(st->nh); free(st->nh_sum);
    memset(st, 0, sizeof(*st));
}

/* exclusive scan of nh (cub::DeviceScan::ExclusiveSum, src/main.cu:579) */
void orc_scan_nh(orc_state *st)
{
    int64_t acc = 0;
    for (int64_t c = 0; c < st->n_cubes; c++) { st->nh_sum[c] = acc; acc += st->nh[c]; }
    st->nh_sum[st->n_cubes] = acc;
}

/* ------------------------------------------------------------------------ */
/* Uniforms                                                                  */
/* ------------------------------------------------------------------------ */
static inline void draw_uniforms(const orc_uniforms *u, uint32_t it, int64_t c, int64_t j,
                                 int64_t s, int dim, double *out)
{
    if (u->kind == ORC_U_BUFFER) {
        for (int d = 0; d < dim; d++) out[d] = (double)u->ubuf[s * dim + d];
        return;
    }
    uint32_t key[2] = {(uint32_t)u->seed, (uint32_t)(u->seed >> 32)};
    for (int b = 0; b * 4 < dim; b++) {
        uint32_t ctr[4] = {(uint32_t)j, (uint32_t)c, it, (uint32_t)b | (u->instance << 8)};
        uint32_t r[4];
        orc_philox4x32_10(ctr, key, r);
        for (int q = 0; q < 4 && b * 4 + q < dim; q++) {
            if (u->kind == ORC_U_PHILOX_F64)
                out[b * 4 + q] = ((double)r[q] + 0.5) * 0x1p-32;
            else
                out[b * 4 + q] = (double)((float)(((r[q] >> 9) << 1) | 1u) * 0x1p-24f);
        }
    }
}

/* Map one sample: stratified y, bin id, x and Jacobian.
 * src/main.cu:41-59 (y = u*dy + coord*dy; id = min((int)(y*N), N-1);
 * x = x_edges[id] + dx_edges[id]*(y*N - id); jac = prod N*dx_edges[id]). */
static inline double map_sample(const orc_state *st, int64_t c, const double *uu, int *id,
                                double *x)
{
    const int N = st->n_intervals, ns = st->n_strat, dim = st->dim;
    const double dy = 1.0 / ns;
    int64_t tmp = c;
    double jac = 1.0;
    for (int d = 0; d < dim; d++) {
        int64_t q = tmp / ns;
        double coord = (double)(tmp - q * ns);
        tmp = q;
        double y = fma(uu[d], dy, coord * dy);
        double z = y * (double)N;
        int b = (int)z;
        if (b >= N) b = N - 1;
        const double *xe = st->x_edges + (size_t)d * (N + 1);
        double dx = xe[b + 1] - xe[b];
        x[d] = fma(dx, z - b, xe[b]);
        id[d] = b;
        jac *= (double)N * dx;
    }
    return jac;
}

#define ORC_MAXDIM 64

/* vegasFill restated (src/main.cu:20-79): per sample of cube c, jf = f(x)*jac;
 * weights[d][id] += jf^2, counts[d][id] += 1, JF[c] += jf, JF2[c] += jf^2.
 * Parallel over cubes; thread-private histograms are summed at the end. */
int64_t orc_fill(orc_state *st, int family, const double *theta, const orc_uniforms *u,
                 uint32_t it, int n_threads)
{
    const int dim = st->dim, N = st->n_intervals;
    const size_t hsz = (size_t)dim * N;
    if (dim > ORC_MAXDIM) return -1;
    memset(st->weights, 0, sizeof(double) * hsz);
    memset(st->counts, 0, sizeof(int64_t) * hsz);
    int nt = 1;
#ifdef _OPENMP
    nt = n_threads > 0 ? n_threads : omp_get_max_threads();
#endif
    double *pw = (double *)calloc(hsz * nt, sizeof(double));
    int64_t *pc = (int64_t *)calloc(hsz * nt, sizeof(int64_t));
    if (!pw || !pc) { free(pw); free(pc); return -1; }
#ifdef _OPENMP
#pragma omp parallel num_threads(nt)
#endif
    {
        int tid = 0;
#ifdef _OPENMP
        tid = omp_get_thread_num();
#endif
        double *w = pw + hsz * tid;
        int64_t *cn = pc + hsz * tid;
        double uu[ORC_MAXDIM], x[ORC_MAXDIM];
        int id[ORC_MAXDIM];
#ifdef _OPENMP
#pragma omp for schedule(dynamic, 256)
#endif
        for (int64_t c = 0; c < st->n_cubes; c++) {
            double jf_s = 0.0, jf2_s = 0.0;
            for (int64_t j = 0; j < st->nh[c]; j++) {
                draw_uniforms(u, it, c, j, st->nh_sum[c] + j, dim, uu);
                double jac = map_sample(st, c, uu, id, x);
                double jf = orc_eval(family, x, dim, theta) * jac;
                double jf2 = jf * jf;
                for (int d = 0; d < dim; d++) {
                    w[(size_t)d * N + id[d]] += jf2;
                    cn[(size_t)d * N + id[d]] += 1;
                }
                jf_s += jf;
                jf2_s += jf2;
            }
            st->JF[c] = jf_s;
            st->JF2[c] = jf2_s;
        }
    }
    for (int t = 0; t < nt; t++)
        for (size_t i = 0; i < hsz; i++) {
            st->weights[i] += pw[hsz * t + i];
            st->counts[i] += pc[hsz * t + i];
        }
    free(pw); free(pc);
    return st->nh_sum[st->n_cubes];
}

/* results (src/main.cu:81-104) and the three DeviceReduce::Sum calls
 * (src/main.cu:677, 681-682). */
void orc_results(orc_state *st, double *dh_sum, double *res_it, double *sig_it)
{
    const double v = st->v_cubes, beta = st->beta;
    double sd = 0.0, sr = 0.0, ss = 0.0;
    for (int64_t i = 0; i < st->n_cubes; i++) {
        int neval = (int)st->nh[i];
        double Ih = st->JF[i] / neval * v;
        double Sig2 = (st->JF2[i] / neval * v * v) - (Ih * Ih);
        sr += Ih;
        ss += Sig2 / neval;
        double t = v * v * st->JF2[i] / neval - pow(v * st->JF[i] / neval, 2);
        if (t < 0) t = 0;
        st->dh[i] = pow(t, beta);
        sd += st->dh[i];
    }
    *dh_sum = sd; *res_it = sr; *sig_it = ss;
}

/* updateNh (src/main.cu:173-187): nh = max(2, (int)(dh/sum * n_eval_it)).
 * A non-finite or negative product (sum == 0) gives 2, the value the
 * reference's GPU conversion produces for NaN. */
void orc_update_nh(orc_state *st, double dh_sum)
{
    for (int64_t i = 0; i < st->n_cubes; i++) {
        double f = st->dh[i] / dh_sum;
        double v = f * (double)st->n_eval_it;
        int64_t nh_s = (v >= 0.0 && v < 2147483647.0) ? (int64_t)(int)v : (v >= 2147483647.0 ? 2147483647 : 0);
        st->nh[i] = nh_s < 2 ? 2 : nh_s;
    }
}

/* Grid refinement, src/main.cu:106-145 (normalize, smooth, alpha damping),
 * 189-209 (setMap), 211-246 (updateXEdges, updateDxEdges), with the per-dim
 * sums and the inclusive scan of src/main.cu:668-690.
 * Deliberate deviation: when a dimension's weight sum is zero or not finite
 * the reference divides 0/0 and writes NaN edges; here that dimension's grid
 * is left unchanged. */
void orc_refine(orc_state *st)
{
    const int N = st->n_intervals, dim = st->dim;
    double *w = (double *)malloc(sizeof(double) * N);
    double *sm = (double *)malloc(sizeof(double) * N);
    double *cs = (double *)malloc(sizeof(double) * N);
    double *xo = (double *)malloc(sizeof(double) * (N + 1));
    int *old = (int *)malloc(sizeof(int) * N);
    for (int d = 0; d < dim; d++) {
        double *xe = st->x_edges + (size_t)d * (N + 1);
        double dsum = 0.0;
        for (int i = 0; i < N; i++) {
            int64_t cn = st->counts[(size_t)d * N + i];
            double wi = st->weights[(size_t)d * N + i];
            w[i] = cn != 0 ? wi / (double)cn : wi;
            dsum += w[i];
        }
        if (!(dsum > 0.0) || !isfinite(dsum)) continue;
        for (int i = 0; i < N; i++) {
            double t;
            if (i == 0) t = (7.0 * w[0] + w[1]) / (8.0 * dsum);
            else if (i == N - 1) t = (w[i - 1] + 7.0 * w[i]) / (8.0 * dsum);
            else t = (w[i - 1] + 6.0 * w[i] + w[i + 1]) / (8.0 * dsum);
            if (t != 0) t = pow((t - 1.0) / log(t), st->alpha);
            sm[i] = t;
        }
        double ssum = 0.0, acc = 0.0;
        for (int i = 0; i < N; i++) { ssum += sm[i]; acc += sm[i]; cs[i] = acc; }
        if (!(ssum > 0.0) || !isfinite(ssum)) continue;
        double delta = ssum / N;
        for (int i = 0; i < N; i++) old[i] = N - 1;
        for (int i = 0; i < N; i++) {                 /* setMap */
            int div = (int)(cs[i] / delta);
            int off = i > 0 ? (int)(cs[i - 1] / delta) : 0;
            for (int j = 0; j < div - off; j++)
                if (off + j < N) old[off + j] = i;
        }
        memcpy(xo, xe, sizeof(double) * (N + 1));
        for (int k = 0; k < N - 1; k++) {             /* updateXEdges */
            int o = old[k];
            double a = (k + 1) * delta - (o > 0 ? cs[o - 1] : 0);
            xe[k + 1] = fma(a / sm[o], xo[o + 1] - xo[o], xo[o]);
        }
    }
    free(w); free(sm); free(cs); free(xo); free(old);
}

/* ------------------------------------------------------------------------ */
/* Full loop: src/main.cu:520-721, weighted mean 698-714, error 791-792.     */
/* ------------------------------------------------------------------------ */
int orc_integrate(int family, const double *theta, int dim, int64_t tot_eval, int max_it,
                  int skip, int n_intervals, int n_strat, double alpha, double beta,
                  const orc_uniforms *u, int n_threads, orc_result *res,
                  double *it_res, double *it_sig, double *x_edges_out)
{
    orc_sizes sz;
    int rc = orc_compute_sizes(tot_eval, max_it, dim, n_strat, &sz);
    if (rc) return rc;
    if (n_intervals < 2) return -4;
    orc_state st;
    if (orc_state_init(&st, dim, n_intervals, &sz, alpha, beta)) return -5;
    double sw = 0.0, swr = 0.0, swr2 = 0.0;
    int used = 0;
    int64_t tot = 0;
    for (int it = 0; it < max_it; it++) {
        int64_t n = orc_fill(&st, family, theta, u, (uint32_t)it, n_threads);
        if (n < 0) { orc_state_free(&st); return -6; }
        tot += n;
        double dh_sum, r, s;
        orc_results(&st, &dh_sum, &r, &s);
        if (it_res) it_res[it] = r;
        if (it_sig) it_sig[it] = s;
        orc_refine(&st);
        orc_update_nh(&st, dh_sum);
        orc_scan_nh(&st);
        if (it >= skip) {
            sw += 1.0 / s; swr += r / s; swr2 += r * r / s;
            used++;
        }
    }
    res->result = used ? swr / sw : 0.0;
    res->error = used ? 1.0 / sqrt(sw) : 0.0;
    res->chi2_dof = used > 1 ? (swr2 - res->result * res->result * sw) / (used - 1) : 0.0;
    res->tot_nevals = tot;
    res->n_it_used = used;
    if (x_edges_out) memcpy(x_edges_out, st.x_edges, sizeof(double) * dim * (n_intervals + 1));
    orc_state_free(&st);
    return 0;
}

/* dI_it/dtheta = sum_c v/nh_c sum_j jac * df/dtheta(x_j), same samples as
 * orc_fill, grid and nh held fixed. */
int orc_grad_iteration(orc_state *st, int family, const double *theta, int n_params,
                       const orc_uniforms *u, uint32_t it, int n_threads, double *grad)
{
    const int dim = st->dim;
    int nt = 1;
#ifdef _OPENMP
    nt = n_threads > 0 ? n_threads : omp_get_max_threads();
#endif
    double *pg = (double *)calloc((size_t)n_params * nt, sizeof(double));
    if (!pg || dim > ORC_MAXDIM || n_params > 256) { free(pg); return -1; }
#ifdef _OPENMP
#pragma omp parallel num_threads(nt)
#endif
    {
        int tid = 0;
#ifdef _OPENMP
        tid = omp_get_thread_num();
#endif
        double uu[ORC_MAXDIM], x[ORC_MAXDIM], g[256], acc[256];
        int id[ORC_MAXDIM];
#ifdef _OPENMP
#pragma omp for schedule(dynamic, 256)
#endif
        for (int64_t c = 0; c < st->n_cubes; c++) {
            for (int p = 0; p < n_params; p++) acc[p] = 0.0;
            for (int64_t j = 0; j < st->nh[c]; j++) {
                draw_uniforms(u, it, c, j, st->nh_sum[c] + j, dim, uu);
                double jac = map_sample(st, c, uu, id, x);
                orc_eval_grad(family, x, dim, theta, g);
                for (int p = 0; p < n_params; p++) acc[p] += g[p] * jac;
            }
            double scale = st->v_cubes / (double)st->nh[c];
            for (int p = 0; p < n_params; p++) pg[(size_t)tid * n_params + p] += acc[p] * scale;
        }
    }
    for (int p = 0; p < n_params; p++) {
        grad[p] = 0.0;
        for (int t = 0; t < nt; t++) grad[p] += pg[(size_t)t * n_params + p];
    }
    free(pg);
    return 0;
}
