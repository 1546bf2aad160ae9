/*
 * vegas_oracle.h -- CPU restatement of the VEGAS+ iteration loop of
 * emiliantolo/cuvegas, used ONLY as test infrastructure (the checker) and as
 * the timed CPU baseline.  Nothing in the product (cuvegas_gb300/) links,
 * imports or calls this code.
 *
 * Every function states the reference lines it follows (paths relative to the
 * reference project root).  Arithmetic is FP64 throughout, like the reference.
 *
 * Parity pinning: the restatement is checked against
 *   - published Philox4x32-10 known-answer vectors (tests/test_oracle.py),
 *   - analytic integrals of the benchmark integrands,
 *   - golden outputs of the reference's own CUDA kernels (vegasFill from
 *     vegas_cuda/src/vegas_cuda_extension/cuda_kernel.cu, the refinement and
 *     reallocation kernels of src/main.cu) fed with dumped curand uniforms,
 *     committed under tests/golden/ with the harness that produced them.
 */
#ifndef CVG_VEGAS_ORACLE_H
#define CVG_VEGAS_ORACLE_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Philox4x32-10 (Salmon, Moraes, Dror, Shaw, "Parallel Random Numbers: As
 * Easy as 1, 2, 3", SC'11).  ctr/key in, 4 words out. */
void orc_philox4x32_10(const uint32_t ctr[4], const uint32_t key[2], uint32_t out[4]);

/* Integrand families known to the oracle. */
enum {
    ORC_F_GAUSS = 0,      /* prod_d exp(-((x_d-p0)/p1)^2)/(p1*sqrt(pi))                     */
    ORC_F_MIXTURE = 1,    /* sum_k w_k prod_d exp(-((x_d-mu_kd)/s_k)^2), theta=[w1,w2,s1,s2,mu1(d),mu2(d)] */
    ORC_F_PRODPEAK = 2,   /* prod_d 1/(c_d^-2 + (x_d-u_d)^2), theta=[c(d), u(d)]             */
    ORC_F_CORNER = 3,     /* (1 + sum_d c_d x_d)^-(d+1), theta=[c(d)]                        */
    ORC_F_CONST = 4,      /* p0                                                              */
    ORC_F_REFLIB = 5      /* reference integrand library, p0 = function index (see .c)       */
};

double orc_eval(int family, const double *x, int dim, const double *theta);

/* Gradient of the parametric families w.r.t. theta (MIXTURE, PRODPEAK,
 * CORNER).  Writes n_params values; returns n_params. */
int orc_eval_grad(int family, const double *x, int dim, const double *theta, double *grad);

/* Sizing as in src/main.cu:304,329-331,337 and
 * vegas_cuda/src/vegas_cuda_extension/python_wrapper.py:16-18. */
typedef struct {
    int64_t n_eval_it;     /* tot_eval / max_it                          */
    int32_t n_strat;       /* (int) pow(n_eval_it/4, 1/dim) unless given */
    int64_t n_cubes;       /* n_strat^dim                                */
    double  v_cubes;       /* (1/n_strat)^dim                            */
    int64_t nh_init;       /* max(2, (int)(1/n_cubes * n_eval_it))       */
} orc_sizes;

int orc_compute_sizes(int64_t tot_eval, int max_it, int dim, int n_strat_in, orc_sizes *out);

/* One VEGAS+ run.  All device state of the reference becomes plain arrays. */
typedef struct {
    int dim, n_intervals, n_strat;
    int64_t n_cubes, n_eval_it;
    double v_cubes, alpha, beta;
    double *x_edges;    /* [dim][n_intervals+1] */
    double *weights;    /* [dim][n_intervals]   */
    int64_t *counts;    /* [dim][n_intervals]   */
    double *JF, *JF2;   /* [n_cubes]            */
    int64_t *nh;        /* [n_cubes]            */
    int64_t *nh_sum;    /* [n_cubes+1] exclusive prefix, last = total */
    double *dh;         /* [n_cubes]            */
} orc_state;

int  orc_state_init(orc_state *st, int dim, int n_intervals, const orc_sizes *sz,
                    double alpha, double beta);
void orc_state_free(orc_state *st);

/* Uniform sources.  ORC_U_PHILOX_F64 / _F32 reproduce the counter-based
 * sampler of the GPU build (counter = (sample-in-cube, cube, iteration,
 * dim-block | instance<<8), key = seed); ORC_U_BUFFER replays explicit float
 * uniforms u[s*dim + d] indexed by the global sample index s in cube order
 * (the order of the reference's evals[] array, src/main.cu:248-262). */
enum { ORC_U_PHILOX_F64 = 0, ORC_U_PHILOX_F32 = 1, ORC_U_BUFFER = 2 };

typedef struct {
    int kind;
    uint64_t seed;
    uint32_t instance;
    const float *ubuf;
} orc_uniforms;

/* fill: vegasFill (src/main.cu:20-79).  Zeroes and refills JF, JF2, weights,
 * counts for iteration `it`.  Returns the number of samples. */
int64_t orc_fill(orc_state *st, int family, const double *theta,
                 const orc_uniforms *u, uint32_t it, int n_threads);

/* results + DeviceReduce sums (src/main.cu:81-104, 677-682). */
void orc_results(orc_state *st, double *dh_sum, double *res_it, double *sig_it);

/* updateNh (src/main.cu:173-187) and the exclusive scan of nh
 * (src/main.cu:579). */
void orc_update_nh(orc_state *st, double dh_sum);
void orc_scan_nh(orc_state *st);

/* grid refinement: normalizeWeights, smoothWeights, the per-dim reduces and
 * inclusive scan, setMap, updateXEdges, updateDxEdges
 * (src/main.cu:106-145, 189-246, 667-694). */
void orc_refine(orc_state *st);

/* Full loop (src/main.cu:520-721) with the weighted mean (698-714) and the
 * reported error 1/sqrt(sum 1/sigma^2) (791-792).  chi2/dof is added.
 * it_res / it_sig (may be NULL) receive per-iteration estimates. */
typedef struct {
    double result, error, chi2_dof;
    int64_t tot_nevals;
    int n_it_used;
} orc_result;

int orc_integrate(int family, const double *theta, int dim, int64_t tot_eval, int max_it,
                  int skip, int n_intervals, int n_strat, double alpha, double beta,
                  const orc_uniforms *u, int n_threads, orc_result *res,
                  double *it_res, double *it_sig, double *x_edges_out);

/* Backward: dI_it/dtheta for one iteration with the grid and nh of that
 * iteration held fixed, same samples as orc_fill. */
int orc_grad_iteration(orc_state *st, int family, const double *theta, int n_params,
                       const orc_uniforms *u, uint32_t it, int n_threads, double *grad);

#ifdef __cplusplus
}
#endif
#endif
