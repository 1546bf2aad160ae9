"""Integrand sources (CUDA C++, compiled by NVRTC) and seeded workloads.

Each source defines ``integrand`` for both ``double*`` and ``float*`` through
one template, so the same text serves the FP64 (plain) and FP32
(compensated) forms.  ``cvg_n_dim`` is the compile-time dimension the JIT
prelude defines.

Workloads (seeded synthetic inputs with the shapes of the benchmark configs):
  gauss      prod_d exp(-((x_d-0.5)/0.1)^2)/(0.1 sqrt(pi)), d = 4 or 8
  mixture    sum_{k=1,2} w_k prod_d exp(-((x_d-mu_kd)/s_k)^2), d = 6, 16 parameters
  prodpeak   prod_d 1/(c_d^-2 + (x_d-u_d)^2), c ~ U(5,25), u ~ U(0,1);
             parameters theta = [c^-2, u] (prodpeak_theta)
  corner     (1 + sum_d c_d x_d)^-(d+1), c ~ U(0.1,1.0), d = 16
"""
import numpy as np

_MATH = r"""
__device__ __forceinline__ float cvg_exp(float x) { return expf(x); }
__device__ __forceinline__ double cvg_exp(double x) { return exp(x); }
"""

GAUSS = _MATH + r"""
// prod_d exp(-((x_d-0.5)/0.1)^2) / (0.1*sqrt(pi)), written as exp(-sum t^2) * norm^d
// with t = x*10 - 5 (one fused multiply-add per dimension, then one for t^2)
template <typename T> __device__ __forceinline__ T cvg_gauss(T* x) {
    const T inv_s = (T)10.0;
    const T norm = (T)5.6418958354775628695;   // 1/(0.1*sqrt(pi))
    T q = (T)0, n = (T)1;
#pragma unroll
    for (int d = 0; d < cvg_n_dim; ++d) { const T t = x[d] * inv_s - (T)5.0; q += t * t; n *= norm; }
    return cvg_exp(-q) * n;
}
__device__ double integrand(double* x) { return cvg_gauss(x); }
__device__ float integrand(float* x) { return cvg_gauss(x); }
"""

MIXTURE = _MATH + r"""
// theta = [w1, w2, s1, s2, mu_1(d), mu_2(d)]
template <typename T> __device__ __forceinline__ T cvg_mix(T* x, const T* th) {
    T f = (T)0;
#pragma unroll
    for (int k = 0; k < 2; ++k) {
        const T inv = (T)1 / th[2 + k];
        T q = (T)0;
#pragma unroll
        for (int d = 0; d < cvg_n_dim; ++d) { const T t = (x[d] - th[4 + k * cvg_n_dim + d]) * inv; q += t * t; }
        f += th[k] * cvg_exp(-q);
    }
    return f;
}
template <typename T> __device__ __forceinline__ void cvg_mix_grad(T* x, const T* th, T* g) {
#pragma unroll
    for (int k = 0; k < 2; ++k) {
        const T w = th[k], s = th[2 + k], inv = (T)1 / s;
        T q = (T)0;
#pragma unroll
        for (int d = 0; d < cvg_n_dim; ++d) { const T t = (x[d] - th[4 + k * cvg_n_dim + d]) * inv; q += t * t; }
        const T e = cvg_exp(-q);
        g[k] = e;
        g[2 + k] = w * e * (T)2 * q * inv;
        const T c = w * e * (T)2 * inv * inv;
#pragma unroll
        for (int d = 0; d < cvg_n_dim; ++d) g[4 + k * cvg_n_dim + d] = c * (x[d] - th[4 + k * cvg_n_dim + d]);
    }
}
__device__ double integrand(double* x, const double* th) { return cvg_mix(x, th); }
__device__ float integrand(float* x, const float* th) { return cvg_mix(x, th); }
__device__ void integrand_grad(double* x, const double* th, double* g) { cvg_mix_grad(x, th, g); }
__device__ void integrand_grad(float* x, const float* th, float* g) { cvg_mix_grad(x, th, g); }
"""

PRODPEAK = r"""
// theta = [c^-2 (d), u(d)] (see prodpeak_theta): prod_d 1/(c_d^-2 + (x_d-u_d)^2)
template <typename T> __device__ __forceinline__ T cvg_pp(T* x, const T* th) {
    T den = (T)1;
#pragma unroll
    for (int d = 0; d < cvg_n_dim; ++d) {
        const T a = x[d] - th[cvg_n_dim + d];
        den *= th[d] + a * a;
    }
    return (T)1 / den;
}
__device__ double integrand(double* x, const double* th) { return cvg_pp(x, th); }
__device__ float integrand(float* x, const float* th) { return cvg_pp(x, th); }
"""

CORNER = r"""
// theta = c(d): (1 + sum_d c_d x_d)^-(d+1)
template <typename T> __device__ __forceinline__ T cvg_corner(T* x, const T* th) {
    T s = (T)1;
#pragma unroll
    for (int d = 0; d < cvg_n_dim; ++d) s += th[d] * x[d];
    T p = (T)1, b = s;
#pragma unroll
    for (int e = cvg_n_dim + 1; e > 0; e >>= 1) { if (e & 1) p *= b; b *= b; }
    return (T)1 / p;
}
__device__ double integrand(double* x, const double* th) { return cvg_corner(x, th); }
__device__ float integrand(float* x, const float* th) { return cvg_corner(x, th); }
"""

# The reference's integrand library (src/commons/functions.cu:5-111) as
# templates over double and float, in the reference's operation order.  The
# reference's float-precision steps are kept: fabsf in roosarnold, sqrtf(12)
# in hellekalek.
REFLIB_NAMES = ("linear", "roosarnold", "morokoffcalfisch", "hellekalek", "ridge", "expon",
                "cosin", "dirichlet", "gaussian", "sinexp", "one")

_REFLIB = r"""
template <typename T> __device__ __forceinline__ T cvg_ref_linear(const T* x, int n) {
    T f = (T)0;
    for (int i = 0; i < n; i++) f += x[i];
    return f;
}
template <typename T> __device__ __forceinline__ T cvg_ref_roosarnold(const T* x, int n) {
    const T f = (T)1 / (T)n;
    T aux = (T)0;
    for (int i = 0; i < n; i++) aux += (T)fabsf((float)((T)4 * x[i] - (T)2));
    return f * aux;
}
template <typename T> __device__ __forceinline__ T cvg_ref_morokoffcalfisch(const T* x, int n) {
    T f = (T)1;
    for (int i = 0; i < n; i++) f *= pow(x[i], (T)1 / (T)n);
    f *= pow((T)1 + (T)1 / (T)n, (T)n);
    return f;
}
template <typename T> __device__ __forceinline__ T cvg_ref_hellekalek(const T* x, int n) {
    T f = (T)1;
    for (int i = 0; i < n; i++) f *= ((x[i] - (T)0.5) / (T)sqrtf(12.0f));
    return f;
}
template <typename T> __device__ __forceinline__ T cvg_ref_ridge(const T* x, int n) {
    const int N = 1000;
    const T norm = pow((T)100 / (T)3.14159265358979323846, (T)2) / (T)N;
    T f = (T)0;
    for (int i = 0; i < N; i++) {
        const T x0 = (T)i / ((T)N - (T)1);
        T dx2 = (T)0;
        for (int j = 0; j < n; j++) { const T a = x[j] - x0; dx2 += a * a; }
        f += exp((T)-100 * dx2);
    }
    return f * norm;
}
template <typename T> __device__ __forceinline__ T cvg_ref_expon(const T* x, int n) {
    T f = (T)0;
    for (int i = 0; i < n; i++) f += x[i] * x[i];
    return exp(-f);
}
template <typename T> __device__ __forceinline__ T cvg_ref_cosin(const T* x, int n) {
    T f = (T)1;
    for (int i = 0; i < n; i++) f *= cos(x[i]);
    return f;
}
template <typename T> __device__ __forceinline__ T cvg_ref_dirichlet(const T* x, int n) {
    const T alpha = (T)5;
    const T b = pow(tgamma(alpha), (T)n) / tgamma(alpha * (T)n);
    T f = (T)1;
    for (int i = 0; i < n; i++) f *= pow(x[i], alpha - (T)1);
    return f / b;
}
template <typename T> __device__ __forceinline__ T cvg_ref_gaussian(const T* x, int n) {
    const T sigma2 = (T)0.0001, mu = (T)0.5;
    T f = (T)0;
    for (int i = 0; i < n; i++) { const T a = x[i] - mu; f += a * a; }
    return exp((T)-0.5 * f / sigma2) / pow((T)2 * (T)3.14159265358979323846 * sigma2, (T)n / (T)2);
}
template <typename T> __device__ __forceinline__ T cvg_ref_sinexp(const T* x, int n) {
    (void)n;
    return sin(x[0]) + exp(x[1]);
}
template <typename T> __device__ __forceinline__ T cvg_ref_one(const T* x, int n) {
    (void)x; (void)n;
    return (T)1;
}
"""


def reflib_source(name):
    """Integrand source for one function of the reference's library (the
    choice config.cuh makes with `return ridge(x, n_dim);`)."""
    if name not in REFLIB_NAMES:
        raise ValueError("unknown reference function %r" % (name,))
    return _REFLIB + (
        "__device__ double integrand(double* x) { return cvg_ref_%s(x, cvg_n_dim); }\n"
        "__device__ float integrand(float* x) { return cvg_ref_%s(x, cvg_n_dim); }\n" % (name, name))


CONST_ONE = r"""
template <typename T> __device__ __forceinline__ T cvg_one(T* x) { (void)x; return (T)1; }
__device__ double integrand(double* x) { return cvg_one(x); }
__device__ float integrand(float* x) { return cvg_one(x); }
"""


def mixture_theta(seed=0, dim=6):
    """16 parameters for d=6 drawn from numpy's default_rng(seed):
    mu ~ U(0.2, 0.8) (2*dim), s ~ U(0.05, 0.2) (2), w ~ U(0.5, 1.5) (2).
    Layout returned: [w1, w2, s1, s2, mu_1(dim), mu_2(dim)]."""
    rng = np.random.default_rng(seed)
    mu = rng.uniform(0.2, 0.8, size=2 * dim)
    s = rng.uniform(0.05, 0.2, size=2)
    w = rng.uniform(0.5, 1.5, size=2)
    return np.concatenate([w, s, mu])


def corner_theta(seed=0, dim=16):
    rng = np.random.default_rng(seed)
    return rng.uniform(0.1, 1.0, size=dim)


def prodpeak_theta(c, u):
    """Parameters of PRODPEAK: [c^-2, u] (the reciprocal is taken once here,
    not per sample)."""
    c = np.asarray(c, dtype=np.float64)
    return np.concatenate([1.0 / (c * c), np.asarray(u, dtype=np.float64)])


def batch_instances(seed=0, n=512):
    """Batched product-peak family: dim ~ U{2..12}, evals/iteration
    log-uniform in [1e4, 1e7], c ~ U(5,25), u ~ U(0,1) per dimension."""
    rng = np.random.default_rng(seed)
    out = []
    for i in range(n):
        d = int(rng.integers(2, 13))
        n_it = int(10 ** rng.uniform(4, 7))
        c = rng.uniform(5, 25, size=d)
        u = rng.uniform(0, 1, size=d)
        out.append(dict(dim=d, n_eval_it=n_it, c=c, u=u, theta=prodpeak_theta(c, u)))
    return out
