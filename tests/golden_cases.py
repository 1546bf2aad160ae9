"""Shared loader for the reference golden vectors in tests/golden/.

Each ref_<case>.npz holds, per kept iteration i, what the reference's own
kernels (reference src/main.cu, compiled for sm_103a and driven by
oracle/ref_harness.cu) consumed and produced: the curand uniforms u_i in
sample order, the grid x_edges_in_i and per-cube counts nh_i before the fill,
the fill outputs JF_i, JF2_i, weights_i, counts_i, the damped variances dh_i,
the next counts nh_next_i, the refined grid x_edges_out_i and the iteration
estimate res_i / sig_i.  The integrand is the normalised Gaussian centred at
0.5, of width 0.2 (small cases) or 0.1 (the benchmark shapes; meta_width).

Full cases hold every sample and hypercube.  Benchmark-shape cases
(meta_cube_stride > 1) hold the uniforms, JF, JF2, dh and nh_next of the
hypercubes 0, stride, 2*stride, ... only, and the whole grid, histograms and
nh; `expand_uniforms` rebuilds a whole uniform buffer from them (the other
samples get 0.5), so a fill replay reproduces the kept hypercubes' sums.
"""
import glob
import os

import numpy as np

HERE = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def gauss_source(width):
    """The reference config's Gaussian, evaluated in the same order
    (per-dimension exp(-t*t) times the normalisation, t = (x - 0.5)/width)."""
    return r"""
template <typename T> __device__ __forceinline__ T gref(T* x) {
    T f = (T)1;
    for (int d = 0; d < cvg_n_dim; ++d) {
        const T t = (x[d] - (T)0.5) / (T)%(w)r;
        f *= exp(-t * t) * (T)(1.0 / (%(w)r * 1.7724538509055160273));
    }
    return f;
}
__device__ double integrand(double* x) { return gref(x); }
""" % {"w": float(width)}


GAUSS_W02 = gauss_source(0.2)
THETA = np.array([0.5, 0.2])


def _load(p):
    z = np.load(p)
    meta = {k[5:]: z[k].item() for k in z.files if k.startswith("meta_")}
    meta.setdefault("width", 0.2)
    meta.setdefault("cube_stride", 1)
    kept = [int(k) for k in z["kept"]] if "kept" in z.files else list(range(meta["iters"]))
    return os.path.basename(p)[4:-4], meta, z, kept


def _all():
    return [_load(p) for p in sorted(glob.glob(os.path.join(HERE, "ref_*.npz")))]


def cases():
    """Full cases: (name, meta, arrays)."""
    return [(n, m, z) for n, m, z, _ in _all() if m["cube_stride"] == 1]


def bench_shape_cases():
    """Benchmark-shape cases: (name, meta, arrays, kept iterations)."""
    return [c for c in _all() if c[1]["cube_stride"] > 1]


def kept_cubes(meta):
    return np.arange(0, meta["n_cubes"], meta["cube_stride"])


def expand_uniforms(meta, z, it):
    """Whole uniform buffer [S][dim] of iteration `it`: the kept hypercubes'
    reference uniforms in their sample rows, 0.5 everywhere else."""
    dim = meta["dim"]
    nh = z["nh_%d" % it].astype(np.int64)
    off = np.concatenate([[0], np.cumsum(nh)])
    u = np.full((int(off[-1]), dim), 0.5, dtype=np.float32)
    cubes = kept_cubes(meta)
    rows = np.concatenate([np.arange(off[c], off[c + 1]) for c in cubes])
    u[rows] = z["u_%d" % it].reshape(-1, dim)
    return u
