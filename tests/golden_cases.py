"""Shared loader for the reference golden vectors in tests/golden/.

Each ref_<case>.npz holds, per iteration i, what the reference's own kernels
(reference src/main.cu, compiled for sm_103a and driven by
tests/golden/ref_harness.cu) consumed and produced: the curand uniforms u_i
in sample order, the grid x_edges_in_i and per-cube counts nh_i before the
fill, the fill outputs JF_i, JF2_i, weights_i, counts_i, the damped variances
dh_i, the next counts nh_next_i, the refined grid x_edges_out_i and the
iteration estimate res_i / sig_i.  The integrand is the normalised Gaussian
of width 0.2 centred at 0.5 (oracle/ref_shim.cuh).
"""
import glob
import os

import numpy as np

HERE = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
GAUSS_W02 = r"""
template <typename T> __device__ __forceinline__ T g02(T* x) {
    T f = (T)1;
    for (int d = 0; d < cvg_n_dim; ++d) {
        const T t = (x[d] - (T)0.5) / (T)0.2;
        f *= exp(-t * t) * (T)(1.0 / (0.2 * 1.7724538509055160273));
    }
    return f;
}
__device__ double integrand(double* x) { return g02(x); }
"""
THETA = np.array([0.5, 0.2])


def cases():
    out = []
    for p in sorted(glob.glob(os.path.join(HERE, "ref_*.npz"))):
        z = np.load(p)
        meta = {k[5:]: z[k].item() for k in z.files if k.startswith("meta_")}
        out.append((os.path.basename(p)[4:-4], meta, z))
    return out
