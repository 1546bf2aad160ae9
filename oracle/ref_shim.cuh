/* ref_shim.cuh -- pre-included in place of the reference's src/config.cuh
 * when its kernels are compiled to PTX for the golden-vector harness
 * (oracle/ref_build.py).  Defines the config globals the reference's main.cu
 * expects (src/config.cuh:7-33) and a Gaussian integrand; CVG_REF_DIM sets
 * n_dim.  Test infrastructure only. */
#ifndef CONFIG_CUH
#define CONFIG_CUH
#include <math.h>
long int tot_eval = 1000000;
int max_it = 4;
int skip = 1;
long int max_batch_size = 1048576;
const int n_intervals = 1024;
double alpha = 0.5;
double beta = 0.75;
const int blockSizeRes = 64;
const int blockSizeRed = 128;
const int blockSizeUpd = 128;
const int blockSizeFill = 64;
const int blockSizeIntervals = 128;
const int blockSizeInit = 128;
const int n_dim = CVG_REF_DIM;
/* prod_d exp(-((x_d-0.5)/s)^2) / (s sqrt(pi)), s = CVG_REF_WIDTH (0.2 for the
 * golden vectors, 0.1 for the benchmark workloads) */
#ifndef CVG_REF_WIDTH
#define CVG_REF_WIDTH 0.2
#endif
__host__ __device__ double integrand(double *x)
{
    double f = 1.0;
    for (int d = 0; d < n_dim; d++) {
        double t = (x[d] - 0.5) / CVG_REF_WIDTH;
        f *= exp(-t * t) * (1.0 / (CVG_REF_WIDTH * 1.7724538509055160273));
    }
    return f;
}
#endif
