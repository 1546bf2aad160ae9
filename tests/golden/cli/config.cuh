#ifndef CONFIG_CUH
#define CONFIG_CUH
// Plug-in configuration in the reference's config.cuh layout (globals read by
// the driver, integrand inlined into the fill): a normalised Gaussian peak,
// width 0.1, centre 0.5, in 4 dimensions; its integral over [0,1]^4 is erf(5)^4.
#include "peaks.cuh"
#define _USE_MATH_DEFINES
#include <math.h>

long int tot_eval = 4000000;
int max_it = 10;
int skip = 3;
long int max_batch_size = 1048576;

const int n_intervals = 512;
double alpha = 0.5;

double beta = 0.75;

const int blockSizeFill = 64;
const int blockSizeRes = 64;

const int n_dim = 4;
__host__ __device__
double integrand(double* x) {
    return gauss_peak(x, n_dim);
}

#endif
