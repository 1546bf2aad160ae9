#define _USE_MATH_DEFINES
#include <math.h>
#include "peaks.cuh"

// prod_d exp(-((x_d - 0.5) / 0.1)^2) / (0.1 sqrt(pi))
__host__ __device__
double gauss_peak(double* x, int n_dim) {
    double q = 0.0, norm = 1.0;
    for (int i = 0; i < n_dim; i++) {
        const double t = (x[i] - 0.5) / 0.1;
        q += t * t;
        norm *= 1.0 / (0.1 * sqrt(M_PI));
    }
    return exp(-q) * norm;
}
