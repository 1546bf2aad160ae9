#ifndef PEAKS_CUH
#define PEAKS_CUH
__host__ __device__ double gauss_peak(double* x, int n_dim);
#endif
