// ref_harness.cu -- golden-vector generator (test infrastructure only).
//
// Loads the reference's own kernels (PTX compiled from the reference's
// src/main.cu by oracle/ref_build.py, with oracle/ref_shim.cuh as config) and
// drives them through the reference's iteration sequence on one GPU
// (src/main.cu:443-473 setup, 520-721 loop; CUB calls as at 500-504, 579,
// 668-690).  For every iteration it writes the uniforms vegasFill consumed,
// the per-cube and per-bin sums, the reallocation and the refined grid.
//
// The uniforms are recovered by replaying the same curand_uniform call
// sequence as vegasFill (src/main.cu:28-46) on a copy of the generator states
// taken just before the fill -- curand is called, not re-implemented.
//
// Usage: ref_harness <ptx> <dim> <n_eval_it> <n_intervals> <iters> <out_dir> [time|keep=i,j,..]
// With "time" nothing is dumped: each iteration (the reference's whole
// sequence, its host reads included) is timed with CUDA events and printed.
// With "keep=..." only the listed iterations are dumped (all are run).
#include <cub/cub.cuh>
#include <cuda_runtime.h>
#include <curand_kernel.h>

#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <algorithm>
#include <cstring>
#include <map>
#include <string>
#include <vector>

#define CK(x)                                                                               \
    do {                                                                                    \
        cudaError_t e_ = (x);                                                               \
        if (e_ != cudaSuccess) {                                                            \
            std::fprintf(stderr, "%s:%d %s: %s\n", __FILE__, __LINE__, #x,                  \
                         cudaGetErrorString(e_));                                           \
            std::exit(2);                                                                   \
        }                                                                                   \
    } while (0)

__global__ void dump_uniforms(const curandState *states, int n_dim, long it_total, long batch,
                              int runs, float *out)
{
    const long idx = threadIdx.x + (long)blockIdx.x * blockDim.x;
    if (idx >= batch) return;
    curandState st = states[idx];
    const int my_runs = (batch * (runs - 1) + idx) < it_total ? runs : (runs - 1);
    for (int run = 0; run < my_runs; run++)
        for (int d = 0; d < n_dim; d++) out[((long)run * batch + idx) * n_dim + d] = curand_uniform(&st);
}

static std::string g_out;

template <typename T>
static void dump(const char *name, int it, const T *dptr, size_t n)
{
    std::vector<T> h(n);
    CK(cudaMemcpy(h.data(), dptr, n * sizeof(T), cudaMemcpyDeviceToHost));
    char path[1024];
    std::snprintf(path, sizeof(path), "%s/%s_%d.bin", g_out.c_str(), name, it);
    FILE *f = std::fopen(path, "wb");
    if (!f) { std::perror(path); std::exit(3); }
    std::fwrite(h.data(), sizeof(T), n, f);
    std::fclose(f);
}

struct Kernels {
    std::map<std::string, cudaKernel_t> k;
    cudaKernel_t get(const char *prefix)
    {
        for (auto &kv : k)
            if (kv.first.rfind(prefix, 0) == 0) return kv.second;
        std::fprintf(stderr, "kernel %s not found\n", prefix);
        std::exit(4);
    }
};

static void launch(cudaKernel_t k, long n, int block, void **args)
{
    const unsigned grid = (unsigned)((n + block - 1) / block);
    CK(cudaLaunchKernel((const void *)k, dim3(grid), dim3(block), args, 0, 0));
    CK(cudaGetLastError());
}

int main(int argc, char **argv)
{
    if (argc != 7 && argc != 8) {
        std::fprintf(stderr,
                     "usage: %s ptx dim n_eval_it n_intervals iters out_dir [time|keep=i,j,..]\n",
                     argv[0]);
        return 1;
    }
    const char *ptx_path = argv[1];
    int n_dim = std::atoi(argv[2]);
    long n_eval_it = std::atol(argv[3]);
    int n_intervals = std::atoi(argv[4]);
    const int iters = std::atoi(argv[5]);
    g_out = argv[6];
    const bool timing = argc > 7 && std::strcmp(argv[7], "time") == 0;
    std::vector<char> keep(iters > 0 ? iters : 1, 1);
    if (argc > 7 && std::strncmp(argv[7], "keep=", 5) == 0) {
        std::fill(keep.begin(), keep.end(), 0);
        for (const char *c = argv[7] + 5; *c;) {
            const int k = std::atoi(c);
            if (k >= 0 && k < iters) keep[k] = 1;
            while (*c && *c != ',') c++;
            if (*c == ',') c++;
        }
    }    double alpha = 0.5, beta = 0.75;
    const long max_batch_size = 1048576;

    FILE *fp = std::fopen(ptx_path, "rb");
    if (!fp) { std::perror(ptx_path); return 1; }
    std::fseek(fp, 0, SEEK_END);
    long sz = std::ftell(fp);
    std::fseek(fp, 0, SEEK_SET);
    std::vector<char> ptx(sz + 1, 0);
    if (std::fread(ptx.data(), 1, sz, fp) != (size_t)sz) return 1;
    std::fclose(fp);
    cudaLibrary_t lib;
    CK(cudaLibraryLoadData(&lib, ptx.data(), nullptr, nullptr, 0, nullptr, nullptr, 0));
    unsigned nk = 0;
    CK(cudaLibraryGetKernelCount(&nk, lib));
    std::vector<cudaKernel_t> ks(nk);
    CK(cudaLibraryEnumerateKernels(ks.data(), nk, lib));
    Kernels K;
    for (auto k : ks) {
        const char *name = nullptr;
        CK(cudaFuncGetName(&name, (const void *)k));
        K.k[name] = k;
    }
    cudaKernel_t k_setup = K.get("_Z12setup_kernel"), k_fill = K.get("_Z9vegasFill"),
                 k_results = K.get("_Z7results"), k_norm = K.get("_Z16normalizeWeights"),
                 k_smooth = K.get("_Z13smoothWeights"), k_resetw = K.get("_Z12resetWeights"),
                 k_resets = K.get("_Z16resetWeightStrat"), k_upnh = K.get("_Z8updateNh"),
                 k_setmap = K.get("_Z6setMap"), k_upx = K.get("_Z12updateXEdges"),
                 k_updx = K.get("_Z13updateDxEdges"), k_map = K.get("_Z8mapCubes");

    // sizing: src/main.cu:317, 329-338
    int n_edges = n_intervals + 1;
    int n_strat = (int)pow((n_eval_it / 4.0), 1.0 / n_dim);
    int n_cubes = (int)pow(n_strat, n_dim);
    double v_cubes = pow((1.0 / n_strat), n_dim);
    long max_eval_it = n_eval_it + 2 * (long)n_cubes;
    long batch_size = max_eval_it < max_batch_size ? max_eval_it : max_batch_size;

    double *x_edges, *dx_edges, *weights, *x_old, *dx_old, *smw, *smw_sum, *summed, *d_sum;
    double *dh, *dh_sum, *JF, *JF2, *sum_r, *sum_s, *res_s, *sig_s;
    int *counts, *evals, *old_int;
    long *nh, *nh_sum;
    bool *hit;
    curandState *states, *states_copy;
    float *ubuf;
    CK(cudaMalloc(&x_edges, sizeof(double) * n_dim * n_edges));
    CK(cudaMalloc(&dx_edges, sizeof(double) * n_dim * n_intervals));
    CK(cudaMalloc(&x_old, sizeof(double) * n_dim * n_edges));
    CK(cudaMalloc(&dx_old, sizeof(double) * n_dim * n_intervals));
    CK(cudaMalloc(&weights, sizeof(double) * n_dim * n_intervals));
    CK(cudaMalloc(&counts, sizeof(int) * n_dim * n_intervals));
    CK(cudaMalloc(&smw, sizeof(double) * n_dim * n_intervals));
    CK(cudaMalloc(&smw_sum, sizeof(double) * n_dim * n_intervals));
    CK(cudaMalloc(&summed, sizeof(double) * n_dim));
    CK(cudaMalloc(&d_sum, sizeof(double) * n_dim));
    CK(cudaMalloc(&old_int, sizeof(int) * n_dim * n_intervals));
    CK(cudaMemset(old_int, 0, sizeof(int) * n_dim * n_intervals));
    CK(cudaMalloc(&dh, sizeof(double) * n_cubes));
    CK(cudaMalloc(&dh_sum, sizeof(double)));
    CK(cudaMalloc(&JF, sizeof(double) * n_cubes));
    CK(cudaMalloc(&JF2, sizeof(double) * n_cubes));
    CK(cudaMalloc(&sum_r, sizeof(double) * n_cubes));
    CK(cudaMalloc(&sum_s, sizeof(double) * n_cubes));
    CK(cudaMalloc(&res_s, sizeof(double)));
    CK(cudaMalloc(&sig_s, sizeof(double)));
    CK(cudaMalloc(&nh, sizeof(long) * n_cubes));
    CK(cudaMalloc(&nh_sum, sizeof(long) * n_cubes));
    CK(cudaMalloc(&evals, sizeof(int) * max_eval_it));
    CK(cudaMalloc(&hit, sizeof(bool)));
    CK(cudaMemset(hit, 0, sizeof(bool)));
    CK(cudaMalloc(&states, sizeof(curandState) * batch_size));
    CK(cudaMalloc(&states_copy, sizeof(curandState) * batch_size));
    ubuf = nullptr;
    if (!timing) CK(cudaMalloc(&ubuf, sizeof(float) * max_eval_it * n_dim));
    cudaEvent_t ev0, ev1;
    CK(cudaEventCreate(&ev0));
    CK(cudaEventCreate(&ev1));

    // initial grid and nh: src/main.cu:432-448
    std::vector<double> hx(n_dim * n_edges), hdx(n_dim * n_intervals);
    double step = 1.0 / n_intervals;
    for (int i = 0; i < n_dim; i++) {
        for (int j = 0; j < n_edges; j++) hx[i * n_edges + j] = j * step;
        for (int j = 0; j < n_intervals; j++)
            hdx[i * n_intervals + j] = hx[i * n_edges + j + 1] - hx[i * n_edges + j];
    }
    int nh_s = 1.0 / (double)n_cubes * n_eval_it;
    nh_s = nh_s < 2 ? 2 : nh_s;
    std::vector<long> hnh(n_cubes, nh_s);
    CK(cudaMemcpy(x_edges, hx.data(), sizeof(double) * hx.size(), cudaMemcpyHostToDevice));
    CK(cudaMemcpy(dx_edges, hdx.data(), sizeof(double) * hdx.size(), cudaMemcpyHostToDevice));
    CK(cudaMemcpy(nh, hnh.data(), sizeof(long) * n_cubes, cudaMemcpyHostToDevice));

    {   // setup_kernel (src/main.cu:462-467), one GPU: offset 0
        long off = 0;
        void *a[] = {&states, &batch_size, &off};
        launch(k_setup, batch_size, 128, a);
        CK(cudaDeviceSynchronize());
    }

    // CUB temporaries
    void *t_red = nullptr, *t_scan = nullptr, *t_ex = nullptr;
    size_t b_red = 0, b_scan = 0, b_ex = 0;
    CK(cub::DeviceReduce::Sum(t_red, b_red, dh, dh_sum, n_cubes > n_intervals ? n_cubes : n_intervals));
    CK(cub::DeviceScan::InclusiveSum(t_scan, b_scan, smw, smw_sum, n_intervals));
    CK(cub::DeviceScan::ExclusiveSum(t_ex, b_ex, nh, nh_sum, n_cubes));
    CK(cudaMalloc(&t_red, b_red));
    CK(cudaMalloc(&t_scan, b_scan));
    CK(cudaMalloc(&t_ex, b_ex));

    FILE *meta = std::fopen((g_out + (timing ? "/meta_time.txt" : "/meta.txt")).c_str(), "w");
    std::fprintf(meta, "dim %d\nn_eval_it %ld\nn_intervals %d\niters %d\nn_strat %d\nn_cubes %d\n"
                       "v_cubes %.17g\nbatch_size %ld\nalpha %.17g\nbeta %.17g\n",
                 n_dim, n_eval_it, n_intervals, iters, n_strat, n_cubes, v_cubes, batch_size,
                 alpha, beta);

    for (int it = 0; it < iters; it++) {
        CK(cudaEventRecord(ev0, 0));
        {   // reset (src/main.cu:525-529)
            void *a1[] = {&n_cubes, &JF, &JF2};
            launch(k_resets, n_cubes, 64, a1);
            void *a2[] = {&n_dim, &n_intervals, &counts, &weights};
            launch(k_resetw, (long)n_dim * n_intervals, 128, a2);
        }
        // map (src/main.cu:579-588)
        CK(cub::DeviceScan::ExclusiveSum(t_ex, b_ex, nh, nh_sum, n_cubes));
        {
            void *a[] = {&n_cubes, &evals, &nh, &nh_sum};
            launch(k_map, n_cubes, 64, a);
        }
        long last_nh, last_sum;
        CK(cudaMemcpy(&last_nh, nh + n_cubes - 1, sizeof(long), cudaMemcpyDeviceToHost));
        CK(cudaMemcpy(&last_sum, nh_sum + n_cubes - 1, sizeof(long), cudaMemcpyDeviceToHost));
        long idx = last_sum + last_nh;
        const bool dumping = !timing && keep[it];
        if (dumping) {
            dump("nh", it, nh, n_cubes);
            dump("x_edges_in", it, x_edges, (size_t)n_dim * n_edges);
        }
        // fill (src/main.cu:618-628)
        int runs = idx / batch_size + (int)((idx % batch_size) != 0);
        if (dumping)
            CK(cudaMemcpy(states_copy, states, sizeof(curandState) * batch_size, cudaMemcpyDeviceToDevice));
        {
            void *a[] = {&n_strat, &n_intervals, &n_edges, &idx, &batch_size, &runs, &counts,
                         &weights, &x_edges, &dx_edges, &JF, &JF2, &evals, &states};
            launch(k_fill, batch_size, 64, a);
        }
        if (dumping) {
            dump_uniforms<<<(unsigned)((batch_size + 127) / 128), 128>>>(states_copy, n_dim, idx,
                                                                       batch_size, runs, ubuf);
            CK(cudaGetLastError());
            CK(cudaDeviceSynchronize());
            dump("u", it, ubuf, (size_t)idx * n_dim);
            dump("JF", it, JF, n_cubes);
            dump("JF2", it, JF2, n_cubes);
            dump("weights", it, weights, (size_t)n_dim * n_intervals);
            dump("counts", it, counts, (size_t)n_dim * n_intervals);
        }
        // remaining (src/main.cu:662-694), serialised on one stream
        {
            void *a[] = {&n_cubes, &v_cubes, &beta, &nh, &JF, &JF2, &dh, &sum_r, &sum_s};
            launch(k_results, n_cubes, 64, a);
        }
        {
            void *a[] = {&n_dim, &n_intervals, &counts, &weights};
            launch(k_norm, (long)n_dim * n_intervals, 128, a);
        }
        for (int i = 0; i < n_dim; i++)
            CK(cub::DeviceReduce::Sum(t_red, b_red, weights + i * n_intervals, d_sum + i, n_intervals));
        {
            void *a[] = {&n_dim, &n_intervals, &alpha, &weights, &smw, &d_sum};
            launch(k_smooth, (long)n_dim * n_intervals, 128, a);
        }
        for (int i = 0; i < n_dim; i++)
            CK(cub::DeviceReduce::Sum(t_red, b_red, smw + i * n_intervals, summed + i, n_intervals));
        CK(cub::DeviceReduce::Sum(t_red, b_red, dh, dh_sum, n_cubes));
        {
            void *a[] = {&n_cubes, &n_eval_it, &nh, &dh, &dh_sum, &hit};
            launch(k_upnh, n_cubes, 128, a);
        }
        CK(cub::DeviceReduce::Sum(t_red, b_red, sum_r, res_s, n_cubes));
        CK(cub::DeviceReduce::Sum(t_red, b_red, sum_s, sig_s, n_cubes));
        CK(cudaMemcpy(x_old, x_edges, sizeof(double) * n_dim * n_edges, cudaMemcpyDeviceToDevice));
        CK(cudaMemcpy(dx_old, dx_edges, sizeof(double) * n_dim * n_intervals, cudaMemcpyDeviceToDevice));
        for (int i = 0; i < n_dim; i++)
            CK(cub::DeviceScan::InclusiveSum(t_scan, b_scan, smw + i * n_intervals,
                                             smw_sum + i * n_intervals, n_intervals));
        {
            void *a[] = {&n_dim, &n_intervals, &old_int, &summed, &smw_sum};
            launch(k_setmap, (long)n_dim * n_intervals, 128, a);
        }
        {
            void *a[] = {&n_dim, &n_intervals, &n_edges, &old_int, &summed, &smw, &smw_sum,
                         &x_edges, &x_old, &dx_old};
            launch(k_upx, (long)n_dim * n_intervals, 128, a);
        }
        {
            void *a[] = {&n_dim, &n_intervals, &n_edges, &x_edges, &dx_edges};
            launch(k_updx, (long)n_dim * n_intervals, 128, a);
        }
        CK(cudaEventRecord(ev1, 0));
        CK(cudaDeviceSynchronize());
        if (timing) {
            float ms = 0.f;
            CK(cudaEventElapsedTime(&ms, ev0, ev1));
            double r = 0.0;
            CK(cudaMemcpy(&r, res_s, sizeof(double), cudaMemcpyDeviceToHost));
            std::printf("iteration %d samples %ld ms %.4f estimate %.9f\n", it, idx, ms, r);
        } else if (dumping) {
            dump("dh", it, dh, n_cubes);
            dump("nh_next", it, nh, n_cubes);
            dump("x_edges_out", it, x_edges, (size_t)n_dim * n_edges);
            dump("res", it, res_s, 1);
            dump("sig", it, sig_s, 1);
            dump("dh_sum", it, dh_sum, 1);
        }
        std::fprintf(meta, "samples_%d %ld\n", it, idx);
    }
    std::fclose(meta);
    if (!timing) std::printf("golden written to %s\n", g_out.c_str());
    return 0;
}
