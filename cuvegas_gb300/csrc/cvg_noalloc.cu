// cvg_noalloc.cu -- the hypercube reallocation step for callers that cannot
// allocate device memory.
//
// Some callers must not call cudaMalloc at all: code running inside another
// framework's memory pool or allocator, or in a process whose device memory
// is fully reserved up front, where an allocation outside the owner's control
// would fail or fragment the pool.  For them this file provides
// cvg_realloc_noalloc: the same reallocation kernels as the iteration loop,
// but every temporary they need lives in one file-scope __device__ array that
// the CUDA module loader places when the library is loaded.  The caller
// passes only its own inputs and outputs.
//
// Limits and rules (also stated in include/cuvegas.h):
//  * at most CVG_NOALLOC_MAX_CUBES hypercubes (larger calls are rejected);
//  * the array is ~3 MiB on every GPU that loads the library, held until exit;
//  * all calls share the array: calls that overlap on the GPU (different
//    streams, or host threads without ordering) race and corrupt each other;
//  * the first call on a device looks up the array's device address with
//    cudaGetSymbolAddress, so make that first call before any stream capture;
//  * each call waits for its kernels and reads their status word back, so it
//    returns CVG_ERR_KERNEL when they found a non-finite estimate.
#include "cuvegas.h"
#include "cvg_kernels.cuh"

#include <cuda_runtime.h>

#include <mutex>
#include <string>

namespace {

constexpr cvg_u32 kMaxCubes = CVG_NOALLOC_MAX_CUBES;   // include/cuvegas.h
constexpr unsigned kMaxBlocks = (kMaxCubes + CVG_REALLOC_CHUNK - 1) / CVG_REALLOC_CHUNK;

constexpr size_t align256(size_t x) { return (x + 255) & ~(size_t)255; }
// layout of the scratch array
constexpr size_t kOffDh = 0;
constexpr size_t kOffNh = kOffDh + align256(sizeof(double) * kMaxCubes);
constexpr size_t kOffPart = kOffNh + align256(sizeof(cvg_u32) * kMaxCubes);
// partials of the results kernel: 4 per block, with 4x the blocks at this
// size (2 hypercubes per thread, as the loop's reallocation uses)
constexpr size_t kOffBsum = kOffPart + align256(sizeof(double) * 4 * 4 * kMaxBlocks);
constexpr size_t kOffAcc = kOffBsum + align256(sizeof(cvg_u64) * (kMaxBlocks + 1));
constexpr size_t kOffIt = kOffAcc + align256(sizeof(cvg_acc_dev));
constexpr size_t kOffStatus = kOffIt + 256;
constexpr size_t kScratchBytes = kOffStatus + 256;

__device__ __align__(256) unsigned char cvg_realloc_scratch[kScratchBytes];

std::mutex g_mu;
void *g_addr[64];   // device address of the array, per device

cvg_status reject(cvg_status s, const std::string &msg)
{
    cvg_internal_set_error(msg.c_str());
    return s;
}
}  // namespace

extern "C" cvg_status cvg_realloc_noalloc(double *JF, double *JF2, uint64_t *nh_sum,
                                          uint32_t n_cubes, double v_cubes, double beta,
                                          int64_t n_eval_it, int32_t precision, double *est,
                                          uint32_t *tile_cube, uint64_t max_tiles,
                                          int32_t tile_samples, void *stream)
{
    if (!JF || !JF2 || !nh_sum || !est)
        return reject(CVG_ERR_INVALID, "cvg_realloc_noalloc: JF, JF2, nh_sum and est are required");
    if (n_cubes == 0 || n_cubes > kMaxCubes)
        return reject(CVG_ERR_INVALID, "cvg_realloc_noalloc: n_cubes = " + std::to_string(n_cubes) +
                                           " outside [1, " + std::to_string(kMaxCubes) +
                                           "] (size of the preallocated scratch)");
    if (precision != CVG_PREC_FP64 && precision != CVG_PREC_FP32)
        return reject(CVG_ERR_INVALID, "cvg_realloc_noalloc: bad precision");
    if (tile_cube && tile_samples < 1)
        return reject(CVG_ERR_INVALID, "cvg_realloc_noalloc: tile_samples must be >= 1");
    // the fill's tile numbers and per-CTA sample claims are 32-bit: the same
    // bound cvg_run_create applies
    if (n_eval_it < 1 ||
        (uint64_t)n_eval_it + 2ull * n_cubes >= (1ull << 31) - (1ull << 20))
        return reject(CVG_ERR_INVALID, "cvg_realloc_noalloc: n_eval_it must be >= 1 and "
                                       "n_eval_it + 2*n_cubes below 2^31 - 2^20");
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64)
        return reject(CVG_ERR_CUDA, "cvg_realloc_noalloc: no current device");
    void *base = nullptr;
    {
        std::lock_guard<std::mutex> lock(g_mu);
        if (!g_addr[dev]) {
            void *p = nullptr;
            const cudaError_t e = cudaGetSymbolAddress(&p, cvg_realloc_scratch);
            if (e != cudaSuccess || !p)
                return reject(CVG_ERR_CUDA, std::string("cudaGetSymbolAddress of the scratch "
                                                        "array: ") + cudaGetErrorString(e));
            g_addr[dev] = p;
        }
        base = g_addr[dev];
    }
    cudaStream_t s = (cudaStream_t)stream;
    unsigned char *b = (unsigned char *)base;
    cvg_realloc_args a{};
    a.nh_sum = (cvg_u64 *)nh_sum;
    a.JF = JF;
    a.JF2 = JF2;
    a.dh = (double *)(b + kOffDh);
    a.nh_new = (cvg_u32 *)(b + kOffNh);
    a.partials = (double *)(b + kOffPart);
    a.bsums = (cvg_u64 *)(b + kOffBsum);
    a.acc = (cvg_acc_dev *)(b + kOffAcc);
    a.iteration = (cvg_u32 *)(b + kOffIt);
    a.status = (cvg_u32 *)(b + kOffStatus);
    // FP32 form: the per-cube sums are split into floats after scaling by
    // 2^-k (JF) and 2^-2k (JF2), with 2^(2k) near the mean (f*jac)^2 of the
    // iteration, worked out on the device from JF2 before the kernels run;
    // the FP64 form takes the sums as they are
    a.scale_exp = precision == CVG_PREC_FP32 ? (int *)(b + kOffIt + 144) : nullptr;
    a.done = (cvg_u32 *)(b + kOffIt + 64);   // block tickets (cleared below)
    a.stats = est;                       // est[0] = I, est[1] = sigma^2, est[2] = samples
    a.tile_cube = tile_cube;
    a.max_tiles = tile_cube ? max_tiles : 0;
    a.tile_samples = tile_cube ? tile_samples : 1;
    a.n_eval_it = n_eval_it;
    a.v_cubes = v_cubes;
    a.beta = beta;
    a.n_cubes = n_cubes;
    a.skip = 0;
    a.max_it = 1;
    a.fast_pow = precision == CVG_PREC_FP32 ? 1 : 0;
    a.adapt = 1;
    a.small_chunks = 1;   // the same per-thread grouping as the loop at this size
    // the array keeps the previous call's contents: clear what the kernels
    // accumulate into (sums, counters, status); the rest is overwritten
    cudaError_t e = cudaMemsetAsync(b + kOffAcc, 0, kOffStatus + 256 - kOffAcc, s);
    if (e == cudaSuccess && a.scale_exp)
        e = cvg_launch_scale_from_sums(JF2, a.nh_sum, n_cubes, (double *)(b + kOffIt + 128),
                                       (cvg_u32 *)(b + kOffIt + 136), a.scale_exp, s);
    if (e == cudaSuccess) e = cvg_launch_realloc(a, s);
    // the kernels report what they found in the array's status word: wait for
    // them and read it (a 4-byte copy into this stack variable, no allocation)
    cvg_u32 status = 0;
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(&status, a.status, sizeof(status), cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    if (e != cudaSuccess) return reject(CVG_ERR_CUDA, cudaGetErrorString(e));
    if (status & CVG_KSTAT_NONFINITE)
        return reject(CVG_ERR_KERNEL, "cvg_realloc_noalloc: the iteration estimate or its "
                                      "variance is not finite (non-finite JF/JF2 or overflow)");
    if (status & (CVG_KSTAT_BAD_TILE | CVG_KSTAT_TIMEOUT))
        return reject(CVG_ERR_KERNEL, "cvg_realloc_noalloc: the reallocation kernels reported "
                                      "an inconsistent state (status " + std::to_string(status) + ")");
    return CVG_OK;
}
