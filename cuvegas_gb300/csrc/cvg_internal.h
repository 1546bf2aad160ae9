// cvg_internal.h -- library-internal types and helpers shared by the host
// translation units (not part of the C ABI).
#ifndef CVG_INTERNAL_H
#define CVG_INTERNAL_H

#include <cuda_runtime.h>

#include <map>
#include <mutex>
#include <string>
#include <unordered_map>

#include "cuvegas.h"

struct cvg_context_s {
    int device = 0;
    cudaStream_t stream = nullptr;
    cudaStream_t aux = nullptr;   // second stream: refinement runs beside the reallocation
    bool own_stream = false;
    int n_sm = 0;
    int smem_optin = 0;
    int smem_per_sm = 0;          // shared memory of one SM (all resident CTAs)
    int cc_major = 0, cc_minor = 0;
    std::string arch;
    std::mutex mu;
    std::unordered_map<uint64_t, cudaLibrary_t> libs;
    // device arenas of destroyed runs and batches, kept for the next one of
    // a similar size (size -> pointer); guarded by arena_mu
    std::mutex arena_mu;
    std::multimap<size_t, void *> arena_cache;
    size_t arena_cached = 0, arena_cache_cap = 0;
    bool arena_poison = false;    // CVG_ARENA_POISON: fill every arena handed out with 0xFF bytes
};

struct cvg_integrand_s {
    cvg_context ctx = nullptr;
    std::string source;
    std::string link_ptx;         // PTX linked into every fill module (numba ABI integrand), or ""
    int dim = 0, abi = 0, n_params = 0, has_grad = 0;
};


cvg_status cvg_internal_fail(cvg_status st, const std::string &msg);
// NVRTC-compile (memory and disk cached) and load a module from source.
// With link_ptx non-empty the source is compiled relocatable and linked with
// that PTX (nvJitLink).
cvg_status cvg_internal_load_module(cvg_context ctx, const std::string &src, cudaLibrary_t *lib,
                                    const std::string &link_ptx = std::string());
// Integrand adaptor type (static f / df forwarding to ns + "integrand").
std::string cvg_internal_fn_struct(const char *name, const cvg_integrand_s &f, int abi,
                                   int n_params, int grad, const std::string &ns);
// NVRTC compile only (no device), for build checks.
cvg_status cvg_internal_compile_only(const std::string &src, const char *arch, std::string &log);
const char *cvg_internal_src_common();
const char *cvg_internal_src_fill();
double cvg_internal_now_ms();
// Device arena of at least `bytes` (a cached one of up to twice the size, else
// cudaMalloc); *got = its size.  Contents are undefined.
cudaError_t cvg_internal_arena_alloc(cvg_context ctx, size_t bytes, void **out, size_t *got);
// Return an arena (no work may be pending on it); it is kept for reuse while
// the cache stays within its cap, else freed.
void cvg_internal_arena_free(cvg_context ctx, void *p, size_t bytes);
// CTAs per SM a fill launch asks the compiler to fit (__launch_bounds__ min
// blocks): as many as shared memory allows, but never a register cap below
// 64 per thread.
int cvg_internal_fill_minb(cvg_context ctx, int block, size_t smem);

// FP32-form scale exponent k from the pilot: 2^k near the rms of f*jac
// (sum of squares ss over n samples), raised so that the largest seen
// |f*jac| (binary exponent emax) stays below 2^60 after scaling.
int cvg_internal_pilot_scale(int emax, double ss, double n);
// Weighted mean, error, chi^2/dof from per-iteration stats [3][max_it].
void cvg_internal_result(const double *stats, int max_it, int done, int skip, cvg_result *out);

#endif
