// cvg_internal.h -- library-internal types and helpers shared by the host
// translation units (not part of the C ABI).
#ifndef CVG_INTERNAL_H
#define CVG_INTERNAL_H

#include <cuda_runtime.h>

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
    int cc_major = 0, cc_minor = 0;
    std::string arch;
    std::mutex mu;
    std::unordered_map<uint64_t, cudaLibrary_t> libs;
};

struct cvg_integrand_s {
    cvg_context ctx = nullptr;
    std::string source;
    int dim = 0, abi = 0, n_params = 0, has_grad = 0;
};


cvg_status cvg_internal_fail(cvg_status st, const std::string &msg);
// NVRTC-compile (memory and disk cached) and load a module from source.
cvg_status cvg_internal_load_module(cvg_context ctx, const std::string &src, cudaLibrary_t *lib);
// Integrand adaptor type (static f / df forwarding to ns + "integrand").
std::string cvg_internal_fn_struct(const char *name, const cvg_integrand_s &f, int abi,
                                   int n_params, int grad, const std::string &ns);
// NVRTC compile only (no device), for build checks.
cvg_status cvg_internal_compile_only(const std::string &src, const char *arch, std::string &log);
const char *cvg_internal_src_common();
const char *cvg_internal_src_fill();
double cvg_internal_now_ms();
// FP32-form scale exponent k from the pilot: 2^k near the rms of f*jac
// (sum of squares ss over n samples), raised so that the largest seen
// |f*jac| (binary exponent emax) stays below 2^60 after scaling.
int cvg_internal_pilot_scale(int emax, double ss, double n);
// Weighted mean, error, chi^2/dof from per-iteration stats [3][max_it].
void cvg_internal_result(const double *stats, int max_it, int done, int skip, cvg_result *out);

#endif
