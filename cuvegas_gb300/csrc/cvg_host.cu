// cvg_host.cu -- host driver and C ABI of libcuvegas.
//
// Replaces the host side of the reference: the per-call setup, allocation and
// iteration loop of integrate_cuda / main (cuda_wrapper.cu:290-872,
// src/main.cu:277-800) and the JIT link step (cuda_wrapper.cu:221-286).
//
// GB300-first choices:
//  * one context per device, caller's stream or its own; no host sync inside
//    an iteration -- the sample count, iteration counter, weighted-mean sums
//    and chi^2 inputs live on the device until the caller asks for them;
//  * integrand source -> NVRTC -> sm_103a cubin, with the fill kernel
//    specialised on dimension, precision and tile shape and the integrand
//    inlined; cubins cached in memory and on disk;
//  * an iteration can be captured once as a CUDA graph and replayed.
#include "cuvegas.h"
#include "cvg_kernels.cuh"

#include <cuda_runtime.h>
#include <nvJitLink.h>
#include <nvrtc.h>

#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <mutex>
#include <string>
#include <sys/stat.h>
#include <unistd.h>
#include <unordered_map>
#include <vector>

#include "cvg_embedded.inc"   // cvg_src_common, cvg_src_fill (generated at build time)

#define CVG_VERSION "cuvegas_gb300 0.1"

namespace {

thread_local std::string g_err;

cvg_status fail(cvg_status s, const std::string &msg)
{
    g_err = msg;
    return s;
}

#define CK(x)                                                                          \
    do {                                                                               \
        cudaError_t e_ = (x);                                                          \
        if (e_ != cudaSuccess)                                                         \
            return fail(e_ == cudaErrorMemoryAllocation ? CVG_ERR_NOMEM : CVG_ERR_CUDA, \
                        std::string(#x) + ": " + cudaGetErrorString(e_));              \
    } while (0)

#define CKS(x)                                   \
    do {                                         \
        cvg_status s_ = (x);                     \
        if (s_ != CVG_OK) return s_;             \
    } while (0)

double now_ms()
{
    using namespace std::chrono;
    return duration<double, std::milli>(steady_clock::now().time_since_epoch()).count();
}

uint64_t fnv1a(const std::string &s, uint64_t h = 1469598103934665603ull)
{
    for (unsigned char c : s) { h ^= c; h *= 1099511628211ull; }
    return h;
}

}  // namespace

void cvg_internal_set_error(const char *msg) { g_err = msg ? msg : ""; }

#include "cvg_internal.h"

struct fill_variant {
    cudaKernel_t kernel = nullptr;
    cudaKernel_t pilot = nullptr;
    size_t smem = 0;
    int occ = 0;
};

struct cvg_run_s {
    cvg_context ctx = nullptr;
    cvg_integrand f = nullptr;
    cvg_params p{};
    // sizes
    int64_t n_eval_it = 0;
    int n_strat = 0;
    cvg_u32 n_cubes = 0;
    double v_cubes = 0.0;
    unsigned nb = 0;
    cvg_u64 max_tiles = 0;
    int block = 0, spt = 0, TS = 0, grid = 0, esm = 1, hsm = 1;
    int wt = 1;                   // warp tiles (TS = 32*spt) or block tiles (TS = block*spt)
    int it_done = 0;
    // device memory (one arena)
    void *arena = nullptr;
    size_t arena_bytes = 0;
    double *x_edges = nullptr, *weights = nullptr, *JF = nullptr, *JF2 = nullptr, *dh = nullptr;
    double *partials = nullptr, *stats = nullptr, *theta = nullptr, *grad = nullptr;
    float *x_edges32 = nullptr, *ubuf = nullptr;
    cvg_u32 *counts = nullptr, *nh_new = nullptr, *tile_cube = nullptr, *iteration = nullptr;
    cvg_u32 *status = nullptr;
    int *scale_exp = nullptr;
    double *scale_ss = nullptr;
    int *bin_exp = nullptr;
    cvg_u32 *hist_state = nullptr;
    cvg_u64 *lb = nullptr;        // look-back words of the one-pass allocation
    cvg_u32 *lb_ctl = nullptr;
    cvg_u32 shard = 0, shards = 1;   // sample split: this run's fills cover one range of tiles
    int lb_spin_limit = 0;        // CVG_LB_SPIN_LIMIT (0: the kernel's default, 2^22 polls)
    cvg_u32 lb_withhold = 0;      // CVG_TEST_LB_WITHHOLD (failure test only; 0: none)
    cvg_u32 *tile_ctl = nullptr;  // the fill's warp-tile counter and CTA-done count
    cvg_u32 *done = nullptr;
    cvg_u64 *nh_sum = nullptr, *bsums = nullptr;
    cvg_acc_dev *acc = nullptr;
    size_t ubuf_samples = 0;
    bool replay = false;
    fill_variant fill, fill_replay, gradk;
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t graph_exec = nullptr;
    cudaEvent_t ev0 = nullptr, ev1 = nullptr;
    std::vector<std::pair<cudaEvent_t, cudaEvent_t>> fill_ev;   // timed fills
    size_t fill_ev_used = 0;
    cudaEvent_t ev0_own = nullptr, ev1_own = nullptr;
    cudaEvent_t ev_fork = nullptr, ev_join = nullptr;   // refinement beside reallocation
};

// ---------------------------------------------------------------------------
// JIT
// ---------------------------------------------------------------------------
namespace {

std::string cache_dir()
{
    const char *e = std::getenv("CVG_CACHE_DIR");
    if (e && *e) return e;
    const char *h = std::getenv("HOME");
    return std::string(h && *h ? h : "/tmp") + "/.cache/cuvegas_gb300";
}

void mkdirs(const std::string &path)
{
    std::string cur;
    for (size_t i = 0; i < path.size(); ++i) {
        cur.push_back(path[i]);
        if (path[i] == '/' || i + 1 == path.size()) mkdir(cur.c_str(), 0755);
    }
}

bool read_file(const std::string &p, std::vector<char> &out)
{
    FILE *fp = std::fopen(p.c_str(), "rb");
    if (!fp) return false;
    std::fseek(fp, 0, SEEK_END);
    long n = std::ftell(fp);
    std::fseek(fp, 0, SEEK_SET);
    out.resize(n > 0 ? (size_t)n : 0);
    bool ok = n > 0 && std::fread(out.data(), 1, out.size(), fp) == out.size();
    std::fclose(fp);
    return ok;
}

void write_file(const std::string &p, const std::vector<char> &data)
{
    std::string tmp = p + ".tmp" + std::to_string((long)getpid());
    FILE *fp = std::fopen(tmp.c_str(), "wb");
    if (!fp) return;
    bool ok = std::fwrite(data.data(), 1, data.size(), fp) == data.size();
    std::fclose(fp);
    if (ok) std::rename(tmp.c_str(), p.c_str());
    else std::remove(tmp.c_str());
}

struct variant_key {
    int dim, prec, block, esm, hsm, replay, n_params, grad, abi, nbins, minb, wt;
};

// Tile shape of single-run fills: CVG_FILL_WARP_TILES=1 in the environment
// forces warp tiles, =0 block tiles (the whole CTA on one tile of block*spt
// samples, a barrier between tiles); unset (-1), a run chooses by its size.
int env_warp_tiles()
{
    const char *e = std::getenv("CVG_FILL_WARP_TILES");
    if (!e || !*e) return -1;
    return e[0] == '0' ? 0 : 1;
}

// Non-negative integer from the environment, or `dflt` when unset or invalid.
long env_long(const char *name, long dflt)
{
    const char *e = std::getenv(name);
    if (!e || !*e) return dflt;
    char *end = nullptr;
    const long v = std::strtol(e, &end, 10);
    return (end && *end == 0 && v >= 0) ? v : dflt;
}

// Integrand adaptor type F of the fill templates: static f (value) and df
// (gradient w.r.t. theta) forwarding to the user's `integrand` /
// `integrand_grad`, qualified by `ns` (a namespace prefix, or "").
std::string fn_struct(const char *name, const cvg_integrand_s &f, int abi, int n_params, int grad,
                      const std::string &ns)
{
    std::string s = std::string("struct ") + name + " {\n";
    s += "  template <class T> static __device__ __forceinline__ T f(T* x, const T* th) {\n";
    if (abi == CVG_ABI_NUMBA)
        s += "    (void)th; double r = 0.0; " + ns + "integrand(&r, x); return r;\n";
    else if (n_params > 0)
        s += "    return " + ns + "integrand(x, th);\n";
    else
        s += "    (void)th; return " + ns + "integrand(x);\n";
    s += "  }\n";
    s += "  template <class T> static __device__ __forceinline__ void df(T* x, const T* th, T* g) {\n";
    if (grad) s += "    " + ns + "integrand_grad(x, th, g);\n";
    else s += "    (void)x; (void)th; (void)g;\n";
    s += "  }\n};\n";
    (void)f;
    return s;
}

std::string make_source(const cvg_integrand_s &f, const variant_key &k)
{
    const char *T = k.prec == CVG_PREC_FP32 ? "float" : "double";
    std::string s;
    s += "#define CVG_JIT 1\n";
    s += "#define CVG_FILL_WARP_TILES " + std::to_string(k.wt) + "\n";
    s += cvg_src_common;
    s += "\nstatic constexpr int cvg_n_dim = " + std::to_string(k.dim) + ";\n";
    s += "#line 1 \"integrand.cu\"\n";
    s += f.source;
    s += "\n#line 1 \"cvg_adaptor\"\n";
    s += cvg_src_fill;
    s += fn_struct("cvg_fn_user", f, k.abi, k.n_params, k.grad, "");
    char entry[1024];
    std::snprintf(entry, sizeof(entry),
                  "\nextern \"C\" __global__ void __launch_bounds__(%d, %d) cvg_fill_entry("
                  "const cvg_fill_args a) { cvg_fill_body<%d, %s, %d, %s, %s, %s, %d, %s, cvg_fn_user, %d>(a); }\n"
                  "extern \"C\" __global__ void __launch_bounds__(256) cvg_pilot_entry("
                  "const cvg_fill_args a) { cvg_pilot_body<%d, %s, 256, %d, cvg_fn_user>(a, blockIdx.x); }\n",
                  k.block, k.minb > 0 ? k.minb : 1, k.dim, T, k.block, k.esm ? "true" : "false",
                  k.hsm ? "true" : "false", k.replay ? "true" : "false", k.n_params,
                  k.grad ? "true" : "false", k.nbins, k.dim, T, k.n_params);
    s += entry;
    return s;
}

cvg_status nvrtc_cubin(const std::string &src, const std::vector<std::string> &opts,
                       std::vector<char> &cubin, std::string &log)
{
    nvrtcProgram prog;
    if (nvrtcCreateProgram(&prog, src.c_str(), "cvg_fill.cu", 0, nullptr, nullptr) != NVRTC_SUCCESS)
        return fail(CVG_ERR_COMPILE, "nvrtcCreateProgram failed");
    std::vector<const char *> copts;
    for (auto &o : opts) copts.push_back(o.c_str());
    nvrtcResult rc = nvrtcCompileProgram(prog, (int)copts.size(), copts.data());
    size_t logn = 0;
    nvrtcGetProgramLogSize(prog, &logn);
    log.assign(logn, '\0');
    if (logn) nvrtcGetProgramLog(prog, &log[0]);
    if (rc != NVRTC_SUCCESS) {
        nvrtcDestroyProgram(&prog);
        return fail(CVG_ERR_COMPILE,
                    std::string("integrand compile failed: ") + nvrtcGetErrorString(rc) + "\n" + log);
    }
    size_t n = 0;
    nvrtcGetCUBINSize(prog, &n);
    cubin.resize(n);
    nvrtcGetCUBIN(prog, cubin.data());
    nvrtcDestroyProgram(&prog);
    return CVG_OK;
}

std::vector<std::string> nvrtc_options(const std::string &arch)
{
    std::vector<std::string> o = {"--gpu-architecture=" + arch, "-std=c++17", "-default-device",
                                  "-lineinfo"};
    const char *extra = std::getenv("CVG_NVRTC_EXTRA");   // e.g. --ptxas-options=-v
    if (extra && *extra) {                                 // space-separated options
        std::string opt;
        for (const char *c = extra;; ++c) {
            if (*c == ' ' || *c == '\0') {
                if (!opt.empty()) o.push_back(opt);
                opt.clear();
                if (!*c) break;
            } else {
                opt += *c;
            }
        }
    }
    return o;
}

// Link a relocatable fill cubin with the integrand's PTX into one cubin.
cvg_status jit_link(const std::vector<char> &obj, const std::string &ptx, const std::string &arch,
                    std::vector<char> &out)
{
    const std::string a = "-arch=" + arch;
    const char *opts[] = {a.c_str()};
    nvJitLinkHandle h = nullptr;
    if (nvJitLinkCreate(&h, 1, opts) != NVJITLINK_SUCCESS) return fail(CVG_ERR_COMPILE, "nvJitLinkCreate failed");
    nvJitLinkResult rc = nvJitLinkAddData(h, NVJITLINK_INPUT_CUBIN, obj.data(), obj.size(), "cvg_fill");
    if (rc == NVJITLINK_SUCCESS)
        rc = nvJitLinkAddData(h, NVJITLINK_INPUT_PTX, ptx.c_str(), ptx.size() + 1, "integrand.ptx");
    if (rc == NVJITLINK_SUCCESS) rc = nvJitLinkComplete(h);
    if (rc != NVJITLINK_SUCCESS) {
        size_t n = 0;
        std::string log;
        if (nvJitLinkGetErrorLogSize(h, &n) == NVJITLINK_SUCCESS && n) {
            log.assign(n, '\0');
            nvJitLinkGetErrorLog(h, &log[0]);
        }
        nvJitLinkDestroy(&h);
        return fail(CVG_ERR_COMPILE, "linking the integrand PTX failed (" + std::to_string((int)rc) + "): " + log);
    }
    size_t n = 0;
    nvJitLinkGetLinkedCubinSize(h, &n);
    out.resize(n);
    nvJitLinkGetLinkedCubin(h, out.data());
    nvJitLinkDestroy(&h);
    return CVG_OK;
}

cvg_status load_module(cvg_context ctx, const std::string &src, cudaLibrary_t *out,
                       const std::string &link_ptx = std::string())
{
    std::vector<std::string> opts = nvrtc_options(ctx->arch);
    if (!link_ptx.empty()) opts.push_back("-rdc=true");
    int nv_major = 0, nv_minor = 0;
    nvrtcVersion(&nv_major, &nv_minor);
    std::string keystr = src;
    for (auto &o : opts) keystr += "\n" + o;
    keystr += "\n" + link_ptx;
    keystr += "\nnvrtc " + std::to_string(nv_major) + "." + std::to_string(nv_minor);
    keystr += "\n" CVG_VERSION;
    const uint64_t key = fnv1a(keystr);

    std::lock_guard<std::mutex> lock(ctx->mu);
    auto it = ctx->libs.find(key);
    cudaLibrary_t lib = nullptr;
    if (it != ctx->libs.end()) {
        lib = it->second;
    } else {
        char name[64];
        std::snprintf(name, sizeof(name), "%016llx.cubin", (unsigned long long)key);
        const std::string dir = cache_dir();
        const std::string path = dir + "/" + name;
        std::vector<char> cubin;
        if (!read_file(path, cubin)) {
            std::string log;
            CKS(nvrtc_cubin(src, opts, cubin, log));
            if (!link_ptx.empty()) {
                std::vector<char> linked;
                CKS(jit_link(cubin, link_ptx, ctx->arch, linked));
                cubin.swap(linked);
            }
            mkdirs(dir);
            write_file(path, cubin);
        }
        CK(cudaSetDevice(ctx->device));
        CK(cudaLibraryLoadData(&lib, cubin.data(), nullptr, nullptr, 0, nullptr, nullptr, 0));
        ctx->libs[key] = lib;
    }
    *out = lib;
    return CVG_OK;
}

cvg_status jit_kernel(cvg_context ctx, const cvg_integrand_s &f, const variant_key &k,
                      cudaKernel_t *out, cudaKernel_t *pilot = nullptr)
{
    cudaLibrary_t lib = nullptr;
    CKS(load_module(ctx, make_source(f, k), &lib, f.link_ptx));
    CK(cudaLibraryGetKernel(out, lib, "cvg_fill_entry"));
    if (pilot) CK(cudaLibraryGetKernel(pilot, lib, "cvg_pilot_entry"));
    return CVG_OK;
}

cvg_status prepare_variant(cvg_run_s *r, bool replay, bool grad, fill_variant *v)
{
    cvg_context ctx = r->ctx;
    const int tsz = r->p.precision == CVG_PREC_FP32 ? 4 : 8;
    variant_key k{r->f->dim, r->p.precision, r->block, r->esm, r->hsm, replay ? 1 : 0,
                  r->f->n_params, grad ? 1 : 0, r->f->abi, r->p.n_intervals, 1, r->wt};
    if (grad) k.hsm = 0;
    const cvg_u64 smem = cvg_fill_smem_bytes(k.dim, r->p.n_intervals, tsz, k.esm, k.hsm, k.grad,
                                             r->TS, k.n_params, k.block,
                                             r->wt ? k.block / 32 : 1);
    k.minb = cvg_internal_fill_minb(ctx, k.block, smem);
    CKS(jit_kernel(ctx, *r->f, k, &v->kernel, &v->pilot));
    const void *fn = (const void *)v->kernel;
    CK(cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    int occ = 0;
    CK(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, fn, r->block, smem));
    if (occ < 1) return fail(CVG_ERR_INVALID, "fill kernel cannot be resident (smem/regs)");
    v->smem = smem;
    v->occ = occ;
    return CVG_OK;
}

// Choose whether the grid and the bin histograms live in shared memory.
void choose_layout(cvg_run_s *r)
{
    const int tsz = r->p.precision == CVG_PREC_FP32 ? 4 : 8;
    const int budget = r->ctx->smem_optin - 256;   // the kernel's static shared words
    const int D = r->f->dim, N = r->p.n_intervals, P = r->f->n_params;
    const int opts[4][2] = {{1, 1}, {0, 1}, {1, 0}, {0, 0}};
    for (auto &o : opts) {
        if (cvg_fill_smem_bytes(D, N, tsz, o[0], o[1], 0, r->TS, P, r->block,
                                r->wt ? r->block / 32 : 1) <= (cvg_u64)budget) {
            r->esm = o[0];
            r->hsm = o[1];
            return;
        }
    }
    r->esm = 0;
    r->hsm = 0;
}

cvg_realloc_args realloc_args(cvg_run_s *r)
{
    cvg_realloc_args a{};
    a.nh_sum = r->nh_sum;
    a.JF = r->JF;
    a.JF2 = r->JF2;
    a.dh = r->dh;
    a.nh_new = r->nh_new;
    a.partials = r->partials;
    a.bsums = r->bsums;
    a.tile_cube = r->tile_cube;
    a.stats = r->stats;
    a.acc = r->acc;
    a.iteration = r->iteration;
    a.status = r->status;
    a.scale_exp = r->p.precision == CVG_PREC_FP32 ? r->scale_exp : nullptr;
    a.done = r->done;
    a.max_tiles = r->max_tiles;
    a.n_eval_it = r->n_eval_it;
    a.v_cubes = r->v_cubes;
    a.beta = r->p.beta;
    a.n_cubes = r->n_cubes;
    a.tile_samples = r->TS;
    a.skip = r->p.skip;
    a.max_it = r->p.max_it;
    a.fast_pow = r->p.precision == CVG_PREC_FP32 ? 1 : 0;
    a.adapt = (r->p.flags & CVG_FLAG_NO_ADAPT) ? 0 : 1;
    a.hist_state = r->p.precision == CVG_PREC_FP32 ? r->hist_state : nullptr;
    a.dim = r->f->dim;
    a.rare_shift = 10;    // fixed point while rare updates stay below 1 in 1024
    a.hist_min_it = 2;    // float bin sums in the fill after the first reallocation
    a.lb = r->lb;
    a.lb_ctl = r->lb_ctl;
    a.small_chunks = 1;
    a.lb_spin_limit = r->lb_spin_limit;
    a.lb_withhold = r->lb_withhold;
    return a;
}

cvg_refine_args refine_args(cvg_run_s *r)
{
    cvg_refine_args a{};
    a.x_edges = r->x_edges;
    a.x_edges32 = r->x_edges32;
    a.weights = r->weights;
    a.counts = r->counts;
    a.bin_exp = r->p.precision == CVG_PREC_FP32 ? r->bin_exp : nullptr;
    a.alpha = r->p.alpha;
    a.dim = r->f->dim;
    a.n_intervals = r->p.n_intervals;
    a.adapt = (r->p.flags & CVG_FLAG_NO_ADAPT) ? 0 : 1;
    return a;
}

cvg_fill_args fill_args(cvg_run_s *r)
{
    cvg_fill_args a{};
    a.x_edges = r->x_edges;
    a.x_edges32 = r->x_edges32;
    a.nh_sum = r->nh_sum;
    a.tile_cube = r->tile_cube;
    a.iteration = r->iteration;
    a.ubuf = r->ubuf;
    a.theta = r->theta;
    a.JF = r->JF;
    a.JF2 = r->JF2;
    a.weights = r->weights;
    a.counts = r->counts;
    a.grad = r->grad;
    a.status = r->status;
    a.tile_ctl = r->tile_ctl;
    a.scale_exp = r->p.precision == CVG_PREC_FP32 ? r->scale_exp : nullptr;
    a.scale_ss = r->p.precision == CVG_PREC_FP32 ? r->scale_ss : nullptr;
    a.bin_exp = r->p.precision == CVG_PREC_FP32 ? r->bin_exp : nullptr;
    a.hist_state = r->p.precision == CVG_PREC_FP32 ? r->hist_state : nullptr;
    a.max_tiles = r->max_tiles;
    a.seed = r->p.seed;
    a.instance = r->p.instance;
    a.n_cubes = r->n_cubes;
    a.n_strat = r->n_strat;
    a.n_intervals = r->p.n_intervals;
    a.tile_samples = r->TS;
    a.spt = r->spt;
    a.n_params = r->f->n_params;
    a.shard = r->shard;
    a.shards = r->shards;
    a.v_cubes = r->v_cubes;
    cvg_philox_schedule(r->p.seed, a.keys);
    return a;
}

cvg_status launch_fill(cvg_run_s *r, const fill_variant &v, bool timed)
{
    cvg_fill_args a = fill_args(r);
    if (&v == &r->gradk) a.shards = 1;   // the gradient pass covers every sample
    void *args[] = {&a};
    const int grid = (int)std::min<cvg_u64>((cvg_u64)v.occ * r->ctx->n_sm, r->max_tiles);
    r->grid = std::max(grid, 1);
    cudaEvent_t e0 = r->ev0, e1 = r->ev1;
    const bool each = timed && (r->p.flags & CVG_FLAG_TIME_FILL);
    if (each) {
        if (r->fill_ev_used == r->fill_ev.size()) {
            cudaEvent_t x, y;
            CK(cudaEventCreate(&x));
            CK(cudaEventCreate(&y));
            r->fill_ev.emplace_back(x, y);
        }
        e0 = r->fill_ev[r->fill_ev_used].first;
        e1 = r->fill_ev[r->fill_ev_used].second;
        r->fill_ev_used++;
    }
    if (timed) CK(cudaEventRecord(e0, r->ctx->stream));
    CK(cudaLaunchKernel((const void *)v.kernel, dim3(r->grid), dim3(r->block), args, v.smem,
                        r->ctx->stream));
    if (timed) CK(cudaEventRecord(e1, r->ctx->stream));
    if (each) {   // keep "last fill" queries valid
        r->ev0 = e0;
        r->ev1 = e1;
    }
    return CVG_OK;
}

// FP32 form: choose the scale exponent of f*jac from a pilot evaluation
cvg_status run_pilot(cvg_run_s *r)
{
    const int init = -1000;
    cudaStream_t st = r->ctx->stream;
    CK(cudaMemcpyAsync(r->scale_exp, &init, sizeof(int), cudaMemcpyHostToDevice, st));
    CK(cudaMemsetAsync(r->scale_ss, 0, sizeof(double), st));
    cvg_fill_args a = fill_args(r);
    void *args[] = {&a};
    const cvg_u64 pts = (cvg_u64)r->ctx->n_sm * 1024;   // ~150 samples per bin at 1024 bins
    const unsigned blocks = (unsigned)((pts + 255) / 256);
    CK(cudaLaunchKernel((const void *)r->fill.pilot, dim3(blocks), dim3(256), args, 0, st));
    // the pilot's bin histograms -> the first fill's per-bin exponents (grid kept)
    cvg_refine_args q = refine_args(r);
    q.adapt = 0;
    CK(cvg_launch_refine(q, st));
    int e = 0;
    double ss = 0.0;
    CK(cudaMemcpyAsync(&e, r->scale_exp, sizeof(int), cudaMemcpyDeviceToHost, st));
    CK(cudaMemcpyAsync(&ss, r->scale_ss, sizeof(double), cudaMemcpyDeviceToHost, st));
    CK(cudaStreamSynchronize(st));
    e = cvg_internal_pilot_scale(e, ss, (double)blocks * 256.0);
    CK(cudaMemcpyAsync(r->scale_exp, &e, sizeof(int), cudaMemcpyHostToDevice, st));
    return CVG_OK;
}

cvg_status enqueue_stages(cvg_run_s *r, int stages, bool timed)
{
    cudaStream_t s = r->ctx->stream;
    if (stages & CVG_STAGE_FILL) {
        if (r->replay) {
            cvg_u64 S = 0;   // the replay buffer must cover every sample of this fill
            CK(cudaMemcpyAsync(&S, r->nh_sum + r->n_cubes, sizeof(S), cudaMemcpyDeviceToHost, s));
            CK(cudaStreamSynchronize(s));
            if (S > r->ubuf_samples)
                return fail(CVG_ERR_INVALID, "replay uniforms cover " + std::to_string(r->ubuf_samples) +
                                                 " samples, the fill needs " + std::to_string(S));
            if (!r->fill_replay.kernel) CKS(prepare_variant(r, true, false, &r->fill_replay));
            CKS(launch_fill(r, r->fill_replay, timed));
        } else {
            CKS(launch_fill(r, r->fill, timed));
        }
    }
    if ((stages & CVG_STAGE_REFINE) && (stages & CVG_STAGE_REALLOC) &&
        r->p.precision == CVG_PREC_FP32) {
        // independent: the grid refinement (few CTAs, latency bound) overlaps the
        // reallocation (HBM bound); joined before the next fill.  FP32 form
        // only: beside the FP64 form's reallocation, itself bound by this GPU's
        // FP64 pipe, the refinement's clusters share its SMs and the iteration
        // slows (graph replay, d=4, 1e6 evaluations: 0.88 ms forked, 0.38 ms
        // in sequence; FP32 form 0.051 ms forked, 0.064 ms in sequence)
        cudaStream_t aux = r->ctx->aux;
        CK(cudaEventRecord(r->ev_fork, s));
        CK(cudaStreamWaitEvent(aux, r->ev_fork, 0));
        CK(cvg_launch_refine(refine_args(r), aux));
        CK(cudaEventRecord(r->ev_join, aux));
        CK(cvg_launch_realloc(realloc_args(r), s));
        CK(cudaStreamWaitEvent(s, r->ev_join, 0));
    } else {
        if (stages & CVG_STAGE_REFINE) CK(cvg_launch_refine(refine_args(r), s));
        if (stages & CVG_STAGE_REALLOC) CK(cvg_launch_realloc(realloc_args(r), s));
    }
    return CVG_OK;
}

cvg_status check_status(cvg_run_s *r)
{
    cvg_u32 st = 0;
    CK(cudaMemcpyAsync(&st, r->status, sizeof(st), cudaMemcpyDeviceToHost, r->ctx->stream));
    CK(cudaStreamSynchronize(r->ctx->stream));
    // a timed-out wait comes first: it leaves the prefix and tile map that
    // the next fill then finds inconsistent
    if (st & CVG_KSTAT_TIMEOUT)
        return fail(CVG_ERR_KERNEL, "the reallocation's look-back wait ran out; results are not valid");
    if (st & CVG_KSTAT_BAD_TILE)
        return fail(CVG_ERR_KERNEL, "fill kernel found an inconsistent tile map");
    return CVG_OK;
}

}  // namespace

// ---------------------------------------------------------------------------
// Library-internal helpers used by the batch driver (cvg_internal.h)
// ---------------------------------------------------------------------------
cvg_status cvg_internal_fail(cvg_status st, const std::string &msg) { return fail(st, msg); }
cvg_status cvg_internal_load_module(cvg_context ctx, const std::string &src, cudaLibrary_t *lib,
                                    const std::string &link_ptx)
{
    return load_module(ctx, src, lib, link_ptx);
}
std::string cvg_internal_fn_struct(const char *name, const cvg_integrand_s &f, int abi,
                                   int n_params, int grad, const std::string &ns)
{
    return fn_struct(name, f, abi, n_params, grad, ns);
}
cvg_status cvg_internal_compile_only(const std::string &src, const char *arch, std::string &log)
{
    std::vector<char> cubin;
    return nvrtc_cubin(src, nvrtc_options(arch), cubin, log);
}
const char *cvg_internal_src_common() { return cvg_src_common; }
const char *cvg_internal_src_fill() { return cvg_src_fill; }
double cvg_internal_now_ms() { return now_ms(); }

cudaError_t cvg_internal_arena_alloc(cvg_context ctx, size_t bytes, void **out, size_t *got)
{
    {
        std::lock_guard<std::mutex> lock(ctx->arena_mu);
        auto it = ctx->arena_cache.lower_bound(bytes);
        if (it != ctx->arena_cache.end() && it->first <= 2 * bytes) {
            *out = it->second;
            *got = it->first;
            ctx->arena_cached -= it->first;
            ctx->arena_cache.erase(it);
            // a debugging aid: NaN doubles / huge integers in every byte a run
            // forgets to initialise
            if (ctx->arena_poison) return cudaMemsetAsync(*out, 0xFF, *got, ctx->stream);
            return cudaSuccess;
        }
    }
    cudaError_t e = cudaMalloc(out, bytes);
    if (e == cudaErrorMemoryAllocation) {   // give the cached arenas back and retry once
        cudaGetLastError();
        cvg_context_trim(ctx);
        e = cudaMalloc(out, bytes);
    }
    *got = e == cudaSuccess ? bytes : 0;
    if (e == cudaSuccess && ctx->arena_poison) e = cudaMemsetAsync(*out, 0xFF, bytes, ctx->stream);
    return e;
}

void cvg_internal_arena_free(cvg_context ctx, void *p, size_t bytes)
{
    if (!p) return;
    std::lock_guard<std::mutex> lock(ctx->arena_mu);
    if (bytes > ctx->arena_cache_cap) {
        cudaFree(p);
        return;
    }
    ctx->arena_cache.emplace(bytes, p);
    ctx->arena_cached += bytes;
    while (ctx->arena_cached > ctx->arena_cache_cap && !ctx->arena_cache.empty()) {
        auto big = std::prev(ctx->arena_cache.end());     // drop the largest first
        ctx->arena_cached -= big->first;
        cudaFree(big->second);
        ctx->arena_cache.erase(big);
    }
}

int cvg_internal_fill_minb(cvg_context ctx, int block, size_t smem)
{
    // without a context (compile checks): the 228 KB of an sm_100/sm_103 SM
    const size_t per_sm = ctx && ctx->smem_per_sm > 0 ? (size_t)ctx->smem_per_sm : 233472u;
    const int by_smem = (int)(per_sm / (smem + 1024));
    const int by_regs = 65536 / (block * 64);
    return std::max(1, std::min(by_smem, by_regs));
}

int cvg_internal_pilot_scale(int emax, double ss, double n)
{
    if (emax < -100) return 0;                  // no finite nonzero value seen: no scaling
    int k = emax;
    const double ms = ss / n;
    if (ms > 0.0 && std::isfinite(ms)) {
        int e = 0;
        std::frexp(ms, &e);
        k = std::max(e / 2, emax - 60);
    }
    return std::min(std::max(k, -100), 100);
}

void cvg_internal_result(const double *stats, int max_it, int done, int skip, cvg_result *out)
{
    // weighted mean over iterations >= skip (src/main.cu:698-714), error
    // 1/sqrt(sum 1/sigma^2) (src/main.cu:792); chi^2 two-pass
    // An iteration with zero variance (an integrand constant on every
    // hypercube; a roundoff-negative sum counts too) is exact: the result is
    // then the mean of the exact iterations with error 0, where the
    // reference's 1/sigma^2 weights give inf/inf = NaN.
    const int M = max_it;
    double sw = 0.0, swr = 0.0, s0 = 0.0;
    int used = 0, n0 = 0;
    for (int i = skip; i < done; ++i) {
        if (!(stats[M + i] > 0.0)) { s0 += stats[i]; ++n0; }
        sw += 1.0 / stats[M + i];
        swr += stats[i] / stats[M + i];
        ++used;
    }
    out->result = n0 ? s0 / n0 : (used ? swr / sw : 0.0);
    out->error = n0 ? 0.0 : (used ? 1.0 / std::sqrt(sw) : 0.0);
    double chi2 = 0.0;
    for (int i = skip; i < done && !n0; ++i) {
        const double dlt = stats[i] - out->result;
        chi2 += dlt * dlt / stats[M + i];
    }
    out->chi2_dof = used > 1 ? chi2 / (used - 1) : 0.0;
    out->n_it_used = used;
    out->n_it_done = done;
}

// ---------------------------------------------------------------------------
// C ABI
// ---------------------------------------------------------------------------
extern "C" {

const char *cvg_last_error(void) { return g_err.c_str(); }
const char *cvg_version(void) { return CVG_VERSION; }

cvg_status cvg_context_create(int device, void *stream, cvg_context *out)
{
    if (!out) return fail(CVG_ERR_INVALID, "out is NULL");
    *out = nullptr;
    int ndev = 0;
    CK(cudaGetDeviceCount(&ndev));
    if (device < 0 || device >= ndev) return fail(CVG_ERR_INVALID, "no such device");
    CK(cudaSetDevice(device));
    auto *c = new cvg_context_s();
    c->device = device;
    cudaDeviceProp prop;
    cudaError_t e = cudaGetDeviceProperties(&prop, device);
    if (e != cudaSuccess) { delete c; return fail(CVG_ERR_CUDA, cudaGetErrorString(e)); }
    c->n_sm = prop.multiProcessorCount;
    c->smem_optin = (int)prop.sharedMemPerBlockOptin;
    c->smem_per_sm = (int)prop.sharedMemPerMultiprocessor;
    c->cc_major = prop.major;
    c->cc_minor = prop.minor;
    {   // arenas kept for reuse: up to CVG_ARENA_CACHE_MB (default 1/8 of the device)
        const char *cap = std::getenv("CVG_ARENA_CACHE_MB");
        c->arena_cache_cap = cap ? (size_t)std::strtoull(cap, nullptr, 10) << 20 : prop.totalGlobalMem / 8;
        const char *poison = std::getenv("CVG_ARENA_POISON");
        c->arena_poison = poison && *poison && *poison != '0';
    }
    char arch[32];
    std::snprintf(arch, sizeof(arch), "sm_%d%da", prop.major, prop.minor);
    c->arch = arch;
    e = cudaStreamCreateWithFlags(&c->aux, cudaStreamNonBlocking);
    if (e != cudaSuccess) { delete c; return fail(CVG_ERR_CUDA, cudaGetErrorString(e)); }
    if (stream) {
        c->stream = (cudaStream_t)stream;
    } else {
        e = cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking);
        if (e != cudaSuccess) { delete c; return fail(CVG_ERR_CUDA, cudaGetErrorString(e)); }
        c->own_stream = true;
    }
    *out = c;
    return CVG_OK;
}

cvg_status cvg_context_trim(cvg_context ctx)
{
    if (!ctx) return fail(CVG_ERR_INVALID, "NULL context");
    std::lock_guard<std::mutex> lock(ctx->arena_mu);
    cudaSetDevice(ctx->device);
    for (auto &kv : ctx->arena_cache) cudaFree(kv.second);
    ctx->arena_cache.clear();
    ctx->arena_cached = 0;
    return CVG_OK;
}

cvg_status cvg_context_destroy(cvg_context ctx)
{
    if (!ctx) return CVG_OK;
    cudaSetDevice(ctx->device);
    if (ctx->stream) cudaStreamSynchronize(ctx->stream);
    cvg_context_trim(ctx);
    for (auto &kv : ctx->libs) cudaLibraryUnload(kv.second);
    if (ctx->own_stream) cudaStreamDestroy(ctx->stream);
    if (ctx->aux) cudaStreamDestroy(ctx->aux);
    delete ctx;
    return CVG_OK;
}

cvg_status cvg_compile_integrand(cvg_context ctx, const char *source, int32_t n_dim, int32_t abi,
                                 int32_t n_params, int32_t has_grad, cvg_integrand *out)
{
    if (!ctx || !source || !out) return fail(CVG_ERR_INVALID, "NULL argument");
    if (n_dim < 1 || n_dim > 32) return fail(CVG_ERR_INVALID, "n_dim must be in [1, 32]");
    if (n_params < 0 || n_params > 64) return fail(CVG_ERR_INVALID, "n_params must be in [0, 64]");
    if (abi != CVG_ABI_NATIVE && abi != CVG_ABI_NUMBA) return fail(CVG_ERR_INVALID, "bad abi");
    if (abi == CVG_ABI_NUMBA && (n_params || has_grad))
        return fail(CVG_ERR_INVALID, "numba ABI takes no parameters");
    auto *f = new cvg_integrand_s();
    f->ctx = ctx;
    f->source = source;
    f->dim = n_dim;
    f->abi = abi;
    f->n_params = n_params;
    f->has_grad = has_grad ? 1 : 0;
    // Kernels are compiled on first use (run creation), per precision and tile
    // shape; source errors are reported there with the NVRTC log.
    *out = f;
    return CVG_OK;
}

cvg_status cvg_compile_integrand_ptx(cvg_context ctx, const char *source, const char *ptx,
                                     int32_t n_dim, cvg_integrand *out)
{
    if (!ctx || !ptx || !out) return fail(CVG_ERR_INVALID, "NULL argument");
    if (n_dim < 1 || n_dim > 32) return fail(CVG_ERR_INVALID, "n_dim must be in [1, 32]");
    if (!std::strstr(ptx, ".func")) return fail(CVG_ERR_INVALID, "ptx defines no device function");
    auto *f = new cvg_integrand_s();
    f->ctx = ctx;
    f->source = (source && *source)
                    ? std::string(source)
                    : std::string("extern \"C\" __device__ int integrand(double* ret, double* x);\n");
    f->link_ptx = ptx;
    f->dim = n_dim;
    f->abi = CVG_ABI_NUMBA;
    *out = f;
    return CVG_OK;
}

cvg_status cvg_integrand_release(cvg_integrand f)
{
    delete f;
    return CVG_OK;
}

cvg_status cvg_run_create(cvg_context ctx, cvg_integrand f, const cvg_params *pp,
                          const double *theta, cvg_run *out)
{
    if (!ctx || !f || !pp || !out) return fail(CVG_ERR_INVALID, "NULL argument");
    *out = nullptr;
    const cvg_params &p = *pp;
    if (p.n_dim != f->dim) return fail(CVG_ERR_INVALID, "n_dim differs from the integrand's");
    if (p.max_it < 1) return fail(CVG_ERR_INVALID, "max_it must be >= 1");
    if (p.skip < 0) return fail(CVG_ERR_INVALID, "skip must be >= 0");
    if (p.tot_eval < 1) return fail(CVG_ERR_INVALID, "tot_eval must be >= 1");
    if (p.n_intervals < 2 || p.n_intervals > CVG_REFINE_MAX_N)
        return fail(CVG_ERR_INVALID, "n_intervals must be in [2, 4096]");
    if (p.precision != CVG_PREC_FP64 && p.precision != CVG_PREC_FP32)
        return fail(CVG_ERR_INVALID, "precision must be CVG_PREC_FP64 or CVG_PREC_FP32");
    if (!(p.alpha >= 0.0) || !(p.beta >= 0.0)) return fail(CVG_ERR_INVALID, "alpha, beta >= 0");
    if (f->n_params > 0 && !theta) return fail(CVG_ERR_INVALID, "integrand needs theta");
    if (f->abi == CVG_ABI_NUMBA && p.precision != CVG_PREC_FP64)
        return fail(CVG_ERR_INVALID, "numba ABI integrands are FP64");

    auto *r = new cvg_run_s();
    r->ctx = ctx;
    r->f = f;
    r->p = p;
    // sizing: src/main.cu:304, 329-331, 337, 444-445
    r->n_eval_it = p.tot_eval / p.max_it;
    const int D = f->dim;
    r->n_strat = p.n_strat > 0 ? p.n_strat : (int)std::pow((double)r->n_eval_it / 4.0, 1.0 / D);
    if (r->n_strat < 1) { delete r; return fail(CVG_ERR_INVALID, "evals per iteration too small for one stratum (n_strat < 1)"); }
    const double nc = std::pow((double)r->n_strat, (double)D);
    if (nc > 4294967295.0) { delete r; return fail(CVG_ERR_INVALID, "n_strat^n_dim exceeds 2^32-1 hypercubes"); }
    r->n_cubes = (cvg_u32)nc;
    r->v_cubes = std::pow(1.0 / r->n_strat, (double)D);
    const cvg_u64 s_max = (cvg_u64)r->n_eval_it + 2ull * r->n_cubes;
    if (s_max >= (1ull << 31) - (1ull << 20)) {
        delete r;
        return fail(CVG_ERR_INVALID, "evals per iteration + 2*n_cubes must stay below 2^31");
    }
    const int64_t nh0 = std::max<int64_t>(2, (int64_t)(1.0 / (double)r->n_cubes * (double)r->n_eval_it));

    // bounded look-back wait of the one-pass allocation: CVG_LB_SPIN_LIMIT
    // polls (default 2^22) before it gives up and reports CVG_ERR_KERNEL;
    // CVG_TEST_LB_WITHHOLD = 1 + a chunk index makes that chunk never publish
    // its word, so the failure test sees the wait run out (0 / unset: none)
    r->lb_spin_limit = (int)std::min<long>(env_long("CVG_LB_SPIN_LIMIT", 0), 1L << 30);
    r->lb_withhold = (cvg_u32)std::min<long>(env_long("CVG_TEST_LB_WITHHOLD", 0), 0xFFFFFFFFL);

    // tile shape
    const int wt_env = env_warp_tiles();
    r->wt = wt_env != 0 ? 1 : 0;
    r->block = p.block > 0 ? p.block : 512;
    r->spt = p.spt > 0 ? p.spt : 8;
    if (r->block % 32 || r->block > 1024) { delete r; return fail(CVG_ERR_INVALID, "block must be a multiple of 32, <= 1024"); }
    if (r->spt < 1 || r->spt > 256) { delete r; return fail(CVG_ERR_INVALID, "spt must be in [1, 256]"); }
    const int tsz = p.precision == CVG_PREC_FP32 ? 4 : 8;
    auto ctas = [&](int spt) {   // fill CTAs per SM that shared memory allows
        const int TS = r->wt ? 32 * spt : r->block * spt;
        for (auto &o : {std::pair<int, int>{1, 1}, {0, 1}, {1, 0}, {0, 0}}) {
            const cvg_u64 b = cvg_fill_smem_bytes(D, p.n_intervals, tsz, o.first, o.second, 0, TS,
                                                  f->n_params, r->block,
                                                  r->wt ? r->block / 32 : 1);
            if (b + 256 <= (cvg_u64)ctx->smem_optin) return (int)(ctx->smem_per_sm / (b + 1024));
        }
        return 0;
    };
    if (p.spt <= 0) {
        // default: 16 samples per thread (half the per-tile staging of 8;
        // measured 4 % faster at d = 8 and d = 16) unless the larger
        // cube-start table costs a CTA per SM ... and unless the iteration has too few tiles to give every CTA of
        // the persistent grid several (small runs keep more, smaller tiles)
        const cvg_u64 tiles16 = s_max / ((cvg_u64)r->block * 16);
        const int c16 = ctas(16);
        if (c16 >= ctas(8) && c16 > 0 && tiles16 >= 4ull * (cvg_u64)c16 * ctx->n_sm) r->spt = 16;
    }
    // warp tiles pay off when every warp of the persistent grid gets several
    // (measured on GB300: d=8, 1e8 samples, fill 1.870 -> 1.758 ms; d=4,
    // 1e6 samples, one or two tiles per warp, 0.029 -> 0.031 ms)
    if (r->wt && wt_env < 0) {
        // resident CTAs: shared memory, and registers at 64 per thread (the
        // fill's launch bounds), whichever is fewer
        const int res = std::max(1, std::min(ctas(r->spt), 65536 / (r->block * 64)));
        const cvg_u64 warps = (cvg_u64)res * ctx->n_sm * (r->block / 32);
        if (s_max / (32ull * r->spt) < 4ull * warps) r->wt = 0;
    }
    // warp tiles: larger tiles (fewer cube-start loads and searches per
    // sample) where shared memory keeps the CTAs per SM, and one block of
    // 1024 where two 512-thread CTAs would each be held to 64 registers
    // anyway (one copy of the grid and histograms per SM leaves room for
    // the larger cube-start buffers).  Measured on GB300, fill ms: d=8 1e8
    // FP32 512x16 1.720, 1024x16 1.695, 1024x24 1.674, 1024x32 1.663; d=16
    // 1e9 FP32 512x16 26.16, 512x24 25.72, 512x32 25.50.
    if (r->wt && p.block <= 0 && p.spt <= 0) {
        if (ctas(16) >= 2) r->block = 1024;
        const int base = ctas(16);
        for (int s : {32, 24})
            if (base > 0 && ctas(s) >= base) { r->spt = s; break; }
    }
    r->TS = r->wt ? 32 * r->spt : r->block * r->spt;
    r->max_tiles = (s_max + r->TS - 1) / r->TS + 1;
    r->nb = cvg_realloc_blocks(r->n_cubes);
    choose_layout(r);

    cudaError_t e = cudaSetDevice(ctx->device);
    if (e != cudaSuccess) { delete r; return fail(CVG_ERR_CUDA, cudaGetErrorString(e)); }

    // arena
    const int N = p.n_intervals;
    struct seg { void **ptr; size_t bytes; };
    std::vector<seg> segs = {
        {(void **)&r->x_edges, sizeof(double) * D * (N + 1)},
        {(void **)&r->x_edges32, sizeof(float) * D * (N + 1)},
        {(void **)&r->weights, sizeof(double) * D * N},
        {(void **)&r->counts, sizeof(cvg_u32) * D * N},
        {(void **)&r->JF, sizeof(double) * r->n_cubes},
        {(void **)&r->JF2, sizeof(double) * r->n_cubes},
        {(void **)&r->dh, sizeof(double) * r->n_cubes},
        {(void **)&r->nh_sum, sizeof(cvg_u64) * ((size_t)r->n_cubes + 1)},
        {(void **)&r->nh_new, sizeof(cvg_u32) * r->n_cubes},
        {(void **)&r->tile_cube, sizeof(cvg_u32) * r->max_tiles},
        {(void **)&r->partials, sizeof(double) * 4 * 4 * r->nb},   // small_chunks: 4x blocks
        {(void **)&r->bsums, sizeof(cvg_u64) * (r->nb + 1)},
        {(void **)&r->stats, sizeof(double) * 3 * p.max_it},
        {(void **)&r->acc, sizeof(cvg_acc_dev)},
        {(void **)&r->iteration, sizeof(cvg_u32)},
        {(void **)&r->status, sizeof(cvg_u32)},
        {(void **)&r->scale_exp, sizeof(int)},
        {(void **)&r->scale_ss, sizeof(double)},
        {(void **)&r->bin_exp, sizeof(int) * ((size_t)D * N + 1)},
        {(void **)&r->hist_state, 2 * sizeof(cvg_u32)},
        {(void **)&r->lb, sizeof(cvg_u64) * r->nb},
        {(void **)&r->lb_ctl, 2 * sizeof(cvg_u32)},
        {(void **)&r->tile_ctl, 2 * sizeof(cvg_u32)},
        {(void **)&r->done, 2 * sizeof(cvg_u32)},
        {(void **)&r->theta, sizeof(double) * std::max(1, f->n_params)},
        {(void **)&r->grad, sizeof(double) * std::max(1, f->n_params)},
    };
    size_t total = 0;
    for (auto &s : segs) total += (s.bytes + 255) & ~(size_t)255;
    e = cvg_internal_arena_alloc(ctx, total, &r->arena, &r->arena_bytes);
    if (e != cudaSuccess) {
        delete r;
        return fail(CVG_ERR_NOMEM, std::string("cudaMalloc of the run arena (") +
                                       std::to_string(total >> 20) + " MiB): " + cudaGetErrorString(e));
    }
    size_t off = 0;
    for (auto &s : segs) {
        *s.ptr = (char *)r->arena + off;
        off += (s.bytes + 255) & ~(size_t)255;
    }
    // initial state; on failure the half-built run is destroyed here
    const cvg_status ist = [&]() -> cvg_status {
    cudaStream_t st = ctx->stream;
    CK(cudaEventCreate(&r->ev0));
    CK(cudaEventCreate(&r->ev1));
    r->ev0_own = r->ev0;
    r->ev1_own = r->ev1;
    CK(cudaEventCreateWithFlags(&r->ev_fork, cudaEventDisableTiming));
    CK(cudaEventCreateWithFlags(&r->ev_join, cudaEventDisableTiming));
    // uniform grid x_j = j/N (src/main.cu:432-441)
    std::vector<double> xe((size_t)D * (N + 1));
    const double step = 1.0 / N;
    for (int d = 0; d < D; ++d)
        for (int j = 0; j <= N; ++j) xe[(size_t)d * (N + 1) + j] = j * step;
    CK(cudaMemcpyAsync(r->x_edges, xe.data(), sizeof(double) * xe.size(), cudaMemcpyHostToDevice, st));
    CK(cvg_launch_grid32(r->x_edges, r->x_edges32, D * (N + 1), st));
    CK(cudaMemsetAsync(r->weights, 0, sizeof(double) * D * N, st));
    CK(cudaMemsetAsync(r->counts, 0, sizeof(cvg_u32) * D * N, st));
    CK(cudaMemsetAsync(r->JF, 0, sizeof(double) * r->n_cubes, st));
    CK(cudaMemsetAsync(r->JF2, 0, sizeof(double) * r->n_cubes, st));
    CK(cudaMemsetAsync(r->acc, 0, sizeof(cvg_acc_dev), st));
    CK(cudaMemsetAsync(r->iteration, 0, sizeof(cvg_u32), st));
    CK(cudaMemsetAsync(r->status, 0, sizeof(cvg_u32), st));
    CK(cudaMemsetAsync(r->done, 0, 2 * sizeof(cvg_u32), st));
    CK(cudaMemsetAsync(r->lb, 0, sizeof(cvg_u64) * r->nb, st));
    CK(cudaMemsetAsync(r->lb_ctl, 0, 2 * sizeof(cvg_u32), st));
    CK(cudaMemsetAsync(r->tile_ctl, 0, 2 * sizeof(cvg_u32), st));
    // the first fill keeps float bin sums: the pilot's ~150 samples per bin
    // cannot bound the mean of a heavy-tailed bin (a d=16 Gaussian lost 2.8 %
    // of a dimension's sum to fixed point on the pilot's table); fixed point
    // starts from the third fill, on a table built from a whole fill's sums
    CK(cudaMemsetAsync(r->hist_state, 0, 2 * sizeof(cvg_u32), st));
    CK(cudaMemsetAsync(r->stats, 0, sizeof(double) * 3 * p.max_it, st));
    CK(cudaMemsetAsync(r->grad, 0, sizeof(double) * std::max(1, f->n_params), st));
    if (f->n_params > 0)
        CK(cudaMemcpyAsync(r->theta, theta, sizeof(double) * f->n_params, cudaMemcpyHostToDevice, st));
    // nh init (src/main.cu:443-448) -> prefix and tile map
    CK(cvg_launch_fill_u32(r->nh_new, (cvg_u32)nh0, r->n_cubes, st));
    CK(cvg_launch_set_nh(realloc_args(r), r->nh_new, st));
    CKS(prepare_variant(r, false, false, &r->fill));
    CK(cudaMemsetAsync(r->scale_exp, 0, sizeof(int), st));
    if (p.precision == CVG_PREC_FP32) CKS(run_pilot(r));
    CK(cudaStreamSynchronize(st));
    return CVG_OK;
    }();
    if (ist != CVG_OK) {
        cvg_run_destroy(r);
        return ist;
    }
    *out = r;
    return CVG_OK;
}

cvg_status cvg_run_destroy(cvg_run r)
{
    if (!r) return CVG_OK;
    cudaSetDevice(r->ctx->device);
    cudaStreamSynchronize(r->ctx->stream);
    if (r->graph_exec) cudaGraphExecDestroy(r->graph_exec);
    if (r->graph) cudaGraphDestroy(r->graph);
    // ev0/ev1 alias either the run's own pair or a pair of fill_ev
    for (auto &pr : r->fill_ev) { cudaEventDestroy(pr.first); cudaEventDestroy(pr.second); }
    if (r->ev0_own) cudaEventDestroy(r->ev0_own);
    if (r->ev1_own) cudaEventDestroy(r->ev1_own);
    if (r->ev_fork) cudaEventDestroy(r->ev_fork);
    if (r->ev_join) cudaEventDestroy(r->ev_join);
    if (r->ubuf) cudaFree(r->ubuf);
    if (r->arena) cvg_internal_arena_free(r->ctx, r->arena, r->arena_bytes);
    delete r;
    return CVG_OK;
}

cvg_status cvg_run_step(cvg_run r, int32_t stages)
{
    if (!r) return fail(CVG_ERR_INVALID, "NULL run");
    CK(cudaSetDevice(r->ctx->device));
    if ((stages & CVG_STAGE_REALLOC) && r->it_done >= r->p.max_it)
        return fail(CVG_ERR_STATE, "all max_it iterations are done");
    CKS(enqueue_stages(r, stages, (stages & CVG_STAGE_FILL) != 0));
    if (stages & CVG_STAGE_REALLOC) r->it_done++;
    return CVG_OK;
}

cvg_status cvg_run_iterate(cvg_run r, int32_t n)
{
    if (!r) return fail(CVG_ERR_INVALID, "NULL run");
    if (n < 0 || r->it_done + n > r->p.max_it)
        return fail(CVG_ERR_STATE, "iterations beyond max_it");
    CK(cudaSetDevice(r->ctx->device));
    const int all = CVG_STAGE_FILL | CVG_STAGE_REFINE | CVG_STAGE_REALLOC;
    if ((r->p.flags & CVG_FLAG_GRAPH) && !r->replay) {
        if (!r->graph_exec) {
            cudaStream_t s = r->ctx->stream;
            CK(cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal));
            cvg_status st = enqueue_stages(r, all, false);
            cudaGraph_t g = nullptr;
            cudaError_t e = cudaStreamEndCapture(s, &g);
            if (st != CVG_OK) { if (g) cudaGraphDestroy(g); return st; }
            CK(e);
            r->graph = g;
            CK(cudaGraphInstantiate(&r->graph_exec, g, 0));
        }
        for (int i = 0; i < n; ++i) CK(cudaGraphLaunch(r->graph_exec, r->ctx->stream));
    } else {
        const bool each = (r->p.flags & CVG_FLAG_TIME_FILL) != 0;
        for (int i = 0; i < n; ++i) CKS(enqueue_stages(r, all, each || i == n - 1));
    }
    r->it_done += n;
    return CVG_OK;
}

cvg_status cvg_run_sync(cvg_run r)
{
    if (!r) return fail(CVG_ERR_INVALID, "NULL run");
    CK(cudaSetDevice(r->ctx->device));
    return check_status(r);
}

cvg_status cvg_run_result(cvg_run r, cvg_result *out, double *it_res, double *it_sig2)
{
    if (!r || !out) return fail(CVG_ERR_INVALID, "NULL argument");
    CK(cudaSetDevice(r->ctx->device));
    const int M = r->p.max_it;
    std::vector<double> stats(3 * (size_t)M);
    CK(cudaMemcpyAsync(stats.data(), r->stats, sizeof(double) * 3 * M, cudaMemcpyDeviceToHost,
                       r->ctx->stream));
    CKS(check_status(r));
    std::memset(out, 0, sizeof(*out));
    const int done = std::min(r->it_done, M);
    cvg_internal_result(stats.data(), M, done, r->p.skip, out);
    out->n_strat = r->n_strat;
    out->n_intervals = r->p.n_intervals;
    out->n_cubes = r->n_cubes;
    double nev = 0.0;   // samples of every iteration done (also those of an imported state)
    for (int i = 0; i < done; ++i) nev += stats[2 * (size_t)M + i];
    out->tot_nevals = (int64_t)nev;
    out->seed = r->p.seed;
    out->gpu_thr = r->p.gpu_thr;
    out->precision = r->p.precision;
    if (it_res) for (int i = 0; i < M; ++i) it_res[i] = stats[i];
    if (it_sig2) for (int i = 0; i < M; ++i) it_sig2[i] = stats[M + i];
    return CVG_OK;
}

cvg_status cvg_integrate(cvg_context ctx, cvg_integrand f, const cvg_params *p,
                         const double *theta, cvg_result *out, double *it_res, double *it_sig2)
{
    if (!out) return fail(CVG_ERR_INVALID, "out is NULL");
    const double t0 = now_ms();
    cvg_run r = nullptr;
    cvg_status s = cvg_run_create(ctx, f, p, theta, &r);
    if (s != CVG_OK) { cvg_run_destroy(r); return s; }
    const double t1 = now_ms();
    s = cvg_run_iterate(r, p->max_it);
    if (s == CVG_OK) s = cvg_run_result(r, out, it_res, it_sig2);
    const double t2 = now_ms();
    cvg_run_destroy(r);
    out->tot_time_ms = now_ms() - t0;
    out->avg_it_time_ms = (t2 - t1) / p->max_it;
    return s;
}

cvg_status cvg_run_get(cvg_run r, int32_t buf, void *host, size_t bytes)
{
    if (!r || !host) return fail(CVG_ERR_INVALID, "NULL argument");
    CK(cudaSetDevice(r->ctx->device));
    const int D = r->f->dim, N = r->p.n_intervals;
    const void *src = nullptr;
    size_t need = 0;
    switch (buf) {
    case CVG_BUF_X_EDGES: src = r->x_edges; need = sizeof(double) * D * (N + 1); break;
    case CVG_BUF_NH: {
        std::vector<cvg_u64> ps((size_t)r->n_cubes + 1);
        need = sizeof(cvg_u32) * r->n_cubes;
        if (bytes != need) return fail(CVG_ERR_INVALID, "size mismatch");
        CK(cudaMemcpyAsync(ps.data(), r->nh_sum, sizeof(cvg_u64) * ps.size(), cudaMemcpyDeviceToHost, r->ctx->stream));
        CK(cudaStreamSynchronize(r->ctx->stream));
        cvg_u32 *o = (cvg_u32 *)host;
        for (size_t c = 0; c < r->n_cubes; ++c) o[c] = (cvg_u32)(ps[c + 1] - ps[c]);
        return CVG_OK;
    }
    case CVG_BUF_NH_SUM: src = r->nh_sum; need = sizeof(cvg_u64) * ((size_t)r->n_cubes + 1); break;
    case CVG_BUF_JF: src = r->JF; need = sizeof(double) * r->n_cubes; break;
    case CVG_BUF_JF2: src = r->JF2; need = sizeof(double) * r->n_cubes; break;
    case CVG_BUF_WEIGHTS: src = r->weights; need = sizeof(double) * D * N; break;
    case CVG_BUF_COUNTS: src = r->counts; need = sizeof(cvg_u32) * D * N; break;
    case CVG_BUF_DH:
        src = r->dh;
        need = sizeof(double) * r->n_cubes;
        if (r->p.precision == CVG_PREC_FP32) {   // stored as float by the FP32 form
            if (bytes != need) return fail(CVG_ERR_INVALID, "size mismatch");
            std::vector<float> tmp(r->n_cubes);
            CK(cudaMemcpyAsync(tmp.data(), r->dh, sizeof(float) * tmp.size(), cudaMemcpyDeviceToHost,
                               r->ctx->stream));
            CK(cudaStreamSynchronize(r->ctx->stream));
            double *o = (double *)host;
            for (size_t c = 0; c < tmp.size(); ++c) o[c] = tmp[c];
            return CVG_OK;
        }
        break;
    case CVG_BUF_THETA: src = r->theta; need = sizeof(double) * r->f->n_params; break;
    case CVG_BUF_ITERATION: src = r->iteration; need = sizeof(cvg_u32); break;
    case CVG_BUF_STATS: src = r->stats; need = sizeof(double) * 3 * r->p.max_it; break;
    case CVG_BUF_SCALE_EXP: src = r->scale_exp; need = sizeof(int); break;
    case CVG_BUF_BIN_EXP: src = r->bin_exp; need = sizeof(int) * ((size_t)D * N + 1); break;
    case CVG_BUF_HIST_STATE: src = r->hist_state; need = 2 * sizeof(cvg_u32); break;
    case CVG_BUF_TILE_CUBE: src = r->tile_cube; need = sizeof(cvg_u32) * r->max_tiles; break;
    default: return fail(CVG_ERR_INVALID, "unknown buffer");
    }
    if (bytes != need) return fail(CVG_ERR_INVALID, "size mismatch: expected " + std::to_string(need));
    CK(cudaMemcpyAsync(host, src, need, cudaMemcpyDeviceToHost, r->ctx->stream));
    CK(cudaStreamSynchronize(r->ctx->stream));
    return CVG_OK;
}

cvg_status cvg_run_set_shard(cvg_run r, int32_t shard, int32_t shards)
{
    if (!r) return fail(CVG_ERR_INVALID, "NULL run");
    if (shards < 1 || shard < 0 || shard >= shards)
        return fail(CVG_ERR_INVALID, "shard must lie in [0, shards), shards >= 1");
    if (r->graph_exec)
        return fail(CVG_ERR_STATE, "set the shard before the first CUDA-graph iteration");
    r->shard = (cvg_u32)shard;
    r->shards = (cvg_u32)shards;
    return CVG_OK;
}

cvg_status cvg_run_buffer(cvg_run r, int32_t buf, void **device_ptr, size_t *bytes)
{
    if (!r || !device_ptr || !bytes) return fail(CVG_ERR_INVALID, "NULL argument");
    const int D = r->f->dim, N = r->p.n_intervals;
    switch (buf) {
    case CVG_BUF_X_EDGES: *device_ptr = r->x_edges; *bytes = sizeof(double) * D * (N + 1); break;
    case CVG_BUF_NH_SUM: *device_ptr = r->nh_sum; *bytes = sizeof(cvg_u64) * ((size_t)r->n_cubes + 1); break;
    case CVG_BUF_JF: *device_ptr = r->JF; *bytes = sizeof(double) * r->n_cubes; break;
    case CVG_BUF_JF2: *device_ptr = r->JF2; *bytes = sizeof(double) * r->n_cubes; break;
    case CVG_BUF_WEIGHTS: *device_ptr = r->weights; *bytes = sizeof(double) * D * N; break;
    case CVG_BUF_COUNTS: *device_ptr = r->counts; *bytes = sizeof(cvg_u32) * D * N; break;
    case CVG_BUF_HIST_STATE:
        if (r->p.precision != CVG_PREC_FP32) return fail(CVG_ERR_INVALID, "FP64 runs keep no histogram state");
        *device_ptr = r->hist_state; *bytes = 2 * sizeof(cvg_u32); break;
    default: return fail(CVG_ERR_INVALID, "no device view of this buffer");
    }
    return CVG_OK;
}

cvg_status cvg_run_set(cvg_run r, int32_t buf, const void *host, size_t bytes)
{
    if (!r) return fail(CVG_ERR_INVALID, "NULL run");
    CK(cudaSetDevice(r->ctx->device));
    const int D = r->f->dim, N = r->p.n_intervals;
    cudaStream_t st = r->ctx->stream;
    void *dst = nullptr;
    size_t need = 0;
    switch (buf) {
    case CVG_BUF_X_EDGES: dst = r->x_edges; need = sizeof(double) * D * (N + 1); break;
    case CVG_BUF_NH: {
        need = sizeof(cvg_u32) * r->n_cubes;
        if (!host || bytes != need) return fail(CVG_ERR_INVALID, "size mismatch");
        const cvg_u32 *nh = (const cvg_u32 *)host;
        cvg_u64 tot = 0;
        for (size_t c = 0; c < r->n_cubes; ++c) {
            if (nh[c] < 2) return fail(CVG_ERR_INVALID, "every hypercube needs >= 2 samples");
            tot += nh[c];
        }
        if (tot > (cvg_u64)(r->max_tiles - 1) * r->TS)
            return fail(CVG_ERR_INVALID, "sum of nh exceeds evals/iteration + 2*n_cubes");
        CK(cvg_launch_set_nh(realloc_args(r), nh, st));
        CK(cudaStreamSynchronize(st));
        return CVG_OK;
    }
    case CVG_BUF_JF: dst = r->JF; need = sizeof(double) * r->n_cubes; break;
    case CVG_BUF_JF2: dst = r->JF2; need = sizeof(double) * r->n_cubes; break;
    case CVG_BUF_WEIGHTS: dst = r->weights; need = sizeof(double) * D * N; break;
    case CVG_BUF_COUNTS: dst = r->counts; need = sizeof(cvg_u32) * D * N; break;
    case CVG_BUF_THETA: dst = r->theta; need = sizeof(double) * r->f->n_params; break;
    case CVG_BUF_ITERATION:
        dst = r->iteration;
        need = sizeof(cvg_u32);
        if (host && bytes == need) {   // the loop continues from this iteration
            const cvg_u32 it = *(const cvg_u32 *)host;
            if (it > (cvg_u32)r->p.max_it) return fail(CVG_ERR_INVALID, "iteration beyond max_it");
            r->it_done = (int)it;
        }
        break;
    case CVG_BUF_SCALE_EXP: dst = r->scale_exp; need = sizeof(int); break;
    case CVG_BUF_STATS: dst = r->stats; need = sizeof(double) * 3 * r->p.max_it; break;
    case CVG_BUF_BIN_EXP: dst = r->bin_exp; need = sizeof(int) * ((size_t)D * N + 1); break;
    case CVG_BUF_HIST_STATE: dst = r->hist_state; need = 2 * sizeof(cvg_u32); break;
    case CVG_BUF_UNIFORMS: {
        if (bytes == 0) { r->replay = false; return CVG_OK; }
        if (!host || bytes % (sizeof(float) * D)) return fail(CVG_ERR_INVALID, "uniforms: [S][dim] floats");
        const size_t ns = bytes / (sizeof(float) * D);
        if (ns > r->ubuf_samples) {
            if (r->ubuf) CK(cudaFree(r->ubuf));
            r->ubuf = nullptr;
            r->ubuf_samples = 0;
            CK(cudaMalloc(&r->ubuf, bytes));
            r->ubuf_samples = ns;
        }
        CK(cudaMemcpyAsync(r->ubuf, host, bytes, cudaMemcpyHostToDevice, st));
        CK(cudaStreamSynchronize(st));
        r->replay = true;
        return CVG_OK;
    }
    default: return fail(CVG_ERR_INVALID, "buffer not settable");
    }
    if (!host || bytes != need) return fail(CVG_ERR_INVALID, "size mismatch: expected " + std::to_string(need));
    CK(cudaMemcpyAsync(dst, host, need, cudaMemcpyHostToDevice, st));
    if (buf == CVG_BUF_X_EDGES) {
        CK(cvg_launch_grid32(r->x_edges, r->x_edges32, D * (N + 1), st));
        // the exponent table belongs to the old grid: float bin sums next
        CK(cudaMemsetAsync(r->hist_state, 0, 2 * sizeof(cvg_u32), st));
    }
    CK(cudaStreamSynchronize(st));
    return CVG_OK;
}

cvg_status cvg_run_info_get(cvg_run r, cvg_run_info *o)
{
    if (!r || !o) return fail(CVG_ERR_INVALID, "NULL argument");
    CK(cudaSetDevice(r->ctx->device));
    cvg_u64 S = 0;
    CK(cudaMemcpyAsync(&S, r->nh_sum + r->n_cubes, sizeof(S), cudaMemcpyDeviceToHost, r->ctx->stream));
    CK(cudaStreamSynchronize(r->ctx->stream));
    std::memset(o, 0, sizeof(*o));
    o->n_eval_it = r->n_eval_it;
    o->n_cubes = r->n_cubes;
    o->next_samples = (int64_t)S;
    o->max_tiles = (int64_t)r->max_tiles;
    o->n_strat = r->n_strat;
    o->n_intervals = r->p.n_intervals;
    o->n_dim = r->f->dim;
    o->block = r->block;
    o->spt = r->spt;
    o->grid = (int32_t)std::min<cvg_u64>((cvg_u64)r->fill.occ * r->ctx->n_sm, r->max_tiles);
    o->edges_smem = r->esm;
    o->hist_smem = r->hsm;
    o->v_cubes = r->v_cubes;
    o->fill_smem_bytes = (int64_t)r->fill.smem;
    o->tile_samples = r->TS;
    o->warp_tiles = r->wt;
    return CVG_OK;
}

cvg_status cvg_run_grad(cvg_run r, uint32_t it, double *grad)
{
    if (!r || !grad) return fail(CVG_ERR_INVALID, "NULL argument");
    if (!r->f->has_grad || r->f->n_params < 1)
        return fail(CVG_ERR_INVALID, "integrand has no integrand_grad / parameters");
    CK(cudaSetDevice(r->ctx->device));
    if (!r->gradk.kernel) CKS(prepare_variant(r, false, true, &r->gradk));
    cudaStream_t st = r->ctx->stream;
    cvg_u32 saved = 0;
    if (it != 0xFFFFFFFFu) {
        CK(cudaMemcpyAsync(&saved, r->iteration, sizeof(saved), cudaMemcpyDeviceToHost, st));
        CK(cudaStreamSynchronize(st));
        CK(cudaMemcpyAsync(r->iteration, &it, sizeof(it), cudaMemcpyHostToDevice, st));
    }
    CK(cudaMemsetAsync(r->grad, 0, sizeof(double) * r->f->n_params, st));
    CKS(launch_fill(r, r->gradk, false));
    CK(cudaMemcpyAsync(grad, r->grad, sizeof(double) * r->f->n_params, cudaMemcpyDeviceToHost, st));
    if (it != 0xFFFFFFFFu)
        CK(cudaMemcpyAsync(r->iteration, &saved, sizeof(saved), cudaMemcpyHostToDevice, st));
    return check_status(r);
}

cvg_status cvg_run_fill_times(cvg_run r, float *ms, int32_t cap, int32_t *n)
{
    if (!r || !n) return fail(CVG_ERR_INVALID, "NULL argument");
    CK(cudaSetDevice(r->ctx->device));
    CK(cudaStreamSynchronize(r->ctx->stream));
    int32_t k = 0;
    for (size_t i = 0; i < r->fill_ev_used; ++i) {
        float t = 0.f;
        CK(cudaEventElapsedTime(&t, r->fill_ev[i].first, r->fill_ev[i].second));
        if (ms && k < cap) ms[k] = t;
        ++k;
    }
    *n = k;
    r->fill_ev_used = 0;
    return CVG_OK;
}

cvg_status cvg_measure_peak(cvg_context ctx, int32_t kind, double *out)
{
    if (!ctx || !out) return fail(CVG_ERR_INVALID, "NULL argument");
    CK(cudaSetDevice(ctx->device));
    cudaStream_t s = ctx->stream;
    cudaEvent_t a, b;
    CK(cudaEventCreate(&a));
    CK(cudaEventCreate(&b));
    float best = 1e30f;
    if (kind == 0 || kind == 1) {
        double *sink = nullptr;
        CK(cudaMalloc(&sink, sizeof(double)));
        const int blocks = ctx->n_sm * 8;
        const int iters = kind == 0 ? 4096 : 256;
        for (int rep = 0; rep < 4; ++rep) {
            CK(cudaEventRecord(a, s));
            CK(cvg_launch_fma_bench(kind, blocks, iters, sink, s));
            CK(cudaEventRecord(b, s));
            CK(cudaEventSynchronize(b));
            float t;
            CK(cudaEventElapsedTime(&t, a, b));
            if (rep > 0) best = std::min(best, t);
        }
        cudaFree(sink);
        const double flops = 2.0 * 8.0 * iters * 256.0 * blocks;
        *out = flops / (best * 1e-3) / 1e12;
    } else if (kind == 2) {
        const size_t bytes = (size_t)1 << 30;
        void *x = nullptr, *y = nullptr;
        CK(cudaMalloc(&x, bytes));
        cudaError_t e = cudaMalloc(&y, bytes);
        if (e != cudaSuccess) { cudaFree(x); return fail(CVG_ERR_NOMEM, cudaGetErrorString(e)); }
        CK(cudaMemsetAsync(x, 0, bytes, s));
        for (int rep = 0; rep < 6; ++rep) {
            CK(cudaEventRecord(a, s));
            CK(cvg_launch_copy_bench((const float4 *)x, (float4 *)y, bytes / 16, s));
            CK(cudaEventRecord(b, s));
            CK(cudaEventSynchronize(b));
            float t;
            CK(cudaEventElapsedTime(&t, a, b));
            if (rep > 0) best = std::min(best, t);
        }
        cudaFree(x);
        cudaFree(y);
        *out = 2.0 * bytes / (best * 1e-3) / 1e9;
    } else if (kind >= 3 && kind <= 6) {
        double *sink = nullptr;
        CK(cudaMalloc(&sink, sizeof(double)));
        const int blocks = ctx->n_sm * 2, iters = 4096;
        for (int rep = 0; rep < 4; ++rep) {
            CK(cudaEventRecord(a, s));
            CK(cvg_launch_smem_atomic_bench(kind - 3, blocks, iters, sink, s));
            CK(cudaEventRecord(b, s));
            CK(cudaEventSynchronize(b));
            float t;
            CK(cudaEventElapsedTime(&t, a, b));
            if (rep > 0) best = std::min(best, t);
        }
        cudaFree(sink);
        *out = (double)blocks * 512.0 * iters / (best * 1e-3) / 1e9;   // G atomics/s
    } else if (kind == 10 || kind == 11) {
        double *gw = nullptr;
        CK(cudaMalloc(&gw, 4096 * sizeof(double)));
        CK(cudaMemsetAsync(gw, 0, 4096 * sizeof(double), s));
        const int blocks = ctx->n_sm * 4, iters = 4096;
        for (int rep = 0; rep < 5; ++rep) {
            CK(cudaEventRecord(a, s));
            CK(cvg_launch_hist_update_bench(kind - 10, blocks, iters, gw, s));
            CK(cudaEventRecord(b, s));
            CK(cudaEventSynchronize(b));
            float t;
            CK(cudaEventElapsedTime(&t, a, b));
            if (rep > 0) best = std::min(best, t);
        }
        cudaFree(gw);
        *out = (double)blocks * 512.0 * iters / (best * 1e-3) / 1e9;   // G updates/s
    } else if (kind >= 7 && kind <= 9) {
        double *sink = nullptr;
        CK(cudaMalloc(&sink, sizeof(double)));
        const int blocks = ctx->n_sm * 8;
        const int iters = kind == 9 ? 256 : 2048;
        for (int rep = 0; rep < 4; ++rep) {
            CK(cudaEventRecord(a, s));
            CK(cvg_launch_pipe_bench(kind - 7, blocks, iters, sink, s));
            CK(cudaEventRecord(b, s));
            CK(cudaEventSynchronize(b));
            float t;
            CK(cudaEventElapsedTime(&t, a, b));
            if (rep > 0) best = std::min(best, t);
        }
        cudaFree(sink);
        const double per_iter = kind == 9 ? 4.0 : 8.0;   // Philox calls / ops per iteration
        *out = per_iter * iters * 256.0 * blocks / (best * 1e-3) / 1e12;   // T ops (calls)/s
    } else {
        return fail(CVG_ERR_INVALID, "kind must be in [0, 11]");
    }
    cudaEventDestroy(a);
    cudaEventDestroy(b);
    return CVG_OK;
}

cvg_status cvg_compile_check(const char *source, int32_t n_dim, int32_t abi, int32_t n_params,
                             int32_t has_grad, int32_t precision, const char *arch, char *log,
                             size_t log_len)
{
    if (!source || !arch) return fail(CVG_ERR_INVALID, "NULL argument");
    if (n_dim < 1 || n_dim > 32) return fail(CVG_ERR_INVALID, "n_dim must be in [1, 32]");
    cvg_integrand_s f;
    f.source = source;
    f.dim = n_dim;
    f.abi = abi;
    f.n_params = n_params;
    f.has_grad = has_grad;
    std::string all;
    cvg_status st = CVG_OK;
    for (int g = 0; g <= (has_grad ? 1 : 0) && st == CVG_OK; ++g) {
        // the default launch shape of a run (512 threads, 8 samples each,
        // 1024 bins, grid and histograms in shared memory when they fit)
        const int tsz = precision == CVG_PREC_FP32 ? 4 : 8;
        variant_key k{n_dim, precision, 512, 1, g ? 0 : 1, 0, n_params, g, abi, 1024, 1,
                      env_warp_tiles() != 0 ? 1 : 0};
        const int TS = k.wt ? 32 * 16 : 512 * 16, groups = k.wt ? 16 : 1;
        if (cvg_fill_smem_bytes(n_dim, 1024, tsz, 1, k.hsm, g, TS, n_params, 512, groups) > 232448)
            k.hsm = 0;
        k.minb = cvg_internal_fill_minb(nullptr, 512,
                                        cvg_fill_smem_bytes(n_dim, 1024, tsz, 1, k.hsm, g, TS,
                                                            n_params, 512, groups));
        std::vector<char> cubin;
        std::string l;
        st = nvrtc_cubin(make_source(f, k), nvrtc_options(arch), cubin, l);
        all += l;
    }
    if (log && log_len) {
        std::strncpy(log, all.c_str(), log_len - 1);
        log[log_len - 1] = '\0';
    }
    return st;
}

cvg_status cvg_run_last_fill_ms(cvg_run r, float *ms)
{
    if (!r || !ms) return fail(CVG_ERR_INVALID, "NULL argument");
    CK(cudaEventSynchronize(r->ev1));
    CK(cudaEventElapsedTime(ms, r->ev0, r->ev1));
    return CVG_OK;
}

}  // extern "C"
