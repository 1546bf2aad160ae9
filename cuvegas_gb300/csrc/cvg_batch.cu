// cvg_batch.cu -- many independent VEGAS+ integrals advanced together.
//
// Instances share one integrand family (one source, parameters theta per
// instance) but differ in dimension, evaluation count and parameters.  Per
// iteration the GPU runs, for the whole batch:
//   one persistent fill launch (tiles of every instance, dimensions
//   dispatched inside the kernel), the batched grid refinement (a cluster per
//   instance and dimension) and the batched reallocation (blocks of every
//   instance), which also numbers the tiles of the next fill.
// With CVG_FLAG_GRAPH the iteration is captured once as a CUDA graph and
// replayed.  Each instance reproduces a single-instance run with the same
// seed and instance id (same Philox samples, same arithmetic).
#include "cuvegas.h"
#include "cvg_internal.h"
#include "cvg_kernels.cuh"

#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <set>
#include <string>
#include <vector>

#define BCK(x)                                                                       \
    do {                                                                             \
        cudaError_t e_ = (x);                                                        \
        if (e_ != cudaSuccess)                                                       \
            return cvg_internal_fail(e_ == cudaErrorMemoryAllocation ? CVG_ERR_NOMEM \
                                                                     : CVG_ERR_CUDA, \
                                     std::string(#x) + ": " + cudaGetErrorString(e_)); \
    } while (0)
#define BCKS(x)                      \
    do {                             \
        cvg_status s_ = (x);         \
        if (s_ != CVG_OK) return s_; \
    } while (0)

namespace {

struct inst_host {
    int dim = 0, n_strat = 0, n_params = 0;
    int64_t n_eval_it = 0;
    cvg_u32 n_cubes = 0;
    double v_cubes = 0.0;
    unsigned nb = 0;
    cvg_u64 max_tiles = 0;
    cvg_u32 nh0 = 0;
    // device pointers
    double *x_edges, *weights, *JF, *JF2, *dh, *partials, *stats, *theta, *grad;
    float *x_edges32;
    cvg_u32 *counts, *nh_new, *tile_cube, *iteration;
    int *scale_exp;
    double *scale_ss;
    int *bin_exp;
    double *exp_dq;         // [0] sum of d_h * q; the int after it: the next fill's exponent shift
    cvg_u32 *done;
    cvg_u64 *nh_sum, *bsums, *lb;
    cvg_u32 *lb_ctl;
    cvg_acc_dev *acc;
};

}  // namespace

struct cvg_batch_s {
    cvg_context ctx = nullptr;
    cvg_integrand_s f;
    cvg_params p{};
    int n = 0, block = 0, spt = 0, TS = 0, grid = 0, it_done = 0;
    std::vector<inst_host> inst;
    std::vector<int> params_per_dim;
    void *arena = nullptr;
    size_t arena_bytes = 0;
    // device tables
    cvg_fill_args *d_fill = nullptr;
    cvg_realloc_args *d_realloc = nullptr;
    cvg_refine_args *d_refine = nullptr;
    int *d_dims = nullptr;
    unsigned *d_blk_base = nullptr, *d_dim_base = nullptr, *d_blk_inst = nullptr;
    cvg_u64 *d_tile_base = nullptr, *d_cost_base = nullptr;
    cvg_u64 *d_range_start = nullptr, *d_claim = nullptr;
    cvg_u32 *d_range_inst = nullptr;
    int max_ranges = 0;               // capacity of the range tables (32 CTAs per SM)
    cvg_u32 *d_status = nullptr;
    unsigned total_blocks = 0, total_dims = 0;
    cudaKernel_t fill = nullptr, pilot = nullptr;
    size_t fill_smem = 0;
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t graph_exec = nullptr;
    cudaEvent_t ev0 = nullptr, ev1 = nullptr, ev_fork = nullptr, ev_join = nullptr;
};

namespace {

size_t seg(size_t bytes) { return (bytes + 255) & ~(size_t)255; }

// Device buffers of one instance, in arena order.  With base == nullptr only
// the offset advances (sizing pass); otherwise the pointers are set too.
template <typename P> void place(P *&ptr, size_t bytes, char *base, size_t &off)
{
    if (base) ptr = (P *)(base + off);
    off += seg(bytes);
}

void inst_layout(inst_host &h, int N, int max_it, char *base, size_t &off)
{
    const size_t D = (size_t)h.dim;
    place(h.x_edges, sizeof(double) * D * (N + 1), base, off);
    place(h.x_edges32, sizeof(float) * D * (N + 1), base, off);
    place(h.weights, sizeof(double) * D * N, base, off);
    place(h.counts, sizeof(cvg_u32) * D * N, base, off);
    place(h.JF, sizeof(double) * h.n_cubes, base, off);
    place(h.JF2, sizeof(double) * h.n_cubes, base, off);
    place(h.dh, sizeof(double) * h.n_cubes, base, off);
    place(h.nh_sum, sizeof(cvg_u64) * (h.n_cubes + 1ull), base, off);
    place(h.nh_new, sizeof(cvg_u32) * h.n_cubes, base, off);
    place(h.tile_cube, sizeof(cvg_u32) * h.max_tiles, base, off);
    place(h.partials, sizeof(double) * 4 * h.nb, base, off);
    place(h.bsums, sizeof(cvg_u64) * (h.nb + 1), base, off);
    place(h.lb, sizeof(cvg_u64) * h.nb, base, off);
    place(h.lb_ctl, 16, base, off);
    place(h.stats, sizeof(double) * 3 * max_it, base, off);
    place(h.acc, sizeof(cvg_acc_dev), base, off);
    place(h.iteration, 16, base, off);
    place(h.scale_exp, 16, base, off);
    place(h.scale_ss, 16, base, off);
    place(h.done, 16, base, off);
    place(h.bin_exp, sizeof(int) * (D * N + 1), base, off);
    place(h.exp_dq, 16, base, off);
    place(h.theta, sizeof(double) * std::max(1, h.n_params), base, off);
    place(h.grad, sizeof(double) * std::max(1, h.n_params), base, off);
}

// Per-batch tables after the instances' buffers.
void tables_layout(cvg_batch_s *b, char *base, size_t &off)
{
    const size_t n = (size_t)b->n;
    place(b->d_status, 16, base, off);
    place(b->d_fill, sizeof(cvg_fill_args) * n, base, off);
    place(b->d_realloc, sizeof(cvg_realloc_args) * n, base, off);
    place(b->d_refine, sizeof(cvg_refine_args) * n, base, off);
    place(b->d_dims, sizeof(int) * n, base, off);
    place(b->d_blk_base, sizeof(unsigned) * (n + 1), base, off);
    place(b->d_blk_inst, sizeof(unsigned) * b->total_blocks, base, off);
    place(b->d_dim_base, sizeof(unsigned) * (n + 1), base, off);
    place(b->d_tile_base, sizeof(cvg_u64) * (n + 1), base, off);
    place(b->d_cost_base, sizeof(cvg_u64) * (n + 1), base, off);
    const size_t R = (size_t)b->max_ranges;
    place(b->d_range_start, sizeof(cvg_u64) * (R + 1), base, off);
    place(b->d_range_inst, sizeof(cvg_u32) * R, base, off);
    place(b->d_claim, sizeof(cvg_u64) * R, base, off);
}

std::string batch_source(const cvg_batch_s &b, const std::set<int> &dims)
{
    const char *T = b.p.precision == CVG_PREC_FP32 ? "float" : "double";
    std::string s = "#define CVG_JIT 1\n";
    // the one-dimension-at-a-time map: measured faster in the batched
    // kernel, which holds every dimension's variant at once (22.7 against
    // 25.1 G evals/s with the packed pairs)
    s += "#ifndef CVG_FILL_PAIRS\n#define CVG_FILL_PAIRS 0\n#endif\n";
    s += cvg_internal_src_common();
    for (int d : dims) {
        s += "\nnamespace cvg_d" + std::to_string(d) + " {\nstatic constexpr int cvg_n_dim = " +
             std::to_string(d) + ";\n#line 1 \"integrand.cu\"\n" + b.f.source + "\n}\n";
    }
    s += "#line 1 \"cvg_batch_adaptor\"\n";
    s += cvg_internal_src_fill();
    for (int d : dims)
        s += cvg_internal_fn_struct(("cvg_fn_d" + std::to_string(d)).c_str(), b.f, b.f.abi,
                                    b.params_per_dim[d], 0, "cvg_d" + std::to_string(d) + "::");
    s += "struct cvg_disp {\n  template <int D> struct sel;\n"
         "  template <int D> using fn = typename sel<D>::type;\n"
         "  template <class Op> static __device__ __forceinline__ void run(int dim, Op &&op) {\n"
         "    switch (dim) {\n";
    for (int d : dims)
        s += "      case " + std::to_string(d) + ": op(cvg_int<" + std::to_string(d) +
             ">{}, cvg_int<" + std::to_string(b.params_per_dim[d]) + ">{}); break;\n";
    s += "      default: break;\n    }\n  }\n};\n";
    for (int d : dims)
        s += "template <> struct cvg_disp::sel<" + std::to_string(d) + "> { using type = cvg_fn_d" +
             std::to_string(d) + "; };\n";
    char entry[512];
    std::snprintf(entry, sizeof(entry),
                  "extern \"C\" __global__ void __launch_bounds__(%d, %d) cvg_fill_batch_entry("
                  "const cvg_batch_args b) { cvg_fill_batch<%s, %d, cvg_disp, %d>(b); }\n"
                  "extern \"C\" __global__ void __launch_bounds__(256) cvg_pilot_batch_entry("
                  "const cvg_batch_args b) { cvg_pilot_batch<%s, 32, cvg_disp>(b); }\n",
                  b.block, cvg_internal_fill_minb(b.ctx, b.block, b.fill_smem), T, b.block,
                  b.p.n_intervals, T);
    s += entry;
    return s;
}

cvg_batch_args batch_args(const cvg_batch_s *b)
{
    cvg_batch_args a{};
    a.inst = b->d_fill;
    a.dims = b->d_dims;
    a.tile_base = b->d_tile_base;
    a.range_start = b->d_range_start;
    a.range_inst = b->d_range_inst;
    a.claim = b->d_claim;
    a.n_inst = b->n;
    a.n_ranges = b->grid;
    a.max_claim = (cvg_u32)(CVG_HIST_MAX_RUN / (unsigned)b->TS);
    cvg_philox_schedule(b->p.seed, a.keys);
    return a;
}

cvg_realloc_batch realloc_batch(const cvg_batch_s *b)
{
    cvg_realloc_batch B{};
    B.A = b->d_realloc;
    B.blk_base = b->d_blk_base;
    B.blk_inst = b->d_blk_inst;
    B.total_blocks = b->total_blocks;
    B.n = b->n;
    return B;
}

cvg_batch_sched batch_sched(const cvg_batch_s *b)
{
    cvg_batch_sched S{};
    S.tile_base = b->d_tile_base;
    S.cost_base = b->d_cost_base;
    S.range_start = b->d_range_start;
    S.range_inst = b->d_range_inst;
    S.claim = b->d_claim;
    S.n_ranges = b->grid;
    return S;
}

cvg_refine_batch refine_batch(const cvg_batch_s *b)
{
    cvg_refine_batch B{};
    B.R = b->d_refine;
    B.dim_base = b->d_dim_base;
    B.total_dims = b->total_dims;
    B.n = b->n;
    return B;
}

cvg_status enqueue_iteration(cvg_batch_s *b, bool timed)
{
    cudaStream_t s = b->ctx->stream;
    cvg_batch_args ba = batch_args(b);
    void *args[] = {&ba};
    if (timed) BCK(cudaEventRecord(b->ev0, s));
    BCK(cudaLaunchKernel((const void *)b->fill, dim3(b->grid), dim3(b->block), args, b->fill_smem, s));
    if (timed) BCK(cudaEventRecord(b->ev1, s));
    // refinement on the second stream, beside the reallocation
    cudaStream_t aux = b->ctx->aux;
    BCK(cudaEventRecord(b->ev_fork, s));
    BCK(cudaStreamWaitEvent(aux, b->ev_fork, 0));
    BCK(cvg_launch_refine_batch(refine_batch(b), b->p.n_intervals, aux));
    BCK(cudaEventRecord(b->ev_join, aux));
    BCK(cvg_launch_realloc_batch(realloc_batch(b), (b->p.flags & CVG_FLAG_NO_ADAPT) ? 0 : 1,
                                 b->p.precision == CVG_PREC_FP32, batch_sched(b), s));
    BCK(cudaStreamWaitEvent(s, b->ev_join, 0));
    return CVG_OK;
}

cvg_status batch_init(cvg_batch_s *b, const cvg_instance *insts, const double *theta,
                      const std::set<int> &dims, size_t total);

}  // namespace

extern "C" {

cvg_status cvg_batch_create(cvg_context ctx, const char *source, int32_t abi, int32_t n,
                            const cvg_instance *insts, const int32_t *params_per_dim,
                            const double *theta, const cvg_params *common, cvg_batch *out)
{
    if (!ctx || !source || !insts || !params_per_dim || !common || !out)
        return cvg_internal_fail(CVG_ERR_INVALID, "NULL argument");
    *out = nullptr;
    if (n < 1 || n > 65536) return cvg_internal_fail(CVG_ERR_INVALID, "batch size must be in [1, 65536]");
    const cvg_params &p = *common;
    if (p.max_it < 1 || p.skip < 0 || p.n_intervals < 2 || p.n_intervals > CVG_REFINE_MAX_N)
        return cvg_internal_fail(CVG_ERR_INVALID, "bad max_it / skip / n_intervals");
    if (p.precision != CVG_PREC_FP64 && p.precision != CVG_PREC_FP32)
        return cvg_internal_fail(CVG_ERR_INVALID, "bad precision");
    if (abi != CVG_ABI_NATIVE) return cvg_internal_fail(CVG_ERR_INVALID, "batches take the native integrand ABI");
    auto *b = new cvg_batch_s();
    b->ctx = ctx;
    b->f.ctx = ctx;
    b->f.source = source;
    b->f.abi = abi;
    b->p = p;
    b->n = n;
    b->params_per_dim.assign(params_per_dim, params_per_dim + 17);
    b->block = p.block > 0 ? p.block : 512;
    b->spt = p.spt > 0 ? p.spt : 8;
    if (b->block % 32 || b->block > 1024 || b->spt < 1 || b->spt > 256) {
        delete b;
        return cvg_internal_fail(CVG_ERR_INVALID, "bad block / spt");
    }
    b->TS = 32 * b->spt;   // warp tiles
    b->max_ranges = 32 * std::max(1, ctx->n_sm);
    const int N = p.n_intervals;
    std::set<int> dims;
    int dmax = 0, pmax = 0;
    b->inst.resize(n);
    size_t total = 0;
    for (int i = 0; i < n; ++i) {
        inst_host &h = b->inst[i];
        const cvg_instance &in = insts[i];
        if (in.n_dim < 1 || in.n_dim > 16 || in.tot_eval < 1) {
            delete b;
            return cvg_internal_fail(CVG_ERR_INVALID, "instance " + std::to_string(i) +
                                                          ": n_dim must be in [1, 16], tot_eval >= 1");
        }
        h.dim = in.n_dim;
        h.n_params = params_per_dim[in.n_dim];
        h.n_eval_it = in.tot_eval / p.max_it;
        h.n_strat = in.n_strat > 0 ? in.n_strat : (int)std::pow((double)h.n_eval_it / 4.0, 1.0 / h.dim);
        if (h.n_strat < 1) { delete b; return cvg_internal_fail(CVG_ERR_INVALID, "instance " + std::to_string(i) + ": too few evaluations"); }
        const double nc = std::pow((double)h.n_strat, (double)h.dim);
        const cvg_u64 s_max = (cvg_u64)h.n_eval_it + 2ull * (cvg_u64)nc;
        if (nc > 4294967295.0 || s_max >= (1ull << 31) - (1ull << 20)) {
            delete b;
            return cvg_internal_fail(CVG_ERR_INVALID, "instance " + std::to_string(i) + " too large");
        }
        h.n_cubes = (cvg_u32)nc;
        h.v_cubes = std::pow(1.0 / h.n_strat, (double)h.dim);
        h.nh0 = (cvg_u32)std::max<int64_t>(2, (int64_t)(1.0 / (double)h.n_cubes * (double)h.n_eval_it));
        h.nb = cvg_realloc_blocks(h.n_cubes);
        if ((uint64_t)b->total_blocks + h.nb > 0x7FFFFFFFull) {
            delete b;
            return cvg_internal_fail(CVG_ERR_INVALID, "batch: too many hypercubes in all");
        }
        b->total_blocks += h.nb;
        h.max_tiles = (s_max + b->TS - 1) / b->TS + 1;
        dims.insert(h.dim);
        dmax = std::max(dmax, h.dim);
        pmax = std::max(pmax, h.n_params);
        inst_layout(h, N, p.max_it, nullptr, total);
    }
    tables_layout(b, nullptr, total);
    const int tsz = p.precision == CVG_PREC_FP32 ? 4 : 8;
    b->fill_smem = cvg_fill_smem_bytes(dmax, N, tsz, 1, 1, 0, b->TS, pmax, b->block, b->block / 32);
    // (+ the fill's few static bytes: its claim slots)
    if (b->fill_smem + 64 > (size_t)ctx->smem_optin) {
        delete b;
        return cvg_internal_fail(CVG_ERR_INVALID, "batch: grid and histograms of the largest "
                                                  "dimension do not fit shared memory");
    }
    cudaError_t e = cudaSetDevice(ctx->device);
    if (e == cudaSuccess) e = cvg_internal_arena_alloc(ctx, total, &b->arena, &b->arena_bytes);
    if (e != cudaSuccess) {
        delete b;
        return cvg_internal_fail(CVG_ERR_NOMEM, std::string("batch arena: ") + cudaGetErrorString(e));
    }
    const cvg_status st_init = batch_init(b, insts, theta, dims, total);
    if (st_init != CVG_OK) {
        cvg_batch_destroy(b);
        return st_init;
    }
    *out = b;
    return CVG_OK;
}

}  // extern "C"

namespace {

// Second half of cvg_batch_create: lays out the arena, uploads the instances'
// initial state and tables, compiles the fill and runs the FP32 pilot.  On
// failure the caller destroys the half-built batch.
cvg_status batch_init(cvg_batch_s *b, const cvg_instance *insts, const double *theta,
                      const std::set<int> &dims, size_t total)
{
    const int n = b->n;
    const cvg_params &p = b->p;
    const int N = p.n_intervals;
    cvg_context ctx = b->ctx;
    cudaStream_t st = ctx->stream;
    BCK(cudaMemsetAsync(b->arena, 0, total, st));
    char *base = (char *)b->arena;
    size_t off = 0;
    std::vector<cvg_fill_args> hf(n);
    std::vector<cvg_realloc_args> hr(n);
    std::vector<cvg_refine_args> hq(n);
    std::vector<int> hdims(n);
    std::vector<unsigned> blk_base(n + 1), dim_base(n + 1);
    std::vector<double> xe;
    for (int i = 0; i < n; ++i) inst_layout(b->inst[i], N, p.max_it, base, off);
    tables_layout(b, base, off);
    if (off != total) return cvg_internal_fail(CVG_ERR_STATE, "batch arena layout mismatch");
    size_t th_off = 0;
    for (int i = 0; i < n; ++i) {
        inst_host &h = b->inst[i];
        const int D = h.dim;
        // uniform grid (src/main.cu:432-441)
        xe.resize((size_t)D * (N + 1));
        for (int d = 0; d < D; ++d)
            for (int j = 0; j <= N; ++j) xe[(size_t)d * (N + 1) + j] = j * (1.0 / N);
        BCK(cudaMemcpyAsync(h.x_edges, xe.data(), sizeof(double) * xe.size(), cudaMemcpyHostToDevice, st));
        BCK(cvg_launch_grid32(h.x_edges, h.x_edges32, D * (N + 1), st));
        if (h.n_params > 0 && theta)
            BCK(cudaMemcpyAsync(h.theta, theta + th_off, sizeof(double) * h.n_params,
                                cudaMemcpyHostToDevice, st));
        th_off += h.n_params;
        BCK(cvg_launch_fill_u32(h.nh_new, h.nh0, h.n_cubes, st));
        BCK(cudaStreamSynchronize(st));   // xe is reused
        cvg_fill_args &a = hf[i];
        a.x_edges = h.x_edges;
        a.x_edges32 = h.x_edges32;
        a.nh_sum = h.nh_sum;
        a.tile_cube = h.tile_cube;
        a.iteration = h.iteration;
        a.theta = h.theta;
        a.JF = h.JF;
        a.JF2 = h.JF2;
        a.weights = h.weights;
        a.counts = h.counts;
        a.grad = h.grad;
        a.status = b->d_status;
        a.scale_exp = p.precision == CVG_PREC_FP32 ? h.scale_exp : nullptr;
        a.scale_ss = p.precision == CVG_PREC_FP32 ? h.scale_ss : nullptr;
        a.bin_exp = p.precision == CVG_PREC_FP32 ? h.bin_exp : nullptr;
        a.hist_state = nullptr;   // batched fills always keep fixed-point bin sums
        a.exp_shift = p.precision == CVG_PREC_FP32 ? reinterpret_cast<const int *>(h.exp_dq + 1)
                                                   : nullptr;
        a.max_tiles = h.max_tiles;
        a.seed = p.seed;
        a.instance = insts[i].instance;
        a.n_cubes = h.n_cubes;
        a.n_strat = h.n_strat;
        a.n_intervals = N;
        a.tile_samples = b->TS;
        a.spt = b->spt;
        a.n_params = h.n_params;
        a.v_cubes = h.v_cubes;
        cvg_philox_schedule(p.seed, a.keys);
        cvg_realloc_args &r = hr[i];
        r.nh_sum = h.nh_sum;
        r.JF = h.JF;
        r.JF2 = h.JF2;
        r.dh = h.dh;
        r.nh_new = h.nh_new;
        r.partials = h.partials;
        r.bsums = h.bsums;
        r.tile_cube = h.tile_cube;
        r.stats = h.stats;
        r.acc = h.acc;
        r.iteration = h.iteration;
        r.status = b->d_status;
        r.scale_exp = a.scale_exp;
        r.done = h.done;
        r.max_tiles = h.max_tiles;
        r.n_eval_it = h.n_eval_it;
        r.v_cubes = h.v_cubes;
        r.beta = p.beta;
        r.n_cubes = h.n_cubes;
        r.tile_samples = b->TS;
        r.skip = p.skip;
        r.max_it = p.max_it;
        r.fast_pow = p.precision == CVG_PREC_FP32 ? 1 : 0;
        r.hist_state = nullptr;
        r.exp_dq = p.precision == CVG_PREC_FP32 ? h.exp_dq : nullptr;
        r.exp_shift = p.precision == CVG_PREC_FP32 ? reinterpret_cast<int *>(h.exp_dq + 1) : nullptr;
        r.dim = D;
        r.adapt = (p.flags & CVG_FLAG_NO_ADAPT) ? 0 : 1;
        r.lb = h.lb;            // one-pass allocation; the words start at zero (arena)
        r.lb_ctl = h.lb_ctl;
        cvg_refine_args &q = hq[i];
        q.x_edges = h.x_edges;
        q.x_edges32 = h.x_edges32;
        q.weights = h.weights;
        q.counts = h.counts;
        q.bin_exp = a.bin_exp;
        q.alpha = p.alpha;
        q.dim = D;
        q.n_intervals = N;
        q.adapt = r.adapt;
        hdims[i] = D;
        blk_base[i + 1] = blk_base[i] + h.nb;
        dim_base[i + 1] = dim_base[i] + D;
    }
    if (b->total_blocks != blk_base[n]) return cvg_internal_fail(CVG_ERR_STATE, "batch block count mismatch");
    std::vector<unsigned> blk_inst(b->total_blocks);
    for (int i = 0; i < n; ++i)
        for (unsigned k = blk_base[i]; k < blk_base[i + 1]; ++k) blk_inst[k] = (unsigned)i;
    b->total_dims = dim_base[n];
    BCK(cudaMemcpyAsync(b->d_fill, hf.data(), sizeof(cvg_fill_args) * n, cudaMemcpyHostToDevice, st));
    BCK(cudaMemcpyAsync(b->d_realloc, hr.data(), sizeof(cvg_realloc_args) * n, cudaMemcpyHostToDevice, st));
    BCK(cudaMemcpyAsync(b->d_refine, hq.data(), sizeof(cvg_refine_args) * n, cudaMemcpyHostToDevice, st));
    BCK(cudaMemcpyAsync(b->d_dims, hdims.data(), sizeof(int) * n, cudaMemcpyHostToDevice, st));
    BCK(cudaMemcpyAsync(b->d_blk_base, blk_base.data(), sizeof(unsigned) * (n + 1), cudaMemcpyHostToDevice, st));
    BCK(cudaMemcpyAsync(b->d_blk_inst, blk_inst.data(), sizeof(unsigned) * b->total_blocks,
                        cudaMemcpyHostToDevice, st));
    BCK(cudaMemcpyAsync(b->d_dim_base, dim_base.data(), sizeof(unsigned) * (n + 1), cudaMemcpyHostToDevice, st));
    // kernels
    cudaLibrary_t lib = nullptr;
    BCKS(cvg_internal_load_module(ctx, batch_source(*b, dims), &lib));
    BCK(cudaLibraryGetKernel(&b->fill, lib, "cvg_fill_batch_entry"));
    BCK(cudaLibraryGetKernel(&b->pilot, lib, "cvg_pilot_batch_entry"));
    BCK(cudaFuncSetAttribute((const void *)b->fill, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             (int)b->fill_smem));
    int occ = 0;
    BCK(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, (const void *)b->fill, b->block, b->fill_smem));
    if (occ < 1) return cvg_internal_fail(CVG_ERR_INVALID, "batched fill kernel cannot be resident");
    b->grid = std::min(occ * ctx->n_sm, b->max_ranges);
    // initial counts -> prefixes, tile maps, tile numbering and the fill's ranges
    BCK(cvg_launch_set_nh_batch(realloc_batch(b), batch_sched(b), st));
    BCK(cudaEventCreate(&b->ev0));
    BCK(cudaEventCreate(&b->ev1));
    BCK(cudaEventCreateWithFlags(&b->ev_fork, cudaEventDisableTiming));
    BCK(cudaEventCreateWithFlags(&b->ev_join, cudaEventDisableTiming));
    // FP32 form: per-instance scale exponent from a pilot evaluation
    if (p.precision == CVG_PREC_FP32) {
        std::vector<int> ex(n, -1000);
        std::vector<double> ss(n, 0.0);
        for (int i = 0; i < n; ++i) {
            BCK(cudaMemcpyAsync(b->inst[i].scale_exp, &ex[i], sizeof(int), cudaMemcpyHostToDevice, st));
            BCK(cudaMemsetAsync(b->inst[i].scale_ss, 0, sizeof(double), st));
        }
        cvg_batch_args ba = batch_args(b);
        void *args[] = {&ba};
        BCK(cudaLaunchKernel((const void *)b->pilot, dim3(32 * n), dim3(256), args, 0, st));
        // the pilot's bin histograms -> first per-bin exponent tables (grids kept)
        cvg_refine_batch rb = refine_batch(b);
        rb.keep_grid = 1;
        BCK(cvg_launch_refine_batch(rb, N, st));
        for (int i = 0; i < n; ++i) {
            BCK(cudaMemcpyAsync(&ex[i], b->inst[i].scale_exp, sizeof(int), cudaMemcpyDeviceToHost, st));
            BCK(cudaMemcpyAsync(&ss[i], b->inst[i].scale_ss, sizeof(double), cudaMemcpyDeviceToHost, st));
        }
        BCK(cudaStreamSynchronize(st));
        for (int i = 0; i < n; ++i) {
            ex[i] = cvg_internal_pilot_scale(ex[i], ss[i], 32.0 * 256.0);
            BCK(cudaMemcpyAsync(b->inst[i].scale_exp, &ex[i], sizeof(int), cudaMemcpyHostToDevice, st));
        }
    }
    BCK(cudaStreamSynchronize(st));
    return CVG_OK;
}

}  // namespace

extern "C" {

cvg_status cvg_batch_destroy(cvg_batch b)
{
    if (!b) return CVG_OK;
    cudaSetDevice(b->ctx->device);
    cudaStreamSynchronize(b->ctx->stream);
    if (b->graph_exec) cudaGraphExecDestroy(b->graph_exec);
    if (b->graph) cudaGraphDestroy(b->graph);
    if (b->ev0) cudaEventDestroy(b->ev0);
    if (b->ev1) cudaEventDestroy(b->ev1);
    if (b->ev_fork) cudaEventDestroy(b->ev_fork);
    if (b->ev_join) cudaEventDestroy(b->ev_join);
    if (b->arena) cvg_internal_arena_free(b->ctx, b->arena, b->arena_bytes);
    delete b;
    return CVG_OK;
}

cvg_status cvg_batch_iterate(cvg_batch b, int32_t n_it)
{
    if (!b) return cvg_internal_fail(CVG_ERR_INVALID, "NULL batch");
    if (n_it < 0 || b->it_done + n_it > b->p.max_it)
        return cvg_internal_fail(CVG_ERR_STATE, "iterations beyond max_it");
    BCK(cudaSetDevice(b->ctx->device));
    if (b->p.flags & CVG_FLAG_GRAPH) {
        if (!b->graph_exec) {
            cudaStream_t s = b->ctx->stream;
            BCK(cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal));
            cvg_status st = enqueue_iteration(b, false);
            cudaGraph_t g = nullptr;
            cudaError_t e = cudaStreamEndCapture(s, &g);
            if (st != CVG_OK) { if (g) cudaGraphDestroy(g); return st; }
            BCK(e);
            b->graph = g;
            BCK(cudaGraphInstantiate(&b->graph_exec, g, 0));
        }
        for (int i = 0; i < n_it; ++i) BCK(cudaGraphLaunch(b->graph_exec, b->ctx->stream));
    } else {
        for (int i = 0; i < n_it; ++i) BCKS(enqueue_iteration(b, i == n_it - 1));
    }
    b->it_done += n_it;
    return CVG_OK;
}

cvg_status cvg_batch_results(cvg_batch b, cvg_result *out, double *it_res, double *it_sig2)
{
    if (!b || !out) return cvg_internal_fail(CVG_ERR_INVALID, "NULL argument");
    BCK(cudaSetDevice(b->ctx->device));
    const int M = b->p.max_it;
    std::vector<double> stats((size_t)3 * M * b->n);
    std::vector<cvg_acc_dev> acc(b->n);
    cvg_u32 status = 0;
    cudaStream_t st = b->ctx->stream;
    for (int i = 0; i < b->n; ++i) {
        BCK(cudaMemcpyAsync(stats.data() + (size_t)3 * M * i, b->inst[i].stats, sizeof(double) * 3 * M,
                            cudaMemcpyDeviceToHost, st));
        BCK(cudaMemcpyAsync(&acc[i], b->inst[i].acc, sizeof(cvg_acc_dev), cudaMemcpyDeviceToHost, st));
    }
    BCK(cudaMemcpyAsync(&status, b->d_status, sizeof(status), cudaMemcpyDeviceToHost, st));
    BCK(cudaStreamSynchronize(st));
    if (status & CVG_KSTAT_TIMEOUT)
        return cvg_internal_fail(CVG_ERR_KERNEL, "batched reallocation: a look-back wait ran out");
    if (status & CVG_KSTAT_BAD_TILE)
        return cvg_internal_fail(CVG_ERR_KERNEL, "batched fill found an inconsistent tile map");
    const int done = std::min(b->it_done, M);
    for (int i = 0; i < b->n; ++i) {
        cvg_result &r = out[i];
        std::memset(&r, 0, sizeof(r));
        const double *s = stats.data() + (size_t)3 * M * i;
        cvg_internal_result(s, M, done, b->p.skip, &r);
        r.n_strat = b->inst[i].n_strat;
        r.n_intervals = b->p.n_intervals;
        r.n_cubes = b->inst[i].n_cubes;
        r.tot_nevals = (int64_t)acc[i].tot_nevals;
        r.seed = b->p.seed;
        r.gpu_thr = b->p.gpu_thr;
        r.precision = b->p.precision;
        if (it_res) for (int k = 0; k < M; ++k) it_res[(size_t)i * M + k] = s[k];
        if (it_sig2) for (int k = 0; k < M; ++k) it_sig2[(size_t)i * M + k] = s[M + k];
    }
    return CVG_OK;
}

cvg_status cvg_batch_info_get(cvg_batch b, int32_t *block, int32_t *spt, int32_t *grid,
                              int64_t *fill_smem_bytes, int64_t *next_samples)
{
    if (!b) return cvg_internal_fail(CVG_ERR_INVALID, "NULL batch");
    if (block) *block = b->block;
    if (spt) *spt = b->spt;
    if (grid) *grid = b->grid;
    if (fill_smem_bytes) *fill_smem_bytes = (int64_t)b->fill_smem;
    if (next_samples) {
        BCK(cudaSetDevice(b->ctx->device));
        int64_t tot = 0;
        for (int i = 0; i < b->n; ++i) {
            cvg_u64 S = 0;
            BCK(cudaMemcpyAsync(&S, b->inst[i].nh_sum + b->inst[i].n_cubes, sizeof(S),
                                cudaMemcpyDeviceToHost, b->ctx->stream));
            BCK(cudaStreamSynchronize(b->ctx->stream));
            tot += (int64_t)S;
        }
        *next_samples = tot;
    }
    return CVG_OK;
}

cvg_status cvg_batch_compile_check(const char *source, int32_t n_dims, const int32_t *dims,
                                   const int32_t *params_per_dim, int32_t precision,
                                   int32_t block, const char *arch, char *log, size_t log_len)
{
    if (!source || !dims || !params_per_dim || !arch || n_dims < 1)
        return cvg_internal_fail(CVG_ERR_INVALID, "NULL argument");
    cvg_batch_s b;
    b.f.source = source;
    b.f.abi = CVG_ABI_NATIVE;
    b.p.precision = precision;
    b.block = block > 0 ? block : 512;
    b.params_per_dim.assign(params_per_dim, params_per_dim + 17);
    std::set<int> ds;
    for (int i = 0; i < n_dims; ++i) {
        if (dims[i] < 1 || dims[i] > 16) return cvg_internal_fail(CVG_ERR_INVALID, "dims in [1, 16]");
        ds.insert(dims[i]);
    }
    std::string l;
    const cvg_status st = cvg_internal_compile_only(batch_source(b, ds), arch, l);
    if (log && log_len) {
        std::strncpy(log, l.c_str(), log_len - 1);
        log[log_len - 1] = '\0';
    }
    return st;
}

cvg_status cvg_batch_last_fill_ms(cvg_batch b, float *ms)
{
    if (!b || !ms) return cvg_internal_fail(CVG_ERR_INVALID, "NULL argument");
    BCK(cudaEventSynchronize(b->ev1));
    BCK(cudaEventElapsedTime(ms, b->ev0, b->ev1));
    return CVG_OK;
}

}  // extern "C"
