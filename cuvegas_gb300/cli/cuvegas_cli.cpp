// cuvegas -- command-line driver with the reference's config.cuh plug-in
// contract (src/config.cuh:7-33, src/main.cu:6, 278-797 of the reference).
//
//   cuvegas [options] config.cuh [source.cu ...]
//
// The reference compiles src/main.cu with config.cuh #included and links the
// device sources its Makefile names (commons/functions.cu, Makefile:21-27);
// the integrand is inlined into its fill kernel.  Here the same files are
// read at run time: #include "..." lines are expanded (relative to the
// including file, then -I directories), system #include <...> lines are
// dropped (NVRTC supplies the device math functions; the M_* constants come
// from a prelude), and the result is JIT-compiled by libcuvegas as the
// integrand's translation unit.  The config's globals (tot_eval, max_it,
// skip, max_batch_size, n_intervals, alpha, beta, n_dim) are read from its
// text; blockSize* constants are accepted and ignored (the kernels choose
// their own shapes).  The run goes through the C ABI (cvg_integrate), and the
// output repeats the reference's lines (src/main.cu:292, 428-430, 791-797)
// plus the chi^2/dof of the iteration estimates.
//
// Options:
//   -I DIR              search DIR for #include "..." (repeatable)
//   --precision P       fp64 (default, the reference's arithmetic) or fp32
//   --seed N            Philox key (default 123, the reference's curand seed)
//   --device N          CUDA device (default 0)
//   --no-graph          iterate eagerly instead of replaying a CUDA graph
//   --check             parse and compile only (no GPU needed); prints the
//                       configuration that would run
//   --dump-source       print the expanded integrand source and exit
#include "cuvegas.h"

#include <cctype>
#include <chrono>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <map>
#include <set>
#include <sstream>
#include <string>
#include <vector>

namespace {

const char *kPrelude =
    "// cuvegas CLI prelude: constants of <math.h> (_USE_MATH_DEFINES)\n"
    "#ifndef M_PI\n"
    "#define M_E 2.71828182845904523536\n"
    "#define M_LOG2E 1.44269504088896340736\n"
    "#define M_LOG10E 0.434294481903251827651\n"
    "#define M_LN2 0.693147180559945309417\n"
    "#define M_LN10 2.30258509299404568402\n"
    "#define M_PI 3.14159265358979323846\n"
    "#define M_PI_2 1.57079632679489661923\n"
    "#define M_PI_4 0.785398163397448309616\n"
    "#define M_1_PI 0.318309886183790671538\n"
    "#define M_2_PI 0.636619772367581343076\n"
    "#define M_2_SQRTPI 1.12837916709551257390\n"
    "#define M_SQRT2 1.41421356237309504880\n"
    "#define M_SQRT1_2 0.707106781186547524401\n"
    "#endif\n";

double now_ms()
{
    using namespace std::chrono;
    return duration<double, std::milli>(steady_clock::now().time_since_epoch()).count();
}

bool read_file(const std::string &path, std::string &out)
{
    std::ifstream f(path, std::ios::binary);
    if (!f) return false;
    std::ostringstream ss;
    ss << f.rdbuf();
    out = ss.str();
    return true;
}

std::string dir_of(const std::string &path)
{
    const size_t p = path.find_last_of('/');
    return p == std::string::npos ? std::string(".") : path.substr(0, p);
}

bool exists(const std::string &path)
{
    std::ifstream f(path);
    return (bool)f;
}

std::string trim(const std::string &s)
{
    size_t a = 0, b = s.size();
    while (a < b && std::isspace((unsigned char)s[a])) ++a;
    while (b > a && std::isspace((unsigned char)s[b - 1])) --b;
    return s.substr(a, b - a);
}

// "#include" directive of a line: kind '"' or '<' and the name; 0 if none.
char include_of(const std::string &line, std::string &name)
{
    std::string t = trim(line);
    if (t.empty() || t[0] != '#') return 0;
    t = trim(t.substr(1));
    if (t.compare(0, 7, "include") != 0) return 0;
    t = trim(t.substr(7));
    if (t.size() < 2) return 0;
    const char open = t[0], close = open == '"' ? '"' : (open == '<' ? '>' : 0);
    if (!close) return 0;
    const size_t e = t.find(close, 1);
    if (e == std::string::npos) return 0;
    name = t.substr(1, e - 1);
    return open;
}

struct Expander {
    std::vector<std::string> incdirs;
    std::set<std::string> once;     // files with #pragma once already expanded
    std::string err;

    bool expand(const std::string &path, std::string &out, int depth)
    {
        if (depth > 32) { err = "#include nesting deeper than 32 at " + path; return false; }
        std::string text;
        if (!read_file(path, text)) { err = "cannot read " + path; return false; }
        if (once.count(path)) return true;
        if (text.find("#pragma once") != std::string::npos) once.insert(path);
        std::istringstream in(text);
        std::string line;
        int ln = 0;
        out += "#line 1 \"" + path + "\"\n";
        while (std::getline(in, line)) {
            ++ln;
            std::string name;
            const char k = include_of(line, name);
            if (k == '<') {          // system header: NVRTC has the device math built in
                out += "\n";
                continue;
            }
            if (k == '"') {
                std::string found;
                const std::string local = dir_of(path) + "/" + name;
                if (exists(local)) found = local;
                for (size_t i = 0; found.empty() && i < incdirs.size(); ++i)
                    if (exists(incdirs[i] + "/" + name)) found = incdirs[i] + "/" + name;
                if (found.empty()) { err = path + ":" + std::to_string(ln) + ": cannot find \"" + name + "\""; return false; }
                if (!expand(found, out, depth + 1)) return false;
                out += "#line " + std::to_string(ln + 1) + " \"" + path + "\"\n";
                continue;
            }
            out += line + "\n";
        }
        return true;
    }
};

// Globals of config.cuh: "[const] <type> name = value;" at the start of a line.
std::map<std::string, std::string> config_globals(const std::string &text)
{
    static const char *types[] = {"long long int", "long long", "long int", "unsigned long",
                                  "unsigned int", "unsigned", "long", "int", "double", "float",
                                  "size_t", "int64_t", "int32_t"};
    std::map<std::string, std::string> g;
    std::istringstream in(text);
    std::string line;
    while (std::getline(in, line)) {
        std::string t = trim(line);
        if (t.compare(0, 6, "const ") == 0) t = trim(t.substr(6));
        if (t.compare(0, 10, "constexpr ") == 0) t = trim(t.substr(10));
        bool typed = false;
        for (const char *ty : types) {
            const size_t n = std::strlen(ty);
            if (t.compare(0, n, ty) == 0 && t.size() > n && std::isspace((unsigned char)t[n])) {
                t = trim(t.substr(n));
                typed = true;
                break;
            }
        }
        if (!typed) continue;
        const size_t eq = t.find('='), sc = t.find(';');
        if (eq == std::string::npos || sc == std::string::npos || sc < eq) continue;
        const std::string name = trim(t.substr(0, eq));
        bool ident = !name.empty();
        for (char c : name) ident = ident && (std::isalnum((unsigned char)c) || c == '_');
        if (ident) g[name] = trim(t.substr(eq + 1, sc - eq - 1));
    }
    return g;
}

bool number(const std::string &s, double &v)
{
    std::string t = s;
    while (!t.empty() && (t.back() == 'L' || t.back() == 'l' || t.back() == 'U' || t.back() == 'u' ||
                          t.back() == 'f' || t.back() == 'F'))
        t.pop_back();
    if (t.empty()) return false;
    char *end = nullptr;
    v = std::strtod(t.c_str(), &end);
    return end && *end == '\0';
}

int usage()
{
    std::fprintf(stderr,
                 "usage: cuvegas [-I DIR] [--precision fp64|fp32] [--seed N] [--device N] "
                 "[--no-graph] [--check] [--dump-source] config.cuh [source.cu ...]\n");
    return 2;
}

}  // namespace

int main(int argc, char **argv)
{
    const double t_start = now_ms();
    Expander ex;
    std::vector<std::string> files;
    int precision = CVG_PREC_FP64, device = 0;
    unsigned long long seed = 123;
    bool graph = true, check = false, dump = false;
    for (int i = 1; i < argc; ++i) {
        const std::string a = argv[i];
        auto next = [&](const char *what) -> const char * {
            if (i + 1 >= argc) { std::fprintf(stderr, "%s needs a value\n", what); std::exit(2); }
            return argv[++i];
        };
        if (a == "-I") ex.incdirs.push_back(next("-I"));
        else if (a.compare(0, 2, "-I") == 0 && a.size() > 2) ex.incdirs.push_back(a.substr(2));
        else if (a == "--precision") {
            const std::string p = next("--precision");
            if (p == "fp64") precision = CVG_PREC_FP64;
            else if (p == "fp32") precision = CVG_PREC_FP32;
            else return usage();
        } else if (a == "--seed") seed = std::strtoull(next("--seed"), nullptr, 10);
        else if (a == "--device") device = std::atoi(next("--device"));
        else if (a == "--no-graph") graph = false;
        else if (a == "--check") check = true;
        else if (a == "--dump-source") dump = true;
        else if (a == "-h" || a == "--help") return usage();
        else if (!a.empty() && a[0] == '-') return usage();
        else files.push_back(a);
    }
    if (files.empty()) return usage();

    // configuration
    std::string cfg_text;
    if (!read_file(files[0], cfg_text)) { std::fprintf(stderr, "cannot read %s\n", files[0].c_str()); return 1; }
    const auto g = config_globals(cfg_text);
    auto get = [&](const char *name, double dflt, bool required, double &out) -> bool {
        auto it = g.find(name);
        if (it == g.end()) {
            if (required) { std::fprintf(stderr, "%s: no value for %s\n", files[0].c_str(), name); return false; }
            out = dflt;
            return true;
        }
        if (!number(it->second, out)) {
            std::fprintf(stderr, "%s: cannot evaluate %s = %s\n", files[0].c_str(), name, it->second.c_str());
            return false;
        }
        return true;
    };
    // defaults: the values of the reference's own config.cuh
    double tot_eval, max_it, skip, max_batch, n_intervals, alpha, beta, n_dim;
    if (!get("tot_eval", 1e7, false, tot_eval) || !get("max_it", 20, false, max_it) ||
        !get("skip", 5, false, skip) || !get("max_batch_size", 1048576, false, max_batch) ||
        !get("n_intervals", 1024, false, n_intervals) || !get("alpha", 0.5, false, alpha) ||
        !get("beta", 0.75, false, beta) || !get("n_dim", 0, true, n_dim))
        return 1;

    // integrand translation unit: prelude, config, the linked device sources
    std::string src = kPrelude;
    for (const std::string &f : files)
        if (!ex.expand(f, src, 0)) { std::fprintf(stderr, "%s\n", ex.err.c_str()); return 1; }
    if (dump) { std::fputs(src.c_str(), stdout); return 0; }

    cvg_params p{};
    p.tot_eval = (int64_t)tot_eval;
    p.max_it = (int32_t)max_it;
    p.skip = (int32_t)skip;
    p.max_batch_size = (int64_t)max_batch;
    p.n_intervals = (int32_t)n_intervals;
    p.n_dim = (int32_t)n_dim;
    p.precision = precision;
    p.alpha = alpha;
    p.beta = beta;
    p.seed = seed;
    p.gpu_thr = 0.1;
    p.flags = graph ? CVG_FLAG_GRAPH : 0;

    if (check) {
        char log[16384];
        const cvg_status st = cvg_compile_check(src.c_str(), p.n_dim, CVG_ABI_NATIVE, 0, 0, precision,
                                                "sm_103a", log, sizeof(log));
        std::printf("n_dim: %d\ntot_eval: %lld\nmax_it: %d\nskip: %d\nn_intervals: %d\n"
                    "alpha: %g\nbeta: %g\nprecision: %s\ncompile: %s\n",
                    p.n_dim, (long long)p.tot_eval, p.max_it, p.skip, p.n_intervals, p.alpha, p.beta,
                    precision == CVG_PREC_FP32 ? "fp32" : "fp64", st == CVG_OK ? "ok" : "failed");
        if (st != CVG_OK) std::fprintf(stderr, "%s\n%s\n", cvg_last_error(), log);
        return st == CVG_OK ? 0 : 1;
    }

    std::printf("GPUs: %d\n", 1);   // one GPU per process; replicas run as separate processes
    cvg_context ctx = nullptr;
    cvg_status st = cvg_context_create(device, nullptr, &ctx);
    if (st != CVG_OK) { std::fprintf(stderr, "cuvegas: %s\n", cvg_last_error()); return 1; }
    const double t_nocontext = now_ms();
    cvg_integrand f = nullptr;
    st = cvg_compile_integrand(ctx, src.c_str(), p.n_dim, CVG_ABI_NATIVE, 0, 0, &f);
    if (st != CVG_OK) {
        std::fprintf(stderr, "cuvegas: %s\n", cvg_last_error());
        cvg_context_destroy(ctx);
        return 1;
    }
    // the reference compiles its integrand ahead of time (inlined into
    // vegasFill at build time); here NVRTC compiles it now, and that time is
    // reported on its own line so "Nocontext" keeps the reference's meaning:
    // the run's own work after the device context exists
    const double t_compiled = now_ms();
    cvg_result res{};
    st = cvg_integrate(ctx, f, &p, nullptr, &res, nullptr, nullptr);
    if (st != CVG_OK) {
        std::fprintf(stderr, "cuvegas: %s\n", cvg_last_error());
        cvg_integrand_release(f);
        cvg_context_destroy(ctx);
        return 1;
    }
    const double t_end = now_ms();
    std::printf("Strat: %d\n", res.n_strat);
    std::printf("Cubes: %lld\n", (long long)res.n_cubes);
    std::printf("Intervals: %d\n", res.n_intervals);
    std::printf("Result: %.12f\n", res.result);
    std::printf("Error: %.12f\n", res.error);
    std::printf("Total evals: %lld\n", (long long)res.tot_nevals);
    std::printf("Time elapsed %f ms\n", t_end - t_start);
    std::printf("Iteration avg time %f ms\n", res.avg_it_time_ms);
    std::printf("Nocontext %f ms\n", t_end - t_compiled);
    std::printf("Context creation %f ms\n", t_nocontext - t_start);
    std::printf("Integrand compile %f ms\n", t_compiled - t_nocontext);
    std::printf("Chi2/dof: %f\n", res.chi2_dof);
    cvg_integrand_release(f);
    cvg_context_destroy(ctx);
    return 0;
}
