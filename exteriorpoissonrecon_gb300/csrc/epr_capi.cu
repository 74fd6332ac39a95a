// The C ABI of libepr_cuda (declared in include/epr.h): context management, host <-> device
// transfers and the solver drivers.  All arithmetic runs in the kernels of epr_solve.cu and
// epr_setup.cu; this file only sequences them on the context's stream.
#include <algorithm>
#include <atomic>
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <mutex>
#include <string>
#include <thread>
#include <type_traits>
#include <utility>
#include <vector>

#include "../../include/epr.h"
#include "epr_common.cuh"
#include "epr_context.h"
#include "epr_kernels.h"
#include "epr_mg.h"
#include "epr_poly.h"

namespace {

thread_local std::string g_error;

// host workers of epr_batch_solve when the caller does not choose: each drives one stream, and
// eight streams fill the device's default number of hardware work queues
// (CUDA_DEVICE_MAX_CONNECTIONS, 8 unless the process raises it before CUDA starts)
constexpr int kBatchThreads = 8;

std::mutex g_create_mutex;

}  // namespace

namespace epr {

void set_global_error(const std::string &msg) { g_error = msg; }

void Context::fail(int code, const char *fmt, ...)
{
    char buf[1024];
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(buf, sizeof(buf), fmt, ap);
    va_end(ap);
    err = buf;
    status = code;
}

bool Context::cuda_ok(cudaError_t e, const char *what)
{
    if (e == cudaSuccess) return true;
    fail(e == cudaErrorMemoryAllocation ? EPR_ERR_NOMEM : EPR_ERR_CUDA, "%s: %s", what, cudaGetErrorString(e));
    cudaGetLastError();
    return false;
}

bool Context::launch_ok(const char *what) { return cuda_ok(cudaGetLastError(), what); }

bool Context::alloc(void **p, size_t bytes, const char *what)
{
    *p = nullptr;
    if (bytes == 0) return true;
    if (alloc_cap && alloc_total + bytes > alloc_cap)
    {
        fail(EPR_ERR_NOMEM, "%s: %zu bytes exceed the allocation cap (%zu of %zu bytes allocated)", what, bytes, alloc_total,
             alloc_cap);
        return false;
    }
    alloc_total += bytes;
    return cuda_ok(cudaMallocAsync(p, bytes, stream), what);
}

void Context::release(void *p)
{
    if (p) cudaFreeAsync(p, stream);
}

int64_t Context::nodes(int level) const
{
    int64_t n = 1;
    for (int d = 0; d < dim; d++) n *= (int64_t)((1 << level) + 1);
    return n;
}
int Context::stencil() const { return dim == 3 ? 27 : 81; }

bool Context::ensure_level(int l)
{
    Level &L = levels[l];
    if (L.N) return true;
    L.N = nodes(l);
    size_t S = (size_t)stencil();
    if (!alloc((void **)&L.xy64, sizeof(double) * 2 * L.N, "alloc xy")) return false;
    if (!alloc((void **)&L.A64, sizeof(double) * S * L.N, "alloc A")) return false;
    if (!alloc((void **)&L.B64, sizeof(double) * S * L.N, "alloc B")) return false;
    if (!cuda_ok(cudaMemsetAsync(L.xy64, 0, sizeof(double) * 2 * L.N, stream), "memset xy")) return false;
    if (!cuda_ok(cudaMemsetAsync(L.A64, 0, sizeof(double) * S * L.N, stream), "memset A")) return false;
    if (!cuda_ok(cudaMemsetAsync(L.B64, 0, sizeof(double) * S * L.N, stream), "memset B")) return false;
    if (P.precision == EPR_FP32)
    {
        if (!alloc((void **)&L.xy32, sizeof(float) * 2 * L.N, "alloc xy32")) return false;
        if (!alloc((void **)&L.A32, sizeof(float) * S * L.N, "alloc A32")) return false;
        if (!alloc((void **)&L.B32, sizeof(float) * S * L.N, "alloc B32")) return false;
        if (!cuda_ok(cudaMemsetAsync(L.xy32, 0, sizeof(float) * 2 * L.N, stream), "memset xy32")) return false;
    }
    if (lvlDF(l))
    {
        if (!alloc((void **)&L.xyd, sizeof(df) * 2 * L.N, "alloc xy df")) return false;
        if (!alloc((void **)&L.Ad, sizeof(df) * S * L.N, "alloc A df")) return false;
        if (!alloc((void **)&L.Bd, sizeof(df) * S * L.N, "alloc B df")) return false;
        if (!cuda_ok(cudaMemsetAsync(L.xyd, 0, sizeof(df) * 2 * L.N, stream), "memset xy df")) return false;
    }
    return true;
}

bool Context::lvl32(int l) const { return P.precision == EPR_FP32 && !(l >= P.fp64_from && l < P.fp64_levels); }

// the coarsest 3D levels of a float solve's band, in double-float when asked (their kernels are the
// point-split and single-block ones, which take the pair type)
constexpr int kMaxDFLevel = 3;
bool Context::lvlDF(int l) const
{
    return P.precision == EPR_FP32 && P.band_precision == EPR_BAND_DF && P.solver == EPR_SOLVER_CASCADIC && dim == 3 &&
           l <= kMaxDFLevel && l >= P.fp64_from && l < P.fp64_levels;
}

// refreshes the derived copies of a level's system: the float stencils (float levels) and the
// colour-blocked stencils of the levels that are relaxed by one kernel per colour
bool Context::sync_system32(int l)
{
    Level &L = levels[l];
    size_t S = (size_t)stencil();
    if (lvl32(l))
    {
        launch_convert_d2f(L.A64, L.A32, (int64_t)S * L.N, stream);
        launch_convert_d2f(L.B64, L.B32, (int64_t)S * L.N, stream);
    }
    if (lvlDF(l))
    {
        // the point-split kernels of these levels read the stencils in natural order
        launch_d2df(L.A64, L.Ad, (int64_t)S * L.N, stream);
        launch_d2df(L.B64, L.Bd, (int64_t)S * L.N, stream);
        return launch_ok("convert system");
    }
    if (L.N > (dim == 3 ? 27 : 81))
    {
        const size_t bytes = S * L.N * (lvl32(l) ? sizeof(float) : sizeof(double));
        if (!L.Acb && (!alloc(&L.Acb, bytes, "alloc colour blocks") || !alloc(&L.Bcb, bytes, "alloc colour blocks"))) return false;
        auto blocks = [&](auto dd) {
            constexpr int D = decltype(dd)::value;
            if (lvl32(l))
            {
                launch_to_colour_blocks<D, float>(l, L.A64, (float *)L.Acb, stream);
                launch_to_colour_blocks<D, float>(l, L.B64, (float *)L.Bcb, stream);
            }
            else
            {
                launch_to_colour_blocks<D, double>(l, L.A64, (double *)L.Acb, stream);
                launch_to_colour_blocks<D, double>(l, L.B64, (double *)L.Bcb, stream);
            }
        };
        if (dim == 3) blocks(std::integral_constant<int, 3>{});
        else blocks(std::integral_constant<int, 4>{});
    }
    return launch_ok("convert system");
}

// device coefficients <-> the precision the solve works in
bool Context::push_xy(int l)
{
    if (lvlDF(l))
    {
        launch_df_push(levels[l].xy64, levels[l].xyd, 2 * levels[l].N, d_kexp, l, stream);
        return launch_ok("convert xy");
    }
    if (!lvl32(l)) return true;
    launch_convert_d2f(levels[l].xy64, levels[l].xy32, 2 * levels[l].N, stream);
    return launch_ok("convert xy");
}
bool Context::pull_xy(int l)
{
    if (lvlDF(l))
    {
        launch_df_pull(levels[l].xyd, levels[l].xy64, 2 * levels[l].N, d_kexp, l, stream);
        return launch_ok("convert xy");
    }
    if (!lvl32(l)) return true;
    launch_convert_f2d(levels[l].xy32, levels[l].xy64, 2 * levels[l].N, stream);
    return launch_ok("convert xy");
}

Context::~Context()
{
    if (stream)
    {
        for (Level &L : levels)
        {
            release(L.xy64); release(L.xy32); release(L.A64); release(L.B64); release(L.A32); release(L.B32);
            release(L.tmp64); release(L.tmp32); release(L.Acb); release(L.Bcb);
            release(L.xyd); release(L.Ad); release(L.Bd);
        }
        release(red.partial); release(red.out); release(d_err); release(d_fit); release(d_kexp);
        setup.release(*this);
        release_adaptive();
        release_mg(*this);
        if (solve_graph) cudaGraphExecDestroy(solve_graph);
        cudaStreamSynchronize(stream);
        cudaStreamDestroy(stream);
    }
    if (ev0) cudaEventDestroy(ev0);
    if (ev1) cudaEventDestroy(ev1);
}

// ---------------------------------------------------------------------------------------------
// typed dispatch helpers
// ---------------------------------------------------------------------------------------------
template <typename F>
int with_dim(Context *c, F &&f)
{
    if (c->dim == 3) return f(std::integral_constant<int, 3>{});
    return f(std::integral_constant<int, 4>{});
}


// Energies are evaluated in double at every level, whatever arithmetic the level relaxes in: a
// float or double-float level's working copy is first converted into its double coefficients,
// and the element integrals, stencil forms and sums run on the double stencils, which every level
// keeps resident.  (The float energy kernel remains for epr_energy_noalloc's float mode and the kernel timer.)
bool Context::energy(int l, double *out3)
{
    if (lvl32(l) || lvlDF(l))
    {
        if (!pull_xy(l)) return false;
        launches++;
    }
    with_dim(this, [&](auto dd) {
        constexpr int D = decltype(dd)::value;
        launch_energy<D, double>(level_ptrs<double>(this, l), levels[l].xy64, red, stream);
        return 0;
    });
    launches += 2;
    if (!launch_ok("energy")) return false;
    double h[3];
    if (!cuda_ok(cudaMemcpyAsync(h, red.out, sizeof(h), cudaMemcpyDeviceToHost, stream), "energy copy")) return false;
    if (!cuda_ok(cudaStreamSynchronize(stream), "energy sync")) return false;
    out3[0] = h[0] - 2. * h[1] + c;
    out3[1] = h[2];
    out3[2] = h[0];
    return true;
}

bool Context::gs(int l, int iters, int64_t persistentMaxNodes)
{
    bool fp32 = lvl32(l);
    if (lvlDF(l))
    {
        launches += launch_gs_sweeps_df(level_ptrs<df>(this, l), iters, d_err, stream, P.separate, persistentMaxNodes, d_kexp);
        stats.node_updates += (int64_t)iters * levels[l].N;
        return launch_ok("gs");
    }
    launches += with_dim(this, [&](auto dd) {
        constexpr int D = decltype(dd)::value;
        if (fp32) return launch_gs_sweeps<D, float>(level_ptrs<float>(this, l), iters, d_err, stream, P.separate, persistentMaxNodes);
        return launch_gs_sweeps<D, double>(level_ptrs<double>(this, l), iters, d_err, stream, P.separate, persistentMaxNodes);
    });
    stats.node_updates += (int64_t)iters * levels[l].N;
    return launch_ok("gs");
}

bool Context::check_errors()
{
    unsigned int h = 0;
    if (!cuda_ok(cudaMemcpyAsync(&h, d_err, sizeof(h), cudaMemcpyDeviceToHost, stream), "error flag")) return false;
    if (!cuda_ok(cudaStreamSynchronize(stream), "sync")) return false;
    if (h & ERR_NONFINITE) { fail(EPR_ERR_NUMERIC, "a Gauss-Seidel update produced a non-finite value"); return false; }
    return true;
}

bool Context::prolong_add(int l)
{
    const bool c32 = lvl32(l), f32 = lvl32(l + 1), cdf = lvlDF(l), fdf = lvlDF(l + 1);
    bool ok = true;
    with_dim(this, [&](auto dd) {
        constexpr int D = decltype(dd)::value;
        if (c32 && f32)
        {
            launch_prolong<D, float>(l, levels[l].xy32, levels[l + 1].xy32, 1, stream, status_of(l + 1));
            return 0;
        }
        // otherwise in double: refresh the double copies of a float or double-float coarse level
        // and fine level, prolong, and refresh the fine level's working copy
        if (c32) { launch_convert_f2d(levels[l].xy32, levels[l].xy64, 2 * levels[l].N, stream); launches++; }
        if (cdf) { ok = ok && pull_xy(l); launches++; }
        if (f32) { launch_convert_f2d(levels[l + 1].xy32, levels[l + 1].xy64, 2 * levels[l + 1].N, stream); launches++; }
        if (fdf) { ok = ok && pull_xy(l + 1); launches++; }
        launch_prolong<D, double>(l, levels[l].xy64, levels[l + 1].xy64, 1, stream, status_of(l + 1));
        if (f32) { launch_convert_d2f(levels[l + 1].xy64, levels[l + 1].xy32, 2 * levels[l + 1].N, stream); launches++; }
        if (fdf) { ok = ok && push_xy(l + 1); launches++; }
        return 0;
    });
    launches++;
    return ok && launch_ok("prolong");
}

// Random<double> (Misha/Geometry.inl:430-438) on the C library generator seeded by srand(seed).
// glibc's rand() is random() on a 128-byte additive-feedback state; random_r runs the same
// generator on a state of the context's own, so the sequence is the one srand(seed) + rand() give,
// and reconstructions solved concurrently on several host threads neither share nor disturb the
// process's rand() state.
class CRandom
{
  public:
    explicit CRandom(unsigned int seed)
    {
        std::memset(&data_, 0, sizeof(data_));
        initstate_r(seed, state_, sizeof(state_), &data_);
    }
    double next_double()
    {
        const unsigned long long ULL_RAND_MAX = (unsigned long long)(RAND_MAX) + 1;
        const double RAND_MAX_SQUARED = double(ULL_RAND_MAX * ULL_RAND_MAX - 1);
        unsigned long long r1 = next(), r2 = next();
        long long v = (long long)(r1 * ULL_RAND_MAX + r2);
        return double(v) / RAND_MAX_SQUARED;
    }

  private:
    unsigned long long next()
    {
        int32_t r = 0;
        random_r(&data_, &r);
        return (unsigned long long)r;
    }
    alignas(8) char state_[128];
    random_data data_;
};

bool Context::random_start(int level, double *energy_out)
{
    CRandom rng((unsigned int)P.seed);
    const int64_t N = levels[level].N;
    std::vector<double> x(N, 0.), y(N, 0.);
    if (adapt.empty())
        for (int64_t i = 0; i < N; i++) { x[i] = rng.next_double(); y[i] = rng.next_double(); }
    else
    {
        // the adaptive indexer's functions in its index order; the grid's other nodes hold none
        const AdaptiveLevel &A = adapt[level];
        std::vector<int64_t> order(A.nF);
        if (A.nF && (!cuda_ok(cudaMemcpyAsync(order.data(), A.fnodes, sizeof(int64_t) * A.nF, cudaMemcpyDeviceToHost, stream), "copy") ||
                     !cuda_ok(cudaStreamSynchronize(stream), "sync")))
            return false;
        for (int64_t f = 0; f < A.nF; f++) { x[order[f]] = rng.next_double(); y[order[f]] = rng.next_double(); }
    }
    if (!upload_xy(level, x.data(), y.data())) return false;
    double e[3];
    if (!energy(level, e)) return false;
    const double s = std::sqrt(std::sqrt(c / e[2]));
    for (int64_t i = 0; i < N; i++) { x[i] *= s; y[i] *= s; }
    if (!upload_xy(level, x.data(), y.data())) return false;
    if (energy_out)
    {
        if (!energy(level, e)) return false;
        *energy_out = e[0] + e[1];
    }
    return true;
}

// host planar arrays <-> device pairs: the two arrays travel as they are and the (de)interleaving
// runs on the device
bool Context::upload_xy(int l, const double *x, const double *y)
{
    const int64_t N = levels[l].N;
    double *planar = nullptr;
    if (!alloc((void **)&planar, sizeof(double) * 2 * N, "alloc planar")) return false;
    bool ok = cuda_ok(cudaMemcpyAsync(planar, x, sizeof(double) * N, cudaMemcpyHostToDevice, stream), "upload x") &&
              cuda_ok(cudaMemcpyAsync(planar + N, y, sizeof(double) * N, cudaMemcpyHostToDevice, stream), "upload y");
    if (ok)
    {
        launch_merge_pairs(planar, planar + N, levels[l].xy64, N, stream);
        ok = launch_ok("merge pairs") && push_xy(l);
    }
    release(planar);
    return ok && cuda_ok(cudaStreamSynchronize(stream), "upload sync");
}

bool Context::download_xy(int l, double *x, double *y, bool fromSolution)
{
    const int64_t N = levels[l].N;
    double *src = fromSolution ? levels[l].tmp64 : levels[l].xy64;
    if (!fromSolution && !pull_xy(l)) return false;
    double *planar = nullptr;
    if (!alloc((void **)&planar, sizeof(double) * 2 * N, "alloc planar")) return false;
    launch_split_pairs(src, planar, planar + N, N, stream);
    bool ok = launch_ok("split pairs") &&
              cuda_ok(cudaMemcpyAsync(x, planar, sizeof(double) * N, cudaMemcpyDeviceToHost, stream), "download x") &&
              cuda_ok(cudaMemcpyAsync(y, planar + N, sizeof(double) * N, cudaMemcpyDeviceToHost, stream), "download y");
    release(planar);
    return ok && cuda_ok(cudaStreamSynchronize(stream), "download sync");
}

// The relaxation sequence of the cascadic schedule (GS on every solve level, prolongation to the
// next), captured once into a CUDA graph and replayed: it is a fixed sequence of ~2,500 launches
// with no host interaction.  In the graph only the two coarsest levels run their sweeps inside one
// block; the others launch one kernel per colour, which the graph issues back to back.
bool Context::relax_levels(int minD, int maxD, bool useGraph)
{
    const int64_t graphPersistentMax = dim == 3 ? 27 : 81;
    if (useGraph && solve_graph)
    {
        launches += graph_launches;
        stats.node_updates += graph_updates;
        return cuda_ok(cudaGraphLaunch(solve_graph, stream), "graph launch");
    }
    // the first solve of a context launches directly (a one-off solve would not repay the graph's
    // instantiation); the second one captures, with the same launch configuration, so every solve
    // computes the same sequence of kernels
    const bool capture = useGraph && solves_done > 0;
    const int64_t l0 = launches, u0 = stats.node_updates;
    cudaGraph_t graph = nullptr;
    if (capture && !cuda_ok(cudaStreamBeginCapture(stream, cudaStreamCaptureModeThreadLocal), "begin capture")) return false;
    bool ok = true;
    for (int l = minD; ok && l <= maxD; l++)
    {
        int iters = (int)std::ceil(std::pow(P.i_mult, depth - l) * P.gs_iters);
        // the same launch configuration whether captured or not (one kernel per colour from level 2
        // on), so that every solve of a context runs the same kernels and gives the same bits
        ok = gs(l, iters, useGraph ? graphPersistentMax : kPersistentMaxNodes);
        if (ok && l < maxD) ok = prolong_add(l);
    }
    if (!capture) return ok;
    cudaError_t e = cudaStreamEndCapture(stream, &graph);
    if (!ok || !cuda_ok(e, "end capture")) { if (graph) cudaGraphDestroy(graph); return false; }
    e = cudaGraphInstantiate(&solve_graph, graph, 0);
    cudaGraphDestroy(graph);
    if (!cuda_ok(e, "graph instantiate")) { solve_graph = nullptr; return false; }
    graph_launches = launches - l0;
    graph_updates = stats.node_updates - u0;
    return cuda_ok(cudaGraphLaunch(solve_graph, stream), "graph launch");
}

// The reference's cascadic schedule (ExteriorPoisson.h:315-409).  Each level is relaxed by paired
// Gauss-Seidel (EPR_SOLVER_CASCADIC, the reference) or by alternating-solve rounds with linear
// multigrid V-cycles until the gradient falls by `tolerance` (EPR_SOLVER_MULTIGRID).
// the solve's first part: every level cleared (but a warm start's level) and the reference's random
// start on the coarsest solve level
bool Context::solve_prologue()
{
    const int minD = std::min(P.min_solve_depth, depth);
    const bool fp32 = P.precision == EPR_FP32;
    for (int l = 0; l <= depth; l++)
    {
        if (P.warm_start && l == minD) continue;  // the given start
        if (!cuda_ok(cudaMemsetAsync(levels[l].xy64, 0, sizeof(double) * 2 * levels[l].N, stream), "clear")) return false;
        if (fp32 && !cuda_ok(cudaMemsetAsync(levels[l].xy32, 0, sizeof(float) * 2 * levels[l].N, stream), "clear")) return false;
        if (levels[l].xyd && !cuda_ok(cudaMemsetAsync(levels[l].xyd, 0, sizeof(df) * 2 * levels[l].N, stream), "clear")) return false;
    }
    if (!P.warm_start && !cuda_ok(cudaMemsetAsync(d_kexp, 0, sizeof(int) * (depth + 1), stream), "clear")) return false;
    // random initial guess at the coarsest solve level, scaled to the target's magnitude
    return P.warm_start || random_start(minD, nullptr);
}

bool Context::solve_cascadic()
{
    const int minD = std::min(P.min_solve_depth, depth);
    const int maxD = P.max_solve_depth < 0 ? depth : std::min(P.max_solve_depth, depth);
    cudaEventRecord(ev0, stream);
    if (!solve_prologue()) return false;
    if (P.single_level)
    {
        // prolong the initial guess to the finest solve level, clear the coarser levels and relax
        // only there with gsIters sweeps (ExteriorPoisson.h:342-360)
        for (int l = minD; l < maxD; l++)
        {
            with_dim(this, [&](auto dd) {
                constexpr int D = decltype(dd)::value;
                launch_prolong<D, double>(l, levels[l].xy64, levels[l + 1].xy64, 0, stream, status_of(l + 1));
                return 0;
            });
            launches++;
        }
        for (int l = minD; l < maxD; l++)
            if (!cuda_ok(cudaMemsetAsync(levels[l].xy64, 0, sizeof(double) * 2 * levels[l].N, stream), "clear")) return false;
        if (!push_xy(maxD)) return false;
        double e0[3] = {0, 0, 0};
        if (P.verbose && !energy(maxD, e0)) return false;
        if (P.solver == EPR_SOLVER_MULTIGRID ? !relax_alternating(*this, maxD, true) : !gs(maxD, P.gs_iters)) return false;
        if (P.verbose)
        {
            double e1[3];
            if (!energy(maxD, e1)) return false;
            printf("Error[%2d]: %9.5f -> %.5f = %.5f + %.5f\n", 1 << maxD, e0[0] + e0[1], e1[0] + e1[1], e1[0], e1[1]);
        }
    }
    const bool useGraph = !P.single_level && !P.verbose && P.solver == EPR_SOLVER_CASCADIC;
    if (useGraph && !relax_levels(minD, maxD, true)) return false;
    for (int l = minD; !P.single_level && !useGraph && l <= maxD; l++)
    {
        int iters = (int)std::ceil(std::pow(P.i_mult, depth - l) * P.gs_iters);
        double e0[3] = {0, 0, 0};
        if (P.verbose && !energy(l, e0)) return false;
        if (P.solver == EPR_SOLVER_MULTIGRID ? !relax_alternating(*this, l, l == maxD) : !gs(l, iters)) return false;
        if (P.verbose)
        {
            double e1[3];
            if (!energy(l, e1)) return false;
            printf("Error[%2d]: %9.5f -> %.5f = %.5f + %.5f\n", 1 << l, e0[0] + e0[1], e1[0] + e1[1], e1[0], e1[1]);
        }
        if (l < maxD && !prolong_add(l)) return false;
    }
    stats.extra_sweeps = 0;
    stats.reached_target = 0;
    if (P.target_energy > 0)
    {
        // time to a target energy: the finest solve level relaxes on, one sweep at a time, until its
        // FP64 energy reaches the target (the checks belong to the timed solve)
        double e[3];
        for (;;)
        {
            if (!energy(maxD, e)) return false;
            if (e[0] + e[1] <= P.target_energy || stats.extra_sweeps >= P.max_extra_sweeps) break;
            if (!gs(maxD, 1)) return false;
            stats.extra_sweeps++;
        }
        stats.reached_target = e[0] + e[1] <= P.target_energy ? 1 : 0;
    }
    cudaEventRecord(ev1, stream);
    return solve_epilogue();
}

// the solve's last part, after ev1 was recorded behind the relaxation: the error flag, the timing,
// the final energy and the solution arrays every level exports
bool Context::solve_epilogue()
{
    const int maxD = P.max_solve_depth < 0 ? depth : std::min(P.max_solve_depth, depth);
    if (!check_errors()) return false;
    float ms = 0;
    cudaEventElapsedTime(&ms, ev0, ev1);
    stats.solve_ms = ms;
    stats.kernel_launches = launches;
    double e[3];
    if (!energy(maxD, e)) return false;
    stats.initial_energy = c;
    stats.fit_energy = e[0];
    stats.reg_energy = e[1];
    if (P.verbose)
        printf("Error: %g -> %g = %g + %g => %g\n", c, e[0] + e[1], e[0], e[1], std::sqrt((e[0] + e[1]) / c));
    // regular coefficients of every level in xy64, then hierarchical residuals into tmp64
    for (int l = 0; l <= depth; l++)
        if (!pull_xy(l)) return false;
    for (int l = maxD; l < depth; l++)
    {
        with_dim(this, [&](auto dd) {
            constexpr int D = decltype(dd)::value;
            launch_prolong<D, double>(l, levels[l].xy64, levels[l + 1].xy64, 0, stream, status_of(l + 1));
            return 0;
        });
    }
    for (int l = 0; l <= depth; l++)
    {
        if (!levels[l].tmp64 && !alloc((void **)&levels[l].tmp64, sizeof(double) * 2 * levels[l].N, "alloc sol")) return false;
        if (!cuda_ok(cudaMemcpyAsync(levels[l].tmp64, levels[l].xy64, sizeof(double) * 2 * levels[l].N, cudaMemcpyDeviceToDevice, stream), "copy")) return false;
    }
    for (int l = depth; l > 0; l--)
    {
        // tmp64[l] -= P xy64[l-1]: prolong into a scratch then subtract
        double *scratch = nullptr;
        if (!alloc((void **)&scratch, sizeof(double) * 2 * levels[l].N, "alloc scratch")) return false;
        with_dim(this, [&](auto dd) {
            constexpr int D = decltype(dd)::value;
            launch_prolong<D, double>(l - 1, levels[l - 1].xy64, scratch, 0, stream, status_of(l));
            return 0;
        });
        launch_axpy<double>(levels[l].tmp64, scratch, 2 * levels[l].N, -1.0, stream);
        release(scratch);
        if (!launch_ok("hierarchical")) return false;
    }
    solved = true;
    solves_done++;
    return cuda_ok(cudaStreamSynchronize(stream), "solve sync");
}

}  // namespace epr

using epr::Context;

// =============================================================================================
// C ABI
// =============================================================================================
extern "C" {

void epr_default_params(epr_params *p)
{
    if (!p) return;
    p->s_weight = 100.;
    p->d_weight = 0.00625;
    p->n_sigma = 0.25;
    p->i_mult = 2.;
    p->t_radius = 1;
    p->d_radius = 1;
    p->gs_iters = 10;
    p->min_solve_depth = 0;
    p->max_solve_depth = -1;
    p->seed = 0;
    p->precision = EPR_FP64;
    p->solver = EPR_SOLVER_CASCADIC;
    p->tolerance = 1e-6;
    p->max_cycles = 200;
    p->verbose = 0;
    p->device = 0;
    p->fp64_levels = 0;
    p->fp64_from = 0;
    p->band_precision = EPR_BAND_FP64;
    p->single_level = 0;
    p->separate = 0;
    p->warm_start = 0;
    p->max_extra_sweeps = 0;
    p->target_energy = 0;
    p->project = 0;
    p->adaptive_radius = -1;
}

const char *epr_global_error(void) { return g_error.c_str(); }


epr_ctx *epr_create(int dim, int depth, const epr_params *params)
{
    if (dim != 3 && dim != 4) { g_error = "dim must be 3 or 4"; return nullptr; }
    int maxDepth = dim == 3 ? 10 : 7;
    if (depth < 1 || depth > maxDepth) { g_error = "depth out of range (1.." + std::to_string(maxDepth) + ")"; return nullptr; }
    epr_params p;
    if (params) p = *params; else epr_default_params(&p);
    if (p.t_radius < 0 || p.t_radius > 4 || p.d_radius < 0 || p.d_radius > 4) { g_error = "kernel radius must be in [0,4]"; return nullptr; }
    if (p.precision != EPR_FP64 && p.precision != EPR_FP32) { g_error = "unknown precision"; return nullptr; }
    if (p.solver != EPR_SOLVER_CASCADIC && p.solver != EPR_SOLVER_MULTIGRID) { g_error = "unknown solver"; return nullptr; }
    if (p.fp64_from < 0 || p.fp64_levels < 0) { g_error = "fp64_from and fp64_levels must not be negative"; return nullptr; }
    if (p.band_precision != EPR_BAND_FP64 && p.band_precision != EPR_BAND_DF) { g_error = "unknown band precision"; return nullptr; }
    if (p.solver == EPR_SOLVER_MULTIGRID && (p.max_cycles < 0 || !(p.tolerance >= 0))) { g_error = "bad multigrid cycle cap or tolerance"; return nullptr; }
    if (p.max_extra_sweeps < 0 || !(p.target_energy >= 0)) { g_error = "bad target energy or extra-sweep cap"; return nullptr; }
    if (p.warm_start && p.single_level) { g_error = "a warm start and --singleLevel cannot be combined"; return nullptr; }
    // the reference instantiates the adaptive indexer for kernel radii 0..5 (Hat.adaptive.inl:361-371)
    if (p.adaptive_radius < -1 || p.adaptive_radius > 5) { g_error = "adaptive radius must be -1 (regular grid) or in [0,5]"; return nullptr; }
    if (p.adaptive_radius >= 0 && p.solver != EPR_SOLVER_CASCADIC)
    {
        g_error = "the adaptive indexer is solved by the cascadic schedule only";
        return nullptr;
    }
    if (p.adaptive_radius >= 0 && p.warm_start)
    {
        g_error = "a warm start is defined on the regular grid only (adaptive_radius -1)";
        return nullptr;
    }
    if (cudaSetDevice(p.device) != cudaSuccess)
    {
        g_error = std::string("cannot select CUDA device: ") + cudaGetErrorString(cudaGetLastError());
        return nullptr;
    }
    {
        std::lock_guard<std::mutex> lock(g_create_mutex);
        if (const char *v = getenv("EPR_GS_VARIANT")) epr::set_gs_variant(atoi(v));
        if (const char *v = getenv("EPR_LANES_VARIANT")) epr::set_lanes_variant(atoi(v));
        if (const char *v = getenv("EPR_TINY_LEVELS")) epr::set_tiny_levels(atoi(v));
        if (const char *v = getenv("EPR_CLUSTER_LEVELS")) epr::set_cluster_levels(atoi(v));
        static uint64_t prepared = 0;  // devices whose kernel attributes are set
        if (p.device >= 0 && p.device < 64 && !(prepared & (1ull << p.device)))
        {
            epr::prepare_gs_kernels();
            prepared |= 1ull << p.device;
        }
    }
    epr_ctx *c = new epr_ctx;
    c->dim = dim;
    c->depth = depth;
    c->P = p;
    if (const char *v = getenv("EPR_ALLOC_CAP_BYTES")) c->alloc_cap = (size_t)strtoull(v, nullptr, 10);
    if (const char *v = getenv("EPR_ADAPTIVE_LISTS")) c->adaptive_lists = atoi(v) != 0;
    c->levels.resize(depth + 1);
    if (cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking) != cudaSuccess ||
        cudaEventCreate(&c->ev0) != cudaSuccess || cudaEventCreate(&c->ev1) != cudaSuccess)
    {
        g_error = std::string("CUDA initialisation failed: ") + cudaGetErrorString(cudaGetLastError());
        delete c;
        return nullptr;
    }
    bool ok = c->alloc((void **)&c->red.partial, sizeof(double) * 4 * epr::Reduce::kMaxBlocks, "alloc reduce") &&
              c->alloc((void **)&c->red.out, sizeof(double) * 4, "alloc reduce") &&
              c->alloc((void **)&c->d_err, sizeof(unsigned int), "alloc flag") &&
              c->cuda_ok(cudaMemsetAsync(c->d_err, 0, sizeof(unsigned int), c->stream), "memset flag") &&
              c->alloc((void **)&c->d_kexp, sizeof(int) * (depth + 1), "alloc exponents") &&
              c->cuda_ok(cudaMemsetAsync(c->d_kexp, 0, sizeof(int) * (depth + 1), c->stream), "memset exponents");
    for (int l = 0; ok && l <= depth; l++) ok = c->ensure_level(l);
    if (!ok)
    {
        g_error = c->err;
        delete c;
        return nullptr;
    }
    return c;
}

void epr_destroy(epr_ctx *ctx) { delete ctx; }

const char *epr_last_error(const epr_ctx *ctx) { return ctx ? ctx->err.c_str() : g_error.c_str(); }

#define EPR_CHECK_CTX(ctx) \
    do { if (!(ctx)) { g_error = "null context"; return EPR_ERR_ARG; } (ctx)->status = EPR_OK; cudaSetDevice((ctx)->P.device); } while (0)
#define EPR_CHECK_LEVEL(ctx, l) \
    do { if ((l) < 0 || (l) > (ctx)->depth) { (ctx)->fail(EPR_ERR_ARG, "level %d out of range", (int)(l)); return EPR_ERR_ARG; } } while (0)
#define EPR_RETURN(ctx, ok) return (ok) ? EPR_OK : ((ctx)->status ? (ctx)->status : EPR_ERR_CUDA)

int epr_set_samples(epr_ctx *ctx, size_t n, const double *pos, const double *skew)
{
    EPR_CHECK_CTX(ctx);
    if (!n || !pos || !skew) { ctx->fail(EPR_ERR_ARG, "expected some samples: %zu", n); return EPR_ERR_ARG; }
    for (size_t i = 0; i < n * (size_t)ctx->dim; i++)
        if (!std::isfinite(pos[i])) { ctx->fail(EPR_ERR_ARG, "sample %zu has a non-finite coordinate", i / ctx->dim); return EPR_ERR_ARG; }
    size_t K = (size_t)(ctx->dim * (ctx->dim - 1) / 2);
    for (size_t i = 0; i < n * K; i++)
        if (!std::isfinite(skew[i])) { ctx->fail(EPR_ERR_ARG, "sample %zu has a non-finite frame", i / K); return EPR_ERR_ARG; }
    EPR_RETURN(ctx, ctx->setup.set_samples(*ctx, n, pos, skew));
}

int epr_build(epr_ctx *ctx)
{
    EPR_CHECK_CTX(ctx);
    if (!ctx->setup.n) { ctx->fail(EPR_ERR_STATE, "epr_build called before epr_set_samples"); return EPR_ERR_STATE; }
    EPR_RETURN(ctx, ctx->setup.build(*ctx));
}

int epr_set_level_system(epr_ctx *ctx, int level, const double *R, const double *B, double c)
{
    EPR_CHECK_CTX(ctx);
    EPR_CHECK_LEVEL(ctx, level);
    if (!R || !B) { ctx->fail(EPR_ERR_ARG, "null stencil"); return EPR_ERR_ARG; }
    epr::Level &L = ctx->levels[level];
    size_t S = (size_t)ctx->stencil();
    // host column stencils (node-major) -> device offset-major
    std::vector<double> a(S * L.N), b(S * L.N);
    for (int64_t i = 0; i < L.N; i++)
        for (size_t o = 0; o < S; o++) { a[o * L.N + i] = R[i * S + o]; b[o * L.N + i] = B[i * S + o]; }
    bool ok = ctx->cuda_ok(cudaMemcpyAsync(L.A64, a.data(), sizeof(double) * a.size(), cudaMemcpyHostToDevice, ctx->stream), "upload R") &&
              ctx->cuda_ok(cudaMemcpyAsync(L.B64, b.data(), sizeof(double) * b.size(), cudaMemcpyHostToDevice, ctx->stream), "upload B") &&
              epr::add_dirichlet(*ctx, level) && ctx->sync_system32(level) &&
              ctx->cuda_ok(cudaStreamSynchronize(ctx->stream), "sync");
    ctx->c = c;
    ctx->have_system = true;
    EPR_RETURN(ctx, ok);
}

int epr_set_coefficients(epr_ctx *ctx, int level, const double *x, const double *y)
{
    EPR_CHECK_CTX(ctx);
    EPR_CHECK_LEVEL(ctx, level);
    if (!x || !y) { ctx->fail(EPR_ERR_ARG, "null coefficients"); return EPR_ERR_ARG; }
    EPR_RETURN(ctx, ctx->upload_xy(level, x, y));
}

int epr_get_coefficients(epr_ctx *ctx, int level, double *x, double *y)
{
    EPR_CHECK_CTX(ctx);
    EPR_CHECK_LEVEL(ctx, level);
    if (!x || !y) { ctx->fail(EPR_ERR_ARG, "null output"); return EPR_ERR_ARG; }
    EPR_RETURN(ctx, ctx->download_xy(level, x, y, false));
}

int epr_energy(epr_ctx *ctx, int level, double *out3)
{
    EPR_CHECK_CTX(ctx);
    EPR_CHECK_LEVEL(ctx, level);
    if (!out3) { ctx->fail(EPR_ERR_ARG, "null output"); return EPR_ERR_ARG; }
    EPR_RETURN(ctx, ctx->energy(level, out3));
}

int epr_quadfit(epr_ctx *ctx, int level, double *out)
{
    EPR_CHECK_CTX(ctx);
    EPR_CHECK_LEVEL(ctx, level);
    if (!out) { ctx->fail(EPR_ERR_ARG, "null output"); return EPR_ERR_ARG; }
    epr::Level &L = ctx->levels[level];
    double *d = nullptr;
    bool ok = ctx->alloc((void **)&d, sizeof(double) * 5 * L.N, "alloc fit");
    if (ok && ctx->lvlDF(level)) ok = ctx->pull_xy(level);  // a double-float level's fit in double
    if (ok)
    {
        bool fp32 = ctx->lvl32(level);
        epr::with_dim(ctx, [&](auto dd) {
            constexpr int D = decltype(dd)::value;
            if (fp32) epr::launch_quadfit<D, float>(epr::level_ptrs<float>(ctx, level), L.xy32, d, ctx->stream);
            else epr::launch_quadfit<D, double>(epr::level_ptrs<double>(ctx, level), L.xy64, d, ctx->stream);
            return 0;
        });
        ok = ctx->launch_ok("quadfit") &&
             ctx->cuda_ok(cudaMemcpyAsync(out, d, sizeof(double) * 5 * L.N, cudaMemcpyDeviceToHost, ctx->stream), "copy fit") &&
             ctx->cuda_ok(cudaStreamSynchronize(ctx->stream), "sync");
        ctx->release(d);
    }
    EPR_RETURN(ctx, ok);
}

int epr_gradient(epr_ctx *ctx, int level, double *gx, double *gy)
{
    EPR_CHECK_CTX(ctx);
    EPR_CHECK_LEVEL(ctx, level);
    if (!gx || !gy) { ctx->fail(EPR_ERR_ARG, "null output"); return EPR_ERR_ARG; }
    std::vector<double> q(5 * ctx->levels[level].N);
    int rc = epr_quadfit(ctx, level, q.data());
    if (rc) return rc;
    for (int64_t i = 0; i < ctx->levels[level].N; i++) { gx[i] = q[5 * i + 3]; gy[i] = q[5 * i + 4]; }
    return EPR_OK;
}

int epr_gs(epr_ctx *ctx, int level, int iters)
{
    EPR_CHECK_CTX(ctx);
    EPR_CHECK_LEVEL(ctx, level);
    if (iters < 0) { ctx->fail(EPR_ERR_ARG, "negative iteration count"); return EPR_ERR_ARG; }
    EPR_RETURN(ctx, ctx->gs(level, iters) && ctx->check_errors());
}

int epr_prolong(epr_ctx *ctx, int level)
{
    EPR_CHECK_CTX(ctx);
    if (level < 0 || level >= ctx->depth) { ctx->fail(EPR_ERR_ARG, "level %d has no finer level", level); return EPR_ERR_ARG; }
    EPR_RETURN(ctx, ctx->prolong_add(level) && ctx->cuda_ok(cudaStreamSynchronize(ctx->stream), "sync"));
}

int epr_gn_matvec(epr_ctx *ctx, int level, const double *dx, const double *dy, double *ox, double *oy)
{
    EPR_CHECK_CTX(ctx);
    EPR_CHECK_LEVEL(ctx, level);
    if (!dx || !dy || !ox || !oy) { ctx->fail(EPR_ERR_ARG, "null vector"); return EPR_ERR_ARG; }
    epr::Level &L = ctx->levels[level];
    std::vector<double> h(2 * L.N);
    for (int64_t i = 0; i < L.N; i++) { h[2 * i] = dx[i]; h[2 * i + 1] = dy[i]; }
    double *d64 = nullptr, *o64 = nullptr;
    float *d32 = nullptr, *o32 = nullptr;
    bool fp32 = ctx->lvl32(level);
    if (ctx->lvlDF(level) && !ctx->pull_xy(level)) EPR_RETURN(ctx, false);  // evaluated in double
    bool ok = ctx->alloc((void **)&d64, sizeof(double) * 2 * L.N, "alloc") && ctx->alloc((void **)&o64, sizeof(double) * 2 * L.N, "alloc") &&
              ctx->cuda_ok(cudaMemcpyAsync(d64, h.data(), sizeof(double) * 2 * L.N, cudaMemcpyHostToDevice, ctx->stream), "upload");
    if (ok && fp32)
    {
        ok = ctx->alloc((void **)&d32, sizeof(float) * 2 * L.N, "alloc") && ctx->alloc((void **)&o32, sizeof(float) * 2 * L.N, "alloc");
        if (ok) epr::launch_convert_d2f(d64, d32, 2 * L.N, ctx->stream);
    }
    if (ok)
    {
        epr::with_dim(ctx, [&](auto dd) {
            constexpr int D = decltype(dd)::value;
            if (fp32) epr::launch_gn_matvec<D, float>(epr::level_ptrs<float>(ctx, level), L.xy32, d32, o32, ctx->stream);
            else epr::launch_gn_matvec<D, double>(epr::level_ptrs<double>(ctx, level), L.xy64, d64, o64, ctx->stream);
            return 0;
        });
        if (fp32) epr::launch_convert_f2d(o32, o64, 2 * L.N, ctx->stream);
        ok = ctx->launch_ok("gn matvec") &&
             ctx->cuda_ok(cudaMemcpyAsync(h.data(), o64, sizeof(double) * 2 * L.N, cudaMemcpyDeviceToHost, ctx->stream), "download") &&
             ctx->cuda_ok(cudaStreamSynchronize(ctx->stream), "sync");
        if (ok)
            for (int64_t i = 0; i < L.N; i++) { ox[i] = h[2 * i]; oy[i] = h[2 * i + 1]; }
    }
    ctx->release(d64); ctx->release(o64); ctx->release(d32); ctx->release(o32);
    EPR_RETURN(ctx, ok);
}

int epr_solve(epr_ctx *ctx, epr_stats *stats)
{
    EPR_CHECK_CTX(ctx);
    if (!ctx->have_system) { ctx->fail(EPR_ERR_STATE, "epr_solve called before epr_build"); return EPR_ERR_STATE; }
    ctx->stats.node_updates = 0;
    ctx->launches = 0;
    ctx->stats.cycles = 0;
    bool ok = ctx->solve_cascadic();
    if (ok && stats) *stats = ctx->stats;
    EPR_RETURN(ctx, ok);
}

// Many independent reconstructions on one GPU.  A reconstruction at depth 5-7 keeps only a part of
// the 152 SMs busy (a colour of a 33^3 grid is 4.5K nodes) and spends much of its time in launch
// latency, so several run at once: host workers each take whole reconstructions, largest first,
// and drive them on the contexts' own non-blocking streams, where the device overlaps their
// kernels.  Every context computes exactly what it computes alone (same kernels, same launch
// configurations, its own stream and memory), so the results do not depend on the schedule.
int epr_batch_solve(epr_ctx *const *ctxs, int n, int build, int threads, epr_stats *stats, int *status)
{
    if (n < 0 || (n > 0 && !ctxs)) { g_error = "bad batch"; return EPR_ERR_ARG; }
    for (int i = 0; i < n; i++)
    {
        if (!ctxs[i]) { g_error = "null context in batch"; return EPR_ERR_ARG; }
        for (int j = 0; j < i; j++)
            if (ctxs[j] == ctxs[i]) { g_error = "a context appears twice in the batch"; return EPR_ERR_ARG; }
    }
    for (int i = 1; i < n; i++)
        if (ctxs[i]->P.device != ctxs[0]->P.device) { g_error = "the batch's contexts are on different devices"; return EPR_ERR_ARG; }
    if (n == 0) return EPR_OK;
    // largest reconstruction first (finest-level nodes, then samples): the long ones start early
    std::vector<int> order(n);
    for (int i = 0; i < n; i++) order[i] = i;
    auto cost = [&](int i) {
        const epr::Context *c = ctxs[i];
        return std::make_pair(c->levels[c->depth].N, (int64_t)c->setup.n);
    };
    std::stable_sort(order.begin(), order.end(), [&](int a, int b) { return cost(a) > cost(b); });
    std::vector<int> rc(n, EPR_OK);
    std::atomic<int> next{0};
    if (threads <= 0) threads = kBatchThreads;
    threads = std::min(threads, n);
    // One stream per worker, created together: the device spreads streams over its hardware work
    // queues in creation order, so the workers' streams do not share a queue (the contexts' own
    // streams, created one per context, would put concurrently running contexts on the same queue
    // and serialise them).  A context runs on its worker's stream while the worker holds it; every
    // build and solve ends with a stream synchronisation, so nothing is in flight when the
    // context's own stream comes back.
    std::vector<cudaStream_t> streams(threads, nullptr);
    cudaSetDevice(ctxs[0]->P.device);
    for (int t = 0; t < threads; t++)
        if (cudaStreamCreateWithFlags(&streams[t], cudaStreamNonBlocking) != cudaSuccess)
        {
            streams[t] = nullptr;  // the worker then uses the contexts' own streams
            cudaGetLastError();
        }
    auto worker = [&](int t) {
        for (int k; (k = next.fetch_add(1)) < n;)
        {
            const int i = order[k];
            epr_ctx *c = ctxs[i];
            cudaStream_t own = c->stream;
            const bool swap = streams[t] != nullptr;
            if (swap)
            {
                cudaStreamSynchronize(own);  // work the context queued before the batch
                c->stream = streams[t];
            }
            int r = build ? epr_build(c) : EPR_OK;
            if (r == EPR_OK) r = epr_solve(c, stats ? &stats[i] : nullptr);
            if (swap)
            {
                cudaStreamSynchronize(c->stream);
                c->stream = own;
            }
            rc[i] = r;
        }
    };
    std::vector<std::thread> pool;
    for (int t = 1; t < threads; t++) pool.emplace_back(worker, t);
    worker(0);
    for (std::thread &t : pool) t.join();
    for (cudaStream_t st : streams)
        if (st) cudaStreamDestroy(st);
    int first = EPR_OK;
    for (int i = 0; i < n; i++)
    {
        if (status) status[i] = rc[i];
        if (first == EPR_OK && rc[i] != EPR_OK)
        {
            first = rc[i];
            g_error = "context " + std::to_string(i) + ": " + ctxs[i]->err;
        }
    }
    return first;
}

int epr_get_solution(epr_ctx *ctx, int level, double *x, double *y)
{
    EPR_CHECK_CTX(ctx);
    EPR_CHECK_LEVEL(ctx, level);
    if (!ctx->solved) { ctx->fail(EPR_ERR_STATE, "no solution yet"); return EPR_ERR_STATE; }
    if (!x || !y) { ctx->fail(EPR_ERR_ARG, "null output"); return EPR_ERR_ARG; }
    EPR_RETURN(ctx, ctx->download_xy(level, x, y, true));
}

int epr_get_array(epr_ctx *ctx, const char *name, int level, double *out, size_t cap, size_t *count)
{
    EPR_CHECK_CTX(ctx);
    if (!name) { ctx->fail(EPR_ERR_ARG, "null name"); return EPR_ERR_ARG; }
    std::string nm(name);
    if (nm == "R" || nm == "B" || nm == "A")
    {
        EPR_CHECK_LEVEL(ctx, level);
        epr::Level &L = ctx->levels[level];
        size_t S = (size_t)ctx->stencil(), n = S * (size_t)L.N;
        if (count) *count = n;
        if (!out) return EPR_OK;
        if (cap < n) { ctx->fail(EPR_ERR_ARG, "output too small (%zu < %zu)", cap, n); return EPR_ERR_ARG; }
        std::vector<double> a(n), r(n);
        bool ok = ctx->cuda_ok(cudaMemcpyAsync(a.data(), nm == "B" ? L.B64 : L.A64, sizeof(double) * n, cudaMemcpyDeviceToHost, ctx->stream), "copy");
        if (ok && nm == "R")
        {
            // R = A - dWeight K
            double *k = nullptr;
            ok = ctx->alloc((void **)&k, sizeof(double) * n, "alloc") &&
                 ctx->cuda_ok(cudaMemsetAsync(k, 0, sizeof(double) * n, ctx->stream), "memset") &&
                 epr::add_dirichlet_to(*ctx, level, k, 1.0) &&
                 ctx->cuda_ok(cudaMemcpyAsync(r.data(), k, sizeof(double) * n, cudaMemcpyDeviceToHost, ctx->stream), "copy");
            ctx->release(k);
        }
        ok = ok && ctx->cuda_ok(cudaStreamSynchronize(ctx->stream), "sync");
        if (!ok) EPR_RETURN(ctx, false);
        for (int64_t i = 0; i < L.N; i++)
            for (size_t o = 0; o < S; o++)
                out[i * S + o] = a[o * L.N + i] - (nm == "R" ? ctx->P.d_weight * r[o * L.N + i] : 0.);
        return EPR_OK;
    }
    if (nm == "c")
    {
        if (count) *count = 1;
        if (out && cap >= 1) out[0] = ctx->c;
        return EPR_OK;
    }
    EPR_RETURN(ctx, ctx->setup.get(*ctx, nm, out, cap, count));
}

int epr_get_density(epr_ctx *ctx, int level, double *out, size_t cap, size_t *count)
{
    EPR_CHECK_CTX(ctx);
    EPR_CHECK_LEVEL(ctx, level);
    const size_t W = (size_t)(1 + ctx->dim + ctx->dim * ctx->dim);
    const size_t num = W * (size_t)ctx->levels[level].N;
    if (count) *count = num;
    if (!out) return EPR_OK;
    if ((int)ctx->setup.density.size() <= level || !ctx->setup.density[level])
    {
        ctx->fail(EPR_ERR_STATE, "the density estimator is not available before epr_build");
        return EPR_ERR_STATE;
    }
    if (cap < num) { ctx->fail(EPR_ERR_ARG, "output too small (%zu < %zu)", cap, num); return EPR_ERR_ARG; }
    EPR_RETURN(ctx, ctx->cuda_ok(cudaMemcpyAsync(out, ctx->setup.density[level], sizeof(double) * num, cudaMemcpyDeviceToHost, ctx->stream), "copy") &&
                        ctx->cuda_ok(cudaStreamSynchronize(ctx->stream), "sync"));
}

int epr_time_kernel(epr_ctx *ctx, const char *kernel, int level, int reps, double *ms)
{
    EPR_CHECK_CTX(ctx);
    EPR_CHECK_LEVEL(ctx, level);
    if (!kernel || !ms || reps < 1) { ctx->fail(EPR_ERR_ARG, "bad arguments"); return EPR_ERR_ARG; }
    std::string k(kernel);
    if (k == "lgs" || k == "residual" || k == "assemble" || k == "biquad")
    {
        if (!ctx->have_system) { ctx->fail(EPR_ERR_STATE, "no system"); return EPR_ERR_STATE; }
        EPR_RETURN(ctx, epr::time_mg_kernel(*ctx, kernel, level, reps, ms));
    }
    epr::Level &L = ctx->levels[level];
    bool fp32 = ctx->lvl32(level);
    double *scratch = nullptr;
    void *pair = nullptr, *out = nullptr;
    size_t rs = fp32 ? sizeof(float) : sizeof(double);
    bool ok = ctx->alloc((void **)&scratch, sizeof(double) * 5 * L.N, "alloc") && ctx->alloc(&pair, rs * 2 * L.N, "alloc") &&
              ctx->alloc(&out, rs * 2 * L.N, "alloc") && ctx->cuda_ok(cudaMemsetAsync(pair, 0, rs * 2 * L.N, ctx->stream), "memset");
    if (ok && (k == "prolong" && level >= ctx->depth)) { ctx->fail(EPR_ERR_ARG, "no finer level"); ok = false; }
    if (ok && k != "gs" && k != "energy" && k != "quadfit" && k != "prolong" && k != "gn")
    {
        ctx->fail(EPR_ERR_ARG, "unknown kernel '%s'", kernel);
        ok = false;
    }
    const bool dfLevel = ctx->lvlDF(level) && k == "gs";
    auto run = [&]() {
        if (dfLevel)
        {
            // one colour of a double-float level (its point-split kernel on pairs of floats)
            epr::launch_gs_colour_df(epr::level_ptrs<epr::df>(ctx, level), 0, ctx->d_err, ctx->stream, ctx->d_kexp);
            return;
        }
        epr::with_dim(ctx, [&](auto dd) {
            constexpr int D = decltype(dd)::value;
            if (fp32)
            {
                auto P = epr::level_ptrs<float>(ctx, level);
                if (k == "gs") epr::launch_gs_colour<D, float>(P, 0, ctx->d_err, ctx->stream);
                else if (k == "energy") epr::launch_energy<D, float>(P, L.xy32, ctx->red, ctx->stream);
                else if (k == "quadfit") epr::launch_quadfit<D, float>(P, L.xy32, scratch, ctx->stream);
                else if (k == "prolong") epr::launch_prolong<D, float>(level, L.xy32, ctx->levels[level + 1].xy32, 1, ctx->stream, ctx->status_of(level + 1));
                else epr::launch_gn_matvec<D, float>(P, L.xy32, (const float *)pair, (float *)out, ctx->stream);
            }
            else
            {
                auto P = epr::level_ptrs<double>(ctx, level);
                if (k == "gs") epr::launch_gs_colour<D, double>(P, 0, ctx->d_err, ctx->stream);
                else if (k == "energy") epr::launch_energy<D, double>(P, L.xy64, ctx->red, ctx->stream);
                else if (k == "quadfit") epr::launch_quadfit<D, double>(P, L.xy64, scratch, ctx->stream);
                else if (k == "prolong") epr::launch_prolong<D, double>(level, L.xy64, ctx->levels[level + 1].xy64, 1, ctx->stream, ctx->status_of(level + 1));
                else epr::launch_gn_matvec<D, double>(P, L.xy64, (const double *)pair, (double *)out, ctx->stream);
            }
            return 0;
        });
    };
    if (ok)
    {
        run();  // warm-up launch
        cudaEventRecord(ctx->ev0, ctx->stream);
        for (int i = 0; i < reps; i++) run();
        cudaEventRecord(ctx->ev1, ctx->stream);
        ok = ctx->launch_ok("time kernel") && ctx->cuda_ok(cudaEventSynchronize(ctx->ev1), "sync");
        float t = 0;
        if (ok) cudaEventElapsedTime(&t, ctx->ev0, ctx->ev1);
        *ms = (double)t / reps;
    }
    ctx->release(scratch); ctx->release(pair); ctx->release(out);
    EPR_RETURN(ctx, ok);
}

int epr_linear_gs(epr_ctx *ctx, int level, const double *M, const double *b, double *v, int iters)
{
    EPR_CHECK_CTX(ctx);
    EPR_CHECK_LEVEL(ctx, level);
    if (!M || !b || !v || iters < 0) { ctx->fail(EPR_ERR_ARG, "bad arguments"); return EPR_ERR_ARG; }
    EPR_RETURN(ctx, epr::linear_gs(*ctx, level, M, b, v, iters));
}

int epr_mg_vcycle(epr_ctx *ctx, int level, const double *M, const double *b, double *v, int gs_iters, int cycles)
{
    EPR_CHECK_CTX(ctx);
    EPR_CHECK_LEVEL(ctx, level);
    if (!M || !b || !v || gs_iters < 0 || cycles < 0) { ctx->fail(EPR_ERR_ARG, "bad arguments"); return EPR_ERR_ARG; }
    EPR_RETURN(ctx, epr::mg_vcycles(*ctx, level, M, b, v, gs_iters, cycles));
}

int epr_alternating_system(epr_ctx *ctx, int level, int which, double *M, double *b)
{
    EPR_CHECK_CTX(ctx);
    EPR_CHECK_LEVEL(ctx, level);
    if (!M || !b || (which != 0 && which != 1)) { ctx->fail(EPR_ERR_ARG, "bad arguments"); return EPR_ERR_ARG; }
    if (!ctx->have_system) { ctx->fail(EPR_ERR_STATE, "no system (call epr_build or epr_set_level_system)"); return EPR_ERR_STATE; }
    EPR_RETURN(ctx, epr::alternating_system(*ctx, level, which, M, b));
}

int epr_alternating_solve(epr_ctx *ctx, int level, int iters, int vcycles, int gs_iters, int single_level)
{
    EPR_CHECK_CTX(ctx);
    EPR_CHECK_LEVEL(ctx, level);
    if (iters < 0 || vcycles < 0 || gs_iters < 0) { ctx->fail(EPR_ERR_ARG, "negative iteration count"); return EPR_ERR_ARG; }
    if (!ctx->have_system) { ctx->fail(EPR_ERR_STATE, "no system (call epr_build or epr_set_level_system)"); return EPR_ERR_STATE; }
    EPR_RETURN(ctx, epr::alternating_solve(*ctx, level, iters, vcycles, gs_iters, single_level != 0) &&
                        ctx->cuda_ok(cudaStreamSynchronize(ctx->stream), "sync"));
}

int epr_biquadratic_fit(epr_ctx *ctx, int level, const double *dx, const double *dy, int as_reference, double *q9)
{
    EPR_CHECK_CTX(ctx);
    EPR_CHECK_LEVEL(ctx, level);
    if (!dx || !dy || !q9) { ctx->fail(EPR_ERR_ARG, "null argument"); return EPR_ERR_ARG; }
    if (!ctx->have_system) { ctx->fail(EPR_ERR_STATE, "no system (call epr_build or epr_set_level_system)"); return EPR_ERR_STATE; }
    epr::Level &L = ctx->levels[level];
    std::vector<double> h(2 * L.N);
    for (int64_t i = 0; i < L.N; i++) { h[2 * i] = dx[i]; h[2 * i + 1] = dy[i]; }
    double *d = nullptr;
    bool ok = ctx->alloc((void **)&d, sizeof(double) * 2 * L.N, "alloc direction") &&
              ctx->cuda_ok(cudaMemcpyAsync(d, h.data(), sizeof(double) * 2 * L.N, cudaMemcpyHostToDevice, ctx->stream), "upload") &&
              epr::biquadratic_fit(*ctx, level, d, as_reference != 0, q9);
    ctx->release(d);
    EPR_RETURN(ctx, ok);
}

int epr_step_size(const double *q9, double *s)
{
    if (!q9 || !s) { g_error = "null argument"; return EPR_ERR_ARG; }
    *s = epr::poly::step_size(q9);
    return std::isfinite(*s) ? EPR_OK : EPR_ERR_NUMERIC;
}

int epr_newton_update(const double *q9, int steps, double *st2)
{
    if (!q9 || !st2 || steps < 0) { g_error = "bad arguments"; return EPR_ERR_ARG; }
    epr::poly::newton_update(q9, steps, st2);
    return std::isfinite(st2[0]) && std::isfinite(st2[1]) ? EPR_OK : EPR_ERR_NUMERIC;
}

int epr_synchronize(epr_ctx *ctx)
{
    EPR_CHECK_CTX(ctx);
    EPR_RETURN(ctx, ctx->cuda_ok(cudaStreamSynchronize(ctx->stream), "sync"));
}

}  // extern "C"
