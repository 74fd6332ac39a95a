// Lockstep batches: many 3D reconstructions relaxed together, one launch per level and colour for
// all of them, the whole relaxation captured as one CUDA graph per batch.
//
// epr_batch_solve (epr_capi.cu) overlaps whole solves on host worker streams; each reconstruction
// still issues its own ~10,000 launches, and the coarse levels of every one of them are latency
// bound.  Here the cascadic schedule (ExteriorPoisson.h:315-409) of all members advances level by
// level: the levels every member has (3D levels 0-1) run in one block per member, and from level 2
// on each sweep's colour is one launch whose grid spans the colour's nodes of every member still
// sweeping that level (members sorted by their sweep count, so the ones still sweeping are a
// prefix of the table).  Every member's nodes see exactly the kernels and arithmetic of its own
// solve (the same bodies, block shapes that change no node's arithmetic), so every member gets its
// solo solve's bits.
//
// The block shapes of the colour kernels (nodes per block of the point-split kernel, threads per
// block of the lane kernel) are the tiles an autotuner picks per level: epr_batch_tune times every
// shape on the batch's own data and keeps the fastest.
#include <algorithm>
#include <atomic>
#include <cmath>
#include <cstring>
#include <string>
#include <thread>
#include <vector>

#include "epr_context.h"

namespace {

using namespace epr;

constexpr int kMaxLevels = 16;
constexpr int kTypeFloat = 0, kTypeDouble = 1, kTypeDF = 2;

struct LevelPlan
{
    int level = 0;
    int type = kTypeFloat;
    int count = 0;             // members that relax this level
    bool tiny = false;         // all sweeps in one launch per member (3D levels 0-1; 2 in double-float)
    std::vector<int> iters;    // per job, non-increasing
    std::vector<int> members;  // per job
    size_t off = 0;            // byte offset of the BatchJob table in the image
};

// level -> level + 1 of every member whose solve goes on (prolong_add of a solo solve)
struct XferPlan
{
    int level = 0;
    int count = 0;
    int ctype = kTypeFloat, ftype = kTypeFloat;
    // XferJob tables: coarse float -> double, coarse double-float -> double, fine float -> double,
    // fine double-float -> double, the prolongation, fine double -> float, fine double -> double-float
    size_t off[7] = {0, 0, 0, 0, 0, 0, 0};
};

template <typename T>
size_t append(std::vector<uint8_t> &img, const std::vector<T> &v)
{
    size_t off = (img.size() + 63) / 64 * 64;
    img.resize(off + sizeof(T) * v.size());
    if (!v.empty()) std::memcpy(img.data() + off, v.data(), sizeof(T) * v.size());
    return off;
}

int level_type(Context *c, int l)
{
    if (c->lvlDF(l)) return kTypeDF;
    return c->lvl32(l) ? kTypeFloat : kTypeDouble;
}

}  // namespace

struct epr_batch
{
    std::vector<epr_ctx *> ctxs;
    int threads = 8;
    int device = 0;
    cudaStream_t stream = nullptr;
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    std::vector<LevelPlan> levels;
    std::vector<XferPlan> xfers;
    std::vector<uint8_t> image, captured;  // job tables (host), and the ones the graph was captured with
    uint8_t *dtab = nullptr;
    size_t dtabBytes = 0;
    int tile[kMaxLevels];
    cudaGraphExec_t graph = nullptr;
    int64_t graphLaunches = 0;
    double relax_ms = 0;
    std::string err;

    bool fail(const std::string &m)
    {
        err = m;
        return false;
    }
    bool ok(cudaError_t e, const char *what)
    {
        if (e == cudaSuccess) return true;
        cudaGetLastError();
        return fail(std::string(what) + ": " + cudaGetErrorString(e));
    }
    ~epr_batch()
    {
        if (graph) cudaGraphExecDestroy(graph);
        if (dtab) cudaFree(dtab);
        if (e0) cudaEventDestroy(e0);
        if (e1) cudaEventDestroy(e1);
        if (stream) cudaStreamDestroy(stream);
    }
};

namespace {

// the plan of the lockstep schedule and the job tables it reads; false (with b.err) when the
// members cannot share it
bool make_plan(epr_batch &b)
{
    const int n = (int)b.ctxs.size();
    std::vector<int> maxD(n);
    int minD = -1, top = 0;
    for (int i = 0; i < n; i++)
    {
        Context *c = b.ctxs[i];
        const std::string who = "context " + std::to_string(i) + ": ";
        if (!c->have_system) return b.fail(who + "not built");
        if (c->dim != 3) return b.fail(who + "lockstep batches are 3D");
        if (c->P.solver != EPR_SOLVER_CASCADIC || c->P.single_level || c->P.verbose || c->P.warm_start || c->P.target_energy > 0 ||
            c->P.adaptive_radius >= 0)
            return b.fail(who + "lockstep batches run the plain cascadic schedule on the regular grid (no multigrid, single "
                                "level, verbose, warm start, target energy or adaptive indexer)");
        const int m = std::min(c->P.min_solve_depth, c->depth);
        if (minD >= 0 && m != minD) return b.fail(who + "all members need the same minimum solve depth");
        minD = m;
        maxD[i] = c->P.max_solve_depth < 0 ? c->depth : std::min(c->P.max_solve_depth, c->depth);
        top = std::max(top, maxD[i]);
    }
    if (top >= kMaxLevels) return b.fail("depth too large for a lockstep batch");
    b.levels.clear();
    b.xfers.clear();
    b.image.clear();
    for (int l = minD; l <= top; l++)
    {
        LevelPlan P;
        P.level = l;
        std::vector<std::pair<int, int>> act;  // (-iters, member): sorted, the longest first
        for (int i = 0; i < n; i++)
        {
            if (maxD[i] < l) continue;
            Context *c = b.ctxs[i];
            const int t = level_type(c, l);
            if (!act.empty() && t != P.type)
                return b.fail("level " + std::to_string(l) + " relaxes in different arithmetic in different members");
            P.type = t;
            const int iters = (int)std::ceil(std::pow(c->P.i_mult, c->depth - l) * c->P.gs_iters);
            act.push_back({-iters, i});
        }
        std::stable_sort(act.begin(), act.end());
        P.count = (int)act.size();
        // all sweeps in one launch per member: levels 0-1, and level 2 in double-float on a cluster
        // per member (the solo solve's kernels)
        P.tiny = b.ctxs[act[0].second]->levels[l].N <= 27 || cluster_level(l, P.type == kTypeDF);
        for (auto &a : act)
        {
            P.iters.push_back(-a.first);
            P.members.push_back(a.second);
        }
        auto jobs = [&](auto tag) {
            using Real = decltype(tag);
            std::vector<BatchJob<Real>> v;
            for (size_t k = 0; k < act.size(); k++)
            {
                Context *c = b.ctxs[P.members[k]];
                BatchJob<Real> j;
                j.L = level_ptrs<Real>(c, l);
                j.err = c->d_err;
                j.kexp = P.type == kTypeDF ? c->d_kexp : nullptr;
                j.iters = P.iters[k];
                j.separate = c->P.separate;
                v.push_back(j);
            }
            return append(b.image, v);
        };
        if (P.type == kTypeFloat) P.off = jobs(float());
        else if (P.type == kTypeDouble) P.off = jobs(double());
        else P.off = jobs(df());
        b.levels.push_back(P);
    }
    for (int l = minD; l < top; l++)
    {
        XferPlan X;
        X.level = l;
        std::vector<int> mem;
        for (int i = 0; i < n; i++)
            if (maxD[i] > l) mem.push_back(i);
        if (mem.empty()) continue;
        X.count = (int)mem.size();
        X.ctype = level_type(b.ctxs[mem[0]], l);
        X.ftype = level_type(b.ctxs[mem[0]], l + 1);
        std::vector<XferJob> t[7];
        for (int i : mem)
        {
            Context *c = b.ctxs[i];
            Level &C = c->levels[l], &F = c->levels[l + 1];
            t[0].push_back({C.xy32, C.xy64, nullptr});
            t[1].push_back({C.xyd, C.xy64, c->d_kexp});
            t[2].push_back({F.xy32, F.xy64, nullptr});
            t[3].push_back({F.xyd, F.xy64, c->d_kexp});
            if (X.ctype == kTypeFloat && X.ftype == kTypeFloat) t[4].push_back({C.xy32, F.xy32, nullptr});
            else t[4].push_back({C.xy64, F.xy64, nullptr});
            t[5].push_back({F.xy64, F.xy32, nullptr});
            t[6].push_back({F.xy64, F.xyd, c->d_kexp});
        }
        for (int k = 0; k < 7; k++) X.off[k] = append(b.image, t[k]);
        b.xfers.push_back(X);
    }
    return true;
}

// the lockstep relaxation on b.stream (captured or not); returns the number of launches
int64_t record(epr_batch &b)
{
    int64_t launches = 0;
    const cudaStream_t s = b.stream;
    size_t xi = 0;
    for (const LevelPlan &P : b.levels)
    {
        const int l = P.level;
        auto run = [&](auto tag) {
            using Real = decltype(tag);
            const BatchJob<Real> *jobs = reinterpret_cast<const BatchJob<Real> *>(b.dtab + P.off);
            if (P.tiny)
            {
                launch_tiny_batch<Real>(jobs, l, P.count, s);
                launches++;
                return;
            }
            int cnt = P.count;
            for (int k = 0; k < P.iters[0]; k++)
            {
                while (cnt > 0 && P.iters[cnt - 1] <= k) cnt--;  // members done with this level
                for (int c = 0; c < 8; c++)
                {
                    launch_colour_batch<Real>(jobs, l, c, cnt, b.tile[l], s);
                    launches++;
                }
                if constexpr (std::is_same<Real, df>::value)
                {
                    launch_df_rescale_batch(jobs, cnt, s);
                    launches++;
                }
            }
        };
        if (P.type == kTypeFloat) run(float());
        else if (P.type == kTypeDouble) run(double());
        else run(df());
        if (xi < b.xfers.size() && b.xfers[xi].level == l)
        {
            // prolong_add of a solo solve, step by step
            const XferPlan &X = b.xfers[xi++];
            const int64_t rc = (1 << l) + 1, rf = (1 << (l + 1)) + 1;
            const int64_t nc = 2 * rc * rc * rc, nf = 2 * rf * rf * rf;  // values of the coarse and fine level
            auto T = [&](int k) { return reinterpret_cast<const XferJob *>(b.dtab + X.off[k]); };
            const bool c32 = X.ctype == kTypeFloat, f32 = X.ftype == kTypeFloat, cdf = X.ctype == kTypeDF, fdf = X.ftype == kTypeDF;
            if (c32 && f32)
            {
                launch_prolong_add_batch<float>(T(4), l, X.count, s);
                launches++;
                continue;
            }
            if (c32) { launch_f2d_batch(T(0), nc, X.count, s); launches++; }
            if (cdf) { launch_df_pull_batch(T(1), nc, l, X.count, s); launches++; }
            if (f32) { launch_f2d_batch(T(2), nf, X.count, s); launches++; }
            if (fdf) { launch_df_pull_batch(T(3), nf, l + 1, X.count, s); launches++; }
            launch_prolong_add_batch<double>(T(4), l, X.count, s);
            launches++;
            if (f32) { launch_d2f_batch(T(5), nf, X.count, s); launches++; }
            if (fdf) { launch_df_push_batch(T(6), nf, l + 1, X.count, s); launches++; }
        }
    }
    return launches;
}

// runs fn(ctx) for every member on host workers, each member on its worker's stream while the
// worker holds it (the contexts' own streams would put concurrent members on one hardware queue)
template <typename F>
void for_each_member(epr_batch &b, std::vector<int> &rc, F fn)
{
    const int n = (int)b.ctxs.size();
    const int threads = std::max(1, std::min(b.threads, n));
    std::vector<cudaStream_t> streams(threads, nullptr);
    for (int t = 0; t < threads; t++)
        if (cudaStreamCreateWithFlags(&streams[t], cudaStreamNonBlocking) != cudaSuccess)
        {
            streams[t] = nullptr;
            cudaGetLastError();
        }
    std::atomic<int> next{0};
    auto worker = [&](int t) {
        cudaSetDevice(b.device);
        for (int i; (i = next.fetch_add(1)) < n;)
        {
            if (rc[i] != EPR_OK) continue;
            epr_ctx *c = b.ctxs[i];
            cudaStream_t own = c->stream;
            const bool swap = streams[t] != nullptr;
            if (swap)
            {
                cudaStreamSynchronize(own);
                c->stream = streams[t];
            }
            c->status = EPR_OK;
            rc[i] = fn(c);
            // nothing of the member stays in flight, and a fault of its work is its failure
            const cudaError_t e = cudaStreamSynchronize(c->stream);
            if (e != cudaSuccess && rc[i] == EPR_OK)
            {
                c->fail(EPR_ERR_CUDA, "batch member work: %s", cudaGetErrorString(e));
                rc[i] = EPR_ERR_CUDA;
            }
            if (swap) c->stream = own;
        }
    };
    std::vector<std::thread> pool;
    for (int t = 1; t < threads; t++) pool.emplace_back(worker, t);
    worker(0);
    for (std::thread &t : pool) t.join();
    for (cudaStream_t st : streams)
        if (st) cudaStreamDestroy(st);
}

bool upload_and_capture(epr_batch &b)
{
    if (b.graph && b.image == b.captured) return true;
    if (b.graph) { cudaGraphExecDestroy(b.graph); b.graph = nullptr; }
    if (b.image.size() > b.dtabBytes)
    {
        if (b.dtab) cudaFree(b.dtab);
        b.dtab = nullptr;
        b.dtabBytes = 0;
        if (!b.ok(cudaMalloc((void **)&b.dtab, b.image.size()), "batch tables")) return false;
        b.dtabBytes = b.image.size();
    }
    if (!b.ok(cudaMemcpyAsync(b.dtab, b.image.data(), b.image.size(), cudaMemcpyHostToDevice, b.stream), "batch tables") ||
        !b.ok(cudaStreamSynchronize(b.stream), "batch tables"))
        return false;
    cudaGraph_t g = nullptr;
    if (!b.ok(cudaStreamBeginCapture(b.stream, cudaStreamCaptureModeThreadLocal), "begin capture")) return false;
    b.graphLaunches = record(b);
    cudaError_t e = cudaStreamEndCapture(b.stream, &g);
    if (!b.ok(e, "end capture")) { if (g) cudaGraphDestroy(g); return false; }
    e = cudaGraphInstantiate(&b.graph, g, 0);
    cudaGraphDestroy(g);
    if (!b.ok(e, "graph instantiate")) { b.graph = nullptr; return false; }
    b.captured = b.image;
    return true;
}

thread_local std::string g_batch_error;

}  // namespace

extern "C" {

epr_batch *epr_batch_create(epr_ctx *const *ctxs, int n, int threads)
{
    if (n <= 0 || !ctxs) { g_batch_error = "empty batch"; return nullptr; }
    for (int i = 0; i < n; i++)
    {
        if (!ctxs[i]) { g_batch_error = "null context in batch"; return nullptr; }
        for (int j = 0; j < i; j++)
            if (ctxs[j] == ctxs[i]) { g_batch_error = "a context appears twice in the batch"; return nullptr; }
        if (ctxs[i]->P.device != ctxs[0]->P.device) { g_batch_error = "the batch's contexts are on different devices"; return nullptr; }
    }
    epr_batch *b = new epr_batch();
    b->ctxs.assign(ctxs, ctxs + n);
    b->threads = threads > 0 ? threads : 8;
    b->device = ctxs[0]->P.device;
    for (int l = 0; l < kMaxLevels; l++) b->tile[l] = kDefaultTile;
    cudaSetDevice(b->device);
    if (cudaStreamCreateWithFlags(&b->stream, cudaStreamNonBlocking) != cudaSuccess || cudaEventCreate(&b->e0) != cudaSuccess ||
        cudaEventCreate(&b->e1) != cudaSuccess)
    {
        cudaGetLastError();
        g_batch_error = "cannot create the batch's stream";
        delete b;
        return nullptr;
    }
    return b;
}

void epr_batch_destroy(epr_batch *b)
{
    if (!b) return;
    cudaSetDevice(b->device);
    delete b;
}

const char *epr_batch_last_error(epr_batch *b) { return b ? b->err.c_str() : g_batch_error.c_str(); }

int epr_batch_run(epr_batch *b, int build, epr_stats *stats, int *status)
{
    if (!b) return EPR_ERR_ARG;
    cudaSetDevice(b->device);
    b->err.clear();
    const int n = (int)b->ctxs.size();
    std::vector<int> rc(n, EPR_OK);
    auto report = [&](int code) {
        int first = code;
        for (int i = 0; i < n; i++)
        {
            if (status) status[i] = rc[i];
            if (first == EPR_OK && rc[i] != EPR_OK)
            {
                first = rc[i];
                b->err = "context " + std::to_string(i) + ": " + b->ctxs[i]->err;
            }
        }
        return first;
    };
    // builds (when asked) and every member's solve prologue: levels cleared, the random start
    for_each_member(*b, rc, [&](epr_ctx *c) {
        if (build)
        {
            const int r = epr_build(c);
            if (r != EPR_OK) return r;
        }
        if (!c->have_system) { c->fail(EPR_ERR_STATE, "epr_batch_run called before epr_build"); return (int)EPR_ERR_STATE; }
        c->stats.node_updates = 0;
        c->launches = 0;
        c->stats.cycles = 0;
        c->stats.extra_sweeps = 0;
        c->stats.reached_target = 0;
        cudaEventRecord(c->ev0, c->stream);
        return c->solve_prologue() ? (int)EPR_OK : (c->status ? c->status : (int)EPR_ERR_CUDA);
    });
    if (report(EPR_OK) != EPR_OK) return report(EPR_OK);
    if (!b->ok(cudaDeviceSynchronize(), "after the member prologues")) return EPR_ERR_CUDA;
    if (!make_plan(*b)) return EPR_ERR_ARG;
    if (!upload_and_capture(*b)) return EPR_ERR_CUDA;
    cudaEventRecord(b->e0, b->stream);
    if (!b->ok(cudaGraphLaunch(b->graph, b->stream), "graph launch")) return EPR_ERR_CUDA;
    cudaEventRecord(b->e1, b->stream);
    if (!b->ok(cudaStreamSynchronize(b->stream), "batch relaxation")) return EPR_ERR_CUDA;
    // the device idle before the epilogues start, and no fault pending from any stream
    if (!b->ok(cudaDeviceSynchronize(), "after the batch relaxation")) return EPR_ERR_CUDA;
    float ms = 0;
    cudaEventElapsedTime(&ms, b->e0, b->e1);
    b->relax_ms = ms;
    // every member's epilogue: error flag, final energy, solution arrays
    for_each_member(*b, rc, [&](epr_ctx *c) {
        int64_t updates = 0;
        for (const LevelPlan &P : b->levels)
            for (size_t k = 0; k < P.members.size(); k++)
                if (b->ctxs[P.members[k]] == c) updates += (int64_t)P.iters[k] * c->levels[P.level].N;
        c->stats.node_updates = updates;
        cudaEventRecord(c->ev1, c->stream);
        if (!c->solve_epilogue()) return c->status ? c->status : (int)EPR_ERR_CUDA;
        c->stats.solve_ms = ms;  // the batch's relaxation, shared by its members
        c->stats.kernel_launches = b->graphLaunches;
        return (int)EPR_OK;
    });
    if (stats)
        for (int i = 0; i < n; i++)
            if (rc[i] == EPR_OK) stats[i] = b->ctxs[i]->stats;
    return report(EPR_OK);
}

int epr_batch_tune(epr_batch *b, int reps, double *ms_out)
{
    if (!b || reps < 1) return EPR_ERR_ARG;
    cudaSetDevice(b->device);
    if (b->levels.empty() && !make_plan(*b)) return EPR_ERR_STATE;
    // the job tables of the current plan on the device (the graph is re-captured afterwards)
    if (b->image.size() > b->dtabBytes)
    {
        if (b->dtab) cudaFree(b->dtab);
        b->dtab = nullptr;
        b->dtabBytes = 0;
        if (!b->ok(cudaMalloc((void **)&b->dtab, b->image.size()), "batch tables")) return EPR_ERR_NOMEM;
        b->dtabBytes = b->image.size();
    }
    if (!b->ok(cudaMemcpyAsync(b->dtab, b->image.data(), b->image.size(), cudaMemcpyHostToDevice, b->stream), "tables"))
        return EPR_ERR_CUDA;
    int nl = 0;
    for (const LevelPlan &P : b->levels)
    {
        if (P.tiny) continue;
        const int l = P.level;
        // save every member's coefficients (and exponents) of this level, time `reps` sweeps of
        // each shape, restore
        const size_t esz = P.type == kTypeFloat ? sizeof(float) : P.type == kTypeDouble ? sizeof(double) : sizeof(df);
        std::vector<void *> saved(P.count, nullptr), xy(P.count, nullptr);
        std::vector<int> kexpSaved;
        bool ok = true;
        for (int k = 0; ok && k < P.count; k++)
        {
            Context *c = b->ctxs[P.members[k]];
            Level &L = c->levels[l];
            xy[k] = P.type == kTypeFloat ? (void *)L.xy32 : P.type == kTypeDouble ? (void *)L.xy64 : (void *)L.xyd;
            ok = b->ok(cudaMallocAsync(&saved[k], esz * 2 * L.N, b->stream), "tune scratch") &&
                 b->ok(cudaMemcpyAsync(saved[k], xy[k], esz * 2 * L.N, cudaMemcpyDeviceToDevice, b->stream), "tune save");
        }
        std::vector<std::vector<int>> kx(P.count);
        for (int k = 0; ok && k < P.count && P.type == kTypeDF; k++)
        {
            Context *c = b->ctxs[P.members[k]];
            kx[k].resize(c->depth + 1);
            ok = b->ok(cudaMemcpyAsync(kx[k].data(), c->d_kexp, sizeof(int) * (c->depth + 1), cudaMemcpyDeviceToHost, b->stream), "tune save");
        }
        ok = ok && b->ok(cudaStreamSynchronize(b->stream), "tune save");
        double best = 1e300;
        int bestTile = kDefaultTile;
        for (int t = 0; ok && t < 3; t++)
        {
            auto sweep = [&](auto tag) {
                using Real = decltype(tag);
                const BatchJob<Real> *jobs = reinterpret_cast<const BatchJob<Real> *>(b->dtab + P.off);
                for (int c = 0; c < 8; c++) launch_colour_batch<Real>(jobs, l, c, P.count, t, b->stream);
            };
            auto one = [&]() {
                if (P.type == kTypeFloat) sweep(float());
                else if (P.type == kTypeDouble) sweep(double());
                else sweep(df());
            };
            one();  // warm-up
            cudaEventRecord(b->e0, b->stream);
            for (int r = 0; r < reps; r++) one();
            cudaEventRecord(b->e1, b->stream);
            ok = b->ok(cudaStreamSynchronize(b->stream), "tune");
            float ms = 0;
            cudaEventElapsedTime(&ms, b->e0, b->e1);
            if (ms_out) ms_out[3 * nl + t] = ms / reps;
            if (ms < best) { best = ms; bestTile = t; }
        }
        for (int k = 0; k < P.count; k++)
        {
            Context *c = b->ctxs[P.members[k]];
            if (saved[k])
            {
                ok = b->ok(cudaMemcpyAsync(xy[k], saved[k], esz * 2 * c->levels[l].N, cudaMemcpyDeviceToDevice, b->stream), "tune restore") && ok;
                cudaFreeAsync(saved[k], b->stream);
            }
            if (P.type == kTypeDF && !kx[k].empty())
                ok = b->ok(cudaMemcpyAsync(c->d_kexp, kx[k].data(), sizeof(int) * kx[k].size(), cudaMemcpyHostToDevice, b->stream), "tune restore") && ok;
        }
        ok = ok && b->ok(cudaStreamSynchronize(b->stream), "tune restore");
        if (!ok) return EPR_ERR_CUDA;
        b->tile[l] = bestTile;
        nl++;
    }
    if (b->graph) { cudaGraphExecDestroy(b->graph); b->graph = nullptr; }
    return EPR_OK;
}

int epr_batch_set_tile(epr_batch *b, int level, int tile)
{
    if (!b) return EPR_ERR_ARG;
    if (tile < 0 || tile > 2 || level < -1 || level >= kMaxLevels)
    {
        b->err = "block shape index 0-2 of a level 0-15 (or -1 for all)";
        return EPR_ERR_ARG;
    }
    for (int l = 0; l < kMaxLevels; l++)
        if (level < 0 || l == level) b->tile[l] = tile;
    if (b->graph) { cudaGraphExecDestroy(b->graph); b->graph = nullptr; }
    return EPR_OK;
}

int epr_batch_info(epr_batch *b, int *tiles, int cap, double *relax_ms, long long *launches)
{
    if (!b) return EPR_ERR_ARG;
    if (tiles)
        for (int l = 0; l < cap && l < kMaxLevels; l++) tiles[l] = b->tile[l];
    if (relax_ms) *relax_ms = b->relax_ms;
    if (launches) *launches = (long long)b->graphLaunches;
    return EPR_OK;
}

}  // extern "C"
