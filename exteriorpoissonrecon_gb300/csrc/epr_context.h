// Internal state of one epr_ctx (see include/epr.h).  Host code only.
#pragma once
#include <cstdint>
#include <string>
#include <vector>

#include <cuda_runtime.h>

#include "../../include/epr.h"
#include "epr_kernels.h"

namespace epr {

struct Context;
struct MGHierarchy;

// Device storage of one level of the hierarchy.
struct Level
{
    int64_t N = 0;
    double *xy64 = nullptr;   // interleaved (x, y), regular coefficients
    double *A64 = nullptr;    // R + dWeight K, column stencil, offset-major
    double *B64 = nullptr;    // frame constraint, column stencil, offset-major
    double *tmp64 = nullptr;  // hierarchical solution after a solve
    float *xy32 = nullptr;    // float copies used when precision == EPR_FP32
    float *A32 = nullptr;
    float *B32 = nullptr;
    float *tmp32 = nullptr;
    void *Acb = nullptr;      // colour-blocked A and B in the level's precision (levels relaxed
    void *Bcb = nullptr;      // by one kernel per colour)
    df *xyd = nullptr;        // double-float copies of a coarse band level (coefficients stored
    df *Ad = nullptr;         // as x 2^-k, k = d_kexp[level]; stencils unscaled)
    df *Bd = nullptr;
};

// Sample-side state of the build (ordered sampling, estimator, splats).  Defined in epr_setup.cu.
struct Setup
{
    size_t n = 0;               // samples
    int64_t ncells = 0;         // occupied finest cells
    double *pos = nullptr;      // n x dim, unit cube
    double *skew = nullptr;     // n x K packed frames
    int *order = nullptr;       // samples sorted by cell (Morton order of the cell, stable)
    int64_t *cellKey = nullptr; // Morton key of each occupied cell
    int *cellStart = nullptr;   // ncells + 1
    int *cellOfFinest = nullptr;// dense map finest cell -> occupied index or -1
    double *measure = nullptr, *noise = nullptr, *sdepth = nullptr;  // per sample
    double *S = nullptr;        // finest elements x K
    int *leaf = nullptr;        // leaf tree depth per finest element
    std::vector<double *> density, skewGrid;  // per tree level
    std::vector<uint8_t *> refinedD, refinedS; // per tree depth

    bool set_samples(Context &c, size_t n, const double *pos, const double *skew);
    // takes device arrays allocated on the context's stream (generated samples) as its own
    bool set_samples_device(Context &c, size_t n, double *dpos, double *dskew);
    bool build(Context &c);
    bool get(Context &c, const std::string &name, double *out, size_t cap, size_t *count);
    void release_built(Context &c);
    void release(Context &c);
};

// One level of the adaptive indexer (Hat::HierarchicalAdaptedIndexer) on the level's dense grid
struct AdaptiveLevel
{
    uint8_t *status = nullptr;   // per node: 0 no function, 1 indexed (held fixed), 2 active
    int64_t *fnodes = nullptr;   // node of every function index (active ones first)
    int64_t *enodes = nullptr;   // element of every element index
    int64_t nF = 0, nA = 0, nE = 0;
    int *clist = nullptr;        // active nodes of every parity colour (colour-local indices)
    int coff[17] = {0};          // colour c at clist[coff[c] .. coff[c+1])
};

struct Context
{
    int dim = 0, depth = 0;
    epr_params P{};
    std::string err;
    int status = 0;
    cudaStream_t stream = nullptr;
    cudaEvent_t ev0 = nullptr, ev1 = nullptr;
    std::vector<Level> levels;
    Reduce red;
    unsigned int *d_err = nullptr;
    int *d_kexp = nullptr;  // per level: power-of-two exponent of a double-float level
    double *d_fit = nullptr;
    double c = 0;
    bool have_system = false;
    bool solved = false;
    epr_stats stats{};
    int64_t launches = 0;  // kernels launched since the last epr_solve started
    // fault injection: device bytes this context may allocate in total (0 = no cap), from the
    // EPR_ALLOC_CAP_BYTES environment variable at epr_create; allocations beyond it fail as an
    // out-of-memory would (EPR_ERR_NOMEM)
    size_t alloc_cap = 0, alloc_total = 0;
    Setup setup;
    // the adaptive indexer's levels (empty for the regular grid), built with the system
    std::vector<AdaptiveLevel> adapt;
    uint8_t *elem_indexed = nullptr;  // finest level: 1 for the elements the indexer holds
    // adaptive levels relax per-colour lists of their active nodes (EPR_ADAPTIVE_LISTS=0 at context
    // creation: every node of the colour, the inactive ones skipped; the same bits)
    bool adaptive_lists = true;
    const uint8_t *status_of(int l) const { return adapt.empty() ? nullptr : adapt[l].status; }
    void release_adaptive();
    MGHierarchy *mg = nullptr;  // linear multigrid storage (epr_mg.cu), allocated on first use
    // the relaxation sequence of the cascadic solve captured as one CUDA graph (built on the first
    // solve, replayed by the next ones), with the host-side counts of what it launches
    cudaGraphExec_t solve_graph = nullptr;
    int64_t graph_launches = 0, graph_updates = 0;
    int solves_done = 0;

    virtual ~Context();
    void fail(int code, const char *fmt, ...);
    bool cuda_ok(cudaError_t e, const char *what);
    bool launch_ok(const char *what);
    bool alloc(void **p, size_t bytes, const char *what);
    void release(void *p);
    int64_t nodes(int level) const;
    int stencil() const;
    bool ensure_level(int l);
    bool lvl32(int l) const;  // level l computes in float
    bool lvlDF(int l) const;  // level l computes in double-float (a 3D coarse band level)
    bool sync_system32(int l);
    bool push_xy(int l);
    bool pull_xy(int l);
    bool energy(int l, double *out3);
    bool gs(int l, int iters, int64_t persistentMaxNodes = kPersistentMaxNodes);
    bool relax_levels(int minD, int maxD, bool useGraph);
    bool check_errors();
    bool prolong_add(int l);
    bool upload_xy(int l, const double *x, const double *y);
    bool download_xy(int l, double *x, double *y, bool fromSolution);
    bool solve_cascadic();
    bool solve_prologue();  // levels cleared, the random start (solve_cascadic's first part)
    bool solve_epilogue();  // error flag, timing, final energy, solution arrays (after ev1)
    // the reference's random start on `level` (rand() pairs after srand(seed), scaled by the fourth
    // root of c over the wedge square norm, ExteriorPoisson.h:333-341), set as the level's
    // coefficients; *energy (may be null) receives its total energy
    bool random_start(int level, double *energy);
};

// the arrays of level l as the solve kernels of arithmetic Real see them (the colour-blocked
// stencil copies only where the level relaxes in that arithmetic)
template <typename Real>
inline LevelPtrs<Real> level_ptrs(Context *c, int l)
{
    Level &L = c->levels[l];
    LevelPtrs<Real> p;
    p.level = l;
    p.N = L.N;
    if (!c->adapt.empty())
    {
        const AdaptiveLevel &A = c->adapt[l];
        p.status = A.status;
        p.alist = c->adaptive_lists ? A.clist : nullptr;
        for (int k = 0; k <= (1 << c->dim); k++) p.aoff[k] = A.coff[k];
    }
    if constexpr (std::is_same<Real, double>::value) { p.xy = L.xy64; p.A = L.A64; p.B = L.B64; }
    else if constexpr (std::is_same<Real, df>::value) { p.xy = L.xyd; p.A = L.Ad; p.B = L.Bd; return p; }
    else { p.xy = L.xy32; p.A = L.A32; p.B = L.B32; }
    if (L.Acb && c->lvl32(l) == std::is_same<Real, float>::value)
    {
        p.Acb = (const Real *)L.Acb;
        p.Bcb = (const Real *)L.Bcb;
    }
    return p;
}

// the adaptive indexer's tables of every level (epr_adaptive.cu), from the finest cell map
bool build_adaptive(Context &c, const int *cellOfFinest);
// has-children flags of the adaptive indexer's tree per tree depth (0 .. depth + 1)
bool adaptive_tree_refinement(Context &c, std::vector<std::vector<uint8_t>> &refined);
// a copy of the finest frame field with the elements outside the adaptive indexer zeroed
bool masked_frames(Context &c, const double *S, int64_t nElements, int K, double **out);

// the text epr_global_error() returns (per host thread)
void set_global_error(const std::string &msg);

// A64[level] += dWeight K (the Dirichlet stiffness of the level, with the reference's
// resolution-1 stencil table, see epr_setup.cu)
bool add_dirichlet(Context &c, int level);
bool add_dirichlet_to(Context &c, int level, double *dst, double w);

}  // namespace epr

// the C ABI's opaque handle is the context itself
struct epr_ctx : public epr::Context
{
};
