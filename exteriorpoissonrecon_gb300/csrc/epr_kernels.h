// Host-side declarations of the CUDA launchers (instantiated for Dim 3/4 and double/float in
// epr_solve.cu and epr_setup.cu).  Only plain pointers and sizes cross this header.
#pragma once
#include <cstddef>
#include <cstdint>
#include <cuda_runtime.h>

#include "epr_df.cuh"

namespace epr {

// One level of the hierarchy as the solve kernels see it.
template <typename Real>
struct LevelPtrs
{
    int level = 0;
    int64_t N = 0;            // nodes
    Real *xy = nullptr;       // 2N interleaved (x, y)
    const Real *A = nullptr;  // 3^Dim * N column stencil of R + dWeight K (offset-major)
    const Real *B = nullptr;  // 3^Dim * N column stencil of the frame constraint
    const Real *Acb = nullptr;  // optional colour-blocked copies of A and B (colour_block_base)
    const Real *Bcb = nullptr;
    // adaptive indexer: per node 0 (no function), 1 (indexed, held fixed), 2 (active); the
    // Gauss-Seidel kernels update active nodes only.  Null for the regular grid (all active).
    const uint8_t *status = nullptr;
    // adaptive indexer: the active nodes of every parity colour as colour-local indices (the
    // Colour::node order), colour c at alist[aoff[c] .. aoff[c+1]); the large levels relax these
    // lists instead of the whole colour.  Null for the regular grid.
    const int *alist = nullptr;
    int aoff[17] = {0};
};

// Scratch for deterministic two-pass reductions
struct Reduce
{
    double *partial = nullptr;  // >= kMaxBlocks * 4 doubles
    double *out = nullptr;      // >= 4 doubles
    static constexpr int kMaxBlocks = 4096;
};

template <int D, typename Real>
void launch_energy(const LevelPtrs<Real> &L, const Real *xy, const Reduce &red, cudaStream_t s);
// red.out[0] = sum_i (dE/dx_i)^2 + (dE/dy_i)^2
template <int D, typename Real>
void launch_grad_norm(const LevelPtrs<Real> &L, const Real *xy, const Reduce &red, cudaStream_t s);
// writes N x 5 doubles (Q20, Q02, Q11, Q10, Q01)
template <int D, typename Real>
void launch_quadfit(const LevelPtrs<Real> &L, const Real *xy, double *out, cudaStream_t s);
// separate != 0: the reference's SeparateGaussSeidelSolve update (x first, then y with the new x)
template <int D, typename Real>
void launch_gs_colour(const LevelPtrs<Real> &L, int colour, unsigned int *err, cudaStream_t s, int separate = 0);
// selects the colour-kernel variant (0: one thread per node, 1: 2^D lanes per node on a row grid,
// 2: 2^D lanes per node on a flat grid; 1 is the default, 0.69 ms against 0.70 ms at depth 8;
// 4: as 1 without the point-split update of the small 3D levels)
void set_gs_variant(int v);
void set_lanes_variant(int v);
// 1 (default): 3D levels 0-1 relax in gs_tiny_kernel (one warp per node-element incidence of a
// colour); 0: in the block kernels
void set_tiny_levels(int v);
// 3D level 2 in double-float on one cluster launch (1; 8 or 16 fix the cluster size) or a launch
// per colour (0, the default)
void set_cluster_levels(int v);
bool cluster_level(int level, bool isDF);
// double-float levels: pairs stored as x 2^-k with k = kexp[level] (epr_df.cuh)
void launch_df_push(const double *in, df *out, int64_t n, int *kexp, int level, cudaStream_t s);
void launch_df_pull(const df *in, double *out, int64_t n, const int *kexp, int level, cudaStream_t s);
void launch_d2df(const double *in, df *out, int64_t n, cudaStream_t s);
int launch_gs_sweeps_df(const LevelPtrs<df> &L, int iters, unsigned int *err, cudaStream_t s, int separate,
                        int64_t persistentMaxNodes, int *kexp);
void launch_gs_colour_df(const LevelPtrs<df> &L, int colour, unsigned int *err, cudaStream_t s, int *kexp);
// iters full sweeps (all 2^D colours in order); levels of at most persistentMaxNodes nodes run all
// sweeps inside one thread block, larger ones launch one kernel per colour.  Returns the number of
// kernels launched.
constexpr int64_t kPersistentMaxNodes = 729;
template <int D, typename Real>
int launch_gs_sweeps(const LevelPtrs<Real> &L, int iters, unsigned int *err, cudaStream_t s, int separate = 0,
                     int64_t persistentMaxNodes = kPersistentMaxNodes);
// sets the shared-memory carve-out of the single-block level kernels (once per process, before
// any stream capture)
void prepare_gs_kernels();
template <int D, typename Real>
void launch_gn_matvec(const LevelPtrs<Real> &L, const Real *xy, const Real *dxy, Real *out, cudaStream_t s);
// fine (2 N_f) = P coarse (2 N_c), pairs; add != 0 accumulates
template <int D, typename Real>
// fineStatus (adaptive indexer): fine nodes without a function (status 0) stay zero
void launch_prolong(int coarseLevel, const Real *coarse, Real *fine, int add, cudaStream_t s,
                    const uint8_t *fineStatus = nullptr);
// coarse = P^T fine, pairs
template <int D, typename Real>
void launch_restrict(int coarseLevel, const Real *fine, Real *coarse, cudaStream_t s);

// coarse = P^T fine P of a column stencil (offset-major, double), fine level -> fineLevel - 1
template <int D>
void launch_galerkin(int fineLevel, const double *Mf, double *Mc, cudaStream_t s);

// colour-blocked copy (Real) of a natural offset-major double stencil of `level`
template <int D, typename Real>
void launch_to_colour_blocks(int level, const double *M, Real *out, cudaStream_t s);

// elementwise helpers
template <typename Real>
void launch_scale(Real *v, int64_t n, double s, cudaStream_t st);
template <typename Real>
void launch_axpy(Real *y, const Real *x, int64_t n, double a, cudaStream_t st);
void launch_convert_d2f(const double *in, float *out, int64_t n, cudaStream_t st);
// interleaved (x, y) pairs <-> two planar arrays
void launch_split_pairs(const double *xy, double *x, double *y, int64_t n, cudaStream_t st);
void launch_merge_pairs(const double *x, const double *y, double *xy, int64_t n, cudaStream_t st);
void launch_convert_f2d(const float *in, double *out, int64_t n, cudaStream_t st);

// ---------------------------------------------------------------------------------------------
// Lockstep batches (3D): one launch relaxes the same level and colour of many reconstructions,
// each with its own arrays, sweep count and error flag.  Every reconstruction's nodes see exactly
// the arithmetic of its own solve's kernels for that level, so the batch gives each one its own
// solve's bits.
// ---------------------------------------------------------------------------------------------
template <typename Real>
struct BatchJob
{
    LevelPtrs<Real> L;
    unsigned int *err = nullptr;
    int *kexp = nullptr;  // the reconstruction's exponent table (double-float levels), else null
    int iters = 0;        // sweeps of this level
    int separate = 0;
};
// a level-to-level transfer of one reconstruction: src and dst arrays of the transfer's types
struct XferJob
{
    const void *src = nullptr;
    void *dst = nullptr;
    int *kexp = nullptr;
};
// the colour kernels' block shapes a batch may pick (none changes any node's arithmetic):
// levels whose colours have at most 125 nodes: nodes per block of the point-split kernel;
// larger levels: threads per block of the lane kernel (8 lanes per node)
constexpr int kSplitTiles[3] = {1, 2, 4};
constexpr int kLanesTiles[3] = {64, 128, 256};
constexpr int kDefaultTile = 1;  // index into the tables: the solo solve's shapes (2 nodes, 128 threads)
// all sweeps of 3D level 0 or 1 of `count` reconstructions (jobs[0..count))
template <typename Real>
void launch_tiny_batch(const BatchJob<Real> *jobs, int level, int count, cudaStream_t s);
// one colour of a level >= 2 of jobs[0..count) with the block shape kSplitTiles / kLanesTiles[tile]
template <typename Real>
void launch_colour_batch(const BatchJob<Real> *jobs, int level, int colour, int count, int tile, cudaStream_t s);
// a new exponent for each double-float level of jobs[0..count) (once per sweep)
void launch_df_rescale_batch(const BatchJob<df> *jobs, int count, cudaStream_t s);
// fine += P coarse for jobs[0..count) (src coarse, dst fine)
template <typename Real>
void launch_prolong_add_batch(const XferJob *jobs, int coarseLevel, int count, cudaStream_t s);
// elementwise n values: float -> double, double -> float, double-float -> double (the exponent of
// `level`), double -> double-float (a new exponent for `level`, one block per reconstruction)
void launch_f2d_batch(const XferJob *jobs, int64_t n, int count, cudaStream_t s);
void launch_d2f_batch(const XferJob *jobs, int64_t n, int count, cudaStream_t s);
void launch_df_pull_batch(const XferJob *jobs, int64_t n, int level, int count, cudaStream_t s);
void launch_df_push_batch(const XferJob *jobs, int64_t n, int level, int count, cudaStream_t s);

}  // namespace epr
