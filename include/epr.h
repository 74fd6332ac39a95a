/* libepr_cuda: the GB300 (sm_103a) implementation of ExteriorPoissonRecon's regular-grid solve path.
 *
 * C ABI: plain pointers and sizes only, every call returns an int status (EPR_OK = 0), no
 * exception crosses the boundary, and epr_last_error() describes the last failure of a context.
 * One context = one reconstruction problem = one CUDA stream on the current device; a context is
 * not thread-safe.  Host arrays are ordinary (pageable or pinned) host memory unless a function
 * says "device".
 *
 * Reference interfaces replaced (paths relative to the reference checkout):
 *   epr_create / epr_set_samples / epr_build
 *       ExteriorPoisson::Reconstructor::Reconstructor      ExteriorPoissonRecon/ExteriorPoisson.h:59-72,126-313
 *       (OrderedSampler OrderedSamples.h, TreeEstimator GridSamples.h:232-277 and the
 *        SingleCycleCascadicSystemEnergy constructor / restrict SystemEnergy.h:135-141,447-477)
 *   epr_solve
 *       ExteriorPoisson::Reconstructor::solve              ExteriorPoisson.h:74-81,315-409
 *   epr_get_solution
 *       Reconstructor::x() / y()                            ExteriorPoisson.h:83-86
 *   epr_energy
 *       SystemEnergy::energies / operator()                 Include/SystemEnergy.h:63,91,486-497
 *   epr_quadfit
 *       SystemEnergy::quadraticFit                          Include/SystemEnergy.h:75,542-643
 *   epr_gradient
 *       SystemEnergy::d                                     Include/SystemEnergy.h:72,248-254
 *   epr_gs
 *       ExteriorPoissonSolvers::PairedGaussSeidelSolve      ExteriorPoissonRecon/ExteriorPoissonSolvers.h:74-76,156-196
 *   epr_prolong
 *       SystemEnergy::prolongation                          Include/SystemEnergy.h:99-100,162
 *   epr_gn_matvec
 *       the matrix of SystemEnergy::quadraticApproximation1/2 applied to a vector
 *                                                           Include/SystemEnergy.h:80-84 (q.q * x, MG.h:120)
 *   epr_linear_gs
 *       GSRelaxer::operator()(b, x, mcIndices)              Include/MG.h:39-72
 *   epr_mg_vcycle
 *       MGSolver::MGSolver + vCycle                         Include/MG.h:74-187
 *   epr_alternating_system
 *       quadraticApproximation1/2 as AlternatingSolve uses them (q.q *= 2, q.l = -q.l)
 *                                                           ExteriorPoissonRecon/ExteriorPoissonSolvers.h:96-131
 *   epr_alternating_solve
 *       ExteriorPoissonSolvers::AlternatingSolve            ExteriorPoissonSolvers.h:66-68,86-154
 *   epr_biquadratic_fit
 *       SystemEnergy::biQuadraticFit                        Include/SystemEnergy.h:78,499-540
 *   epr_step_size / epr_newton_update
 *       SystemEnergy::stepSize / newtonUpdate               Include/SystemEnergy.h:66-69,256-303
 *   epr_batch_solve, epr_batch_create / run / tune / info / destroy
 *       no reference counterpart: the reference reconstructs one input per process; these run
 *       Reconstructor::Reconstructor + solve (ExteriorPoisson.h:59-81) for many inputs at once
 *   epr_generate_samples / epr_set_generated_samples
 *       the Sample tool's shapes and noise              Include/Samples.h, Sample/Sample.cpp:137-199
 *   epr_get_density / epr_get_density_refined
 *       the density estimator's tree data and structure: TreeEstimator (GridSamples.h:232-277,
 *       DensityAndNoiseInfo GridSamples.h:79-94)
 *   epr_write_density_tree
 *       the <out>.density.tree file: ExteriorPoissonRecon.cpp:272-277 with TreeEstimator::write
 *       (GridSamples.inl:734-738) and RegularTreeNode::write (Misha/RegularTree.inl:615-642)
 *   epr_write_tree
 *       the <out>.tree file: ExteriorPoissonRecon.cpp:259-270 with HierarchicalRegularIndexer::write
 *       (Hat.adaptive.inl:198-203) or HierarchicalAdaptedIndexer::write (Hat.adaptive.inl:399-405)
 *   epr_get_regular_coefficients
 *       BaseHierarchicalIndexer::regularCoefficients        Include/Hat.adaptive.inl:154-176
 *   epr_get_adaptive_index
 *       HierarchicalAdaptedIndexer's tables: numFunctions / numActiveFunctions / numElements,
 *       functionIndex / elementIndex (Hat.adaptive.h:238-328, Hat.adaptive.inl:415-450)
 *   epr_get_array
 *       read-only views of the reference's internal state (TreeEstimator::measure/noise/depth
 *       GridSamples.inl:838-862, S(E) ExteriorPoisson.h:290-307, _R/_B SystemEnergy.h:172-175)
 *   epr_conv3*, epr_unet_*
 *       no reference counterpart: the learned warm start replaces the reference's random initial
 *       guess (ExteriorPoisson.h:333-341) and the coarse levels of its cascadic schedule
 */
#ifndef EPR_H
#define EPR_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define EPR_OK 0
#define EPR_ERR_ARG (-1)      /* invalid argument (sizes, level, null pointer) */
#define EPR_ERR_CUDA (-2)     /* a CUDA runtime call failed */
#define EPR_ERR_STATE (-3)    /* call out of order (e.g. solve before build) */
#define EPR_ERR_NUMERIC (-4)  /* a kernel produced a non-finite value */
#define EPR_ERR_NOMEM (-5)    /* device allocation failed (or exceeded the cap that the environment variable
                                 EPR_ALLOC_CAP_BYTES, read at epr_create, sets on a context's total
                                 allocations: fault injection for out-of-memory handling) */

#define EPR_FP64 0  /* all arithmetic in double (parity with the reference to 1e-12) */
#define EPR_FP32 1  /* smoothing / matvecs in float; energies, norms and the coarse solve in double */

#define EPR_BAND_FP64 0  /* the double band of EPR_FP32 in double */
#define EPR_BAND_DF 1    /* its 3D levels up to 3 in double-float */
#define EPR_SOLVER_CASCADIC 0   /* the reference schedule: coarse-to-fine paired Gauss-Seidel */
#define EPR_SOLVER_MULTIGRID 1  /* cascadic, each level relaxed by the alternating solve with linear
                                   multigrid V-cycles (AlternatingSolve, sType MULTIGRID) */

typedef struct epr_ctx epr_ctx;

typedef struct epr_params {
    double s_weight;      /* --sWeight   screening weight (code default 100) */
    double d_weight;      /* --dWeight   Dirichlet weight (0.00625) */
    double n_sigma;       /* --nSigma    noise-to-weight sigma (0.25) */
    double i_mult;        /* --iMult     iteration multiplier per level (2) */
    int t_radius;         /* --tRadius   frame splat kernel radius, 0..4 (1) */
    int d_radius;         /* --dRadius   density kernel radius, 0..4 (1) */
    int gs_iters;         /* --gsIters   Gauss-Seidel iterations at the finest level (10) */
    int min_solve_depth;  /* --minSolveDepth (0) */
    int max_solve_depth;  /* --maxSolveDepth (-1 = depth) */
    unsigned int seed;    /* --seed      initial-guess seed (0) */
    int precision;        /* EPR_FP64 or EPR_FP32 */
    int solver;           /* EPR_SOLVER_CASCADIC or EPR_SOLVER_MULTIGRID */
    double tolerance;     /* multigrid: stop when |grad E| / |grad E(x0)| <= tolerance (1e-6) */
    int max_cycles;       /* multigrid: cycle cap (200) */
    int verbose;          /* print the reference's per-level "Error[...]" lines */
    int device;           /* CUDA device ordinal the context runs on (0) */
    int fp64_levels;      /* EPR_FP32 only: levels fp64_from .. fp64_levels-1 still run in double (0) */
    int single_level;     /* --singleLevel: prolong the initial guess and relax only the finest solve level */
    int separate;         /* --separate: update x then y per node instead of the paired 2x2 step */
    int fp64_from;        /* EPR_FP32 only: first level of the double band (0) */
    int band_precision;   /* EPR_FP32 only: EPR_BAND_FP64 (0) runs the band in double; EPR_BAND_DF runs
                             its 3D levels up to 3 in double-float (pairs of floats, 48 bits, on the
                             FP32 pipe, with a power-of-two exponent per level) and the rest in double;
                             cascadic solver only */
    int warm_start;       /* 1: the solve starts from the coefficients already set on level minSolveDepth
                             (epr_set_coefficients or epr_unet_warm_start) instead of the reference's
                             random start (0) */
    int max_extra_sweeps; /* with target_energy: cap on the finest-level sweeps added after the schedule (0) */
    double target_energy; /* > 0: after the schedule the finest solve level keeps relaxing, one paired
                             Gauss-Seidel sweep at a time, until its FP64 energy is <= target_energy or
                             max_extra_sweeps were added; the energy checks are part of the timed solve (0) */
    int project;          /* --project: every element's S(E) projected onto its best blade before the
                             constraint is built (FitBlade, ExteriorPoisson.h:300-305, 411-438) (0) */
    int adaptive_radius;  /* --aRadius: -1 the regular grid (HierarchicalRegularIndexer); 0..5 the
                             adaptive indexer (HierarchicalAdaptedIndexer, ExteriorPoissonRecon.cpp:
                             183-198, Hat.adaptive.inl:342-732): only the functions within that many
                             cells of a sample's cell (at every level) are relaxed, the ones a step
                             further are held at their prolonged values, all others are zero; the
                             constraint and c integrate the elements it holds.  Cascadic solver,
                             no warm start (-1) */
} epr_params;

typedef struct epr_stats {
    double initial_energy;   /* E0 = squareNorm of the target (the reference's "_err") */
    double fit_energy;       /* final fitting term */
    double reg_energy;       /* final regularisation term */
    double solve_ms;         /* device time of the solve (CUDA events) */
    double build_ms;         /* device time of epr_build */
    double grad_norm0;       /* multigrid: |grad E| at the start of the finest level */
    double grad_norm;        /* multigrid: |grad E| at exit */
    int cycles;              /* multigrid cycles run */
    int64_t node_updates;    /* paired Gauss-Seidel node updates performed */
    int64_t kernel_launches; /* kernels this library launched during the solve */
    int extra_sweeps;        /* finest-level sweeps added to reach target_energy */
    int reached_target;      /* 1 when the final energy is <= target_energy (0 without a target) */
} epr_stats;

void epr_default_params(epr_params *p);

/* Context for a dim (3 or 4) reconstruction at the given depth (1..10 in 3D, 1..7 in 4D).
 * Returns NULL on error; epr_global_error() then describes it. */
epr_ctx *epr_create(int dim, int depth, const epr_params *params);
void epr_destroy(epr_ctx *ctx);
const char *epr_last_error(const epr_ctx *ctx);
const char *epr_global_error(void);

/* Samples in the unit cube (n x dim doubles) with their packed skew frames
 * (n x dim(dim-1)/2 doubles, entry i(i-1)/2 + j holds (m(i,j) - m(j,i))/2 for i > j). */
int epr_set_samples(epr_ctx *ctx, size_t n, const double *pos, const double *skew);

/* Ordered sampling, density estimation, frame splatting, S(E), screening / constraint /
 * Dirichlet stencils and the Galerkin hierarchy, all on the device. */
int epr_build(epr_ctx *ctx);

/* Replaces the system of one level with host column stencils: R (screening) and B (constraint)
 * with 3^dim entries per node (entry o of node i holds M(i+off(o), i)), plus the constant c. */
int epr_set_level_system(epr_ctx *ctx, int level, const double *R, const double *B, double c);

/* Coefficients of one level (regular, not hierarchical), host arrays of (2^level+1)^dim doubles. */
int epr_set_coefficients(epr_ctx *ctx, int level, const double *x, const double *y);
int epr_get_coefficients(epr_ctx *ctx, int level, double *x, double *y);

/* out[0] = fitting energy, out[1] = regularisation energy, out[2] = wedge square norm, for the
 * level's current coefficients. */
int epr_energy(epr_ctx *ctx, int level, double *out3);
/* Quadratic fit of every node (N x 5: Q20, Q02, Q11, Q10, Q01). */
int epr_quadfit(epr_ctx *ctx, int level, double *out);
/* Energy gradient (dE/dx, dE/dy). */
int epr_gradient(epr_ctx *ctx, int level, double *gx, double *gy);
/* iters paired Gauss-Seidel sweeps over the 2^dim parity colours, in place. */
int epr_gs(epr_ctx *ctx, int level, int iters);
/* coefficients[level+1] += P coefficients[level] */
int epr_prolong(epr_ctx *ctx, int level);
/* (J^T J + A)(dx, dy) at the level's current coefficients: J is the linearised wedge residual,
 * A = R + dWeight K.  This is half the Gauss-Newton Hessian of the energy. */
int epr_gn_matvec(epr_ctx *ctx, int level, const double *dx, const double *dy, double *ox, double *oy);

/* Runs the configured solver; stats may be NULL. */
int epr_solve(epr_ctx *ctx, epr_stats *stats);
/* Builds (build != 0) and solves n independent reconstructions concurrently on one GPU: `threads`
 * host threads (<= 0: 8) each take whole reconstructions, largest first, and drive each one on a
 * non-blocking stream the worker owns (created together, so that concurrent workers sit on
 * distinct hardware work queues), so their kernels overlap on the device.  A context's own stream
 * is synchronised before the worker takes the context over and gets the context back afterwards;
 * when the call returns nothing is in flight on either stream.  The contexts must be distinct and
 * on the same device; they may differ in dim, depth, samples and parameters, and each computes
 * exactly what epr_build + epr_solve compute for it alone.  stats[i] and status[i] (either may be
 * NULL) receive context i's statistics and return code.  Returns EPR_OK, or the code of the first
 * failing context in index order (epr_global_error() names it).  The contexts must not be used by
 * other threads meanwhile. */
int epr_batch_solve(epr_ctx *const *ctxs, int n, int build, int threads, epr_stats *stats, int *status);

/* Lockstep batch of 3D reconstructions: the cascadic schedule of every member advances level by
 * level, and each level's relaxation is a few launches for all members together (levels 0-1: one
 * block per member for all its sweeps; from level 2 on one launch per sweep and colour whose grid
 * spans the colour's nodes of every member still sweeping that level).  The whole relaxation is
 * one CUDA graph, captured on the first epr_batch_run and replayed while the members' arrays stay
 * where they are.  Members may differ in depth, samples, sweep counts and parameters, but must run
 * the plain cascadic schedule (no multigrid, single level, verbose, warm start or target energy),
 * share the minimum solve depth and relax each level in the same arithmetic; every member gets
 * exactly the bits of its own epr_solve.  The contexts must be distinct, on one device, and not be
 * used elsewhere while the batch runs.  NULL on failure (epr_batch_last_error(NULL)). */
typedef struct epr_batch epr_batch;
epr_batch *epr_batch_create(epr_ctx *const *ctxs, int n, int threads);
/* Builds (build != 0) every member, then solves them all: member prologues (levels cleared, random
 * start) and epilogues (error flags, final energies, solution arrays) on `threads` host workers,
 * the relaxation as the batch's graph.  stats[i].solve_ms is the batch relaxation's device time,
 * shared by all members.  stats / status as for epr_batch_solve. */
int epr_batch_run(epr_batch *b, int build, epr_stats *stats, int *status);
/* The autotuner: for every level relaxed by per-colour launches, times `reps` sweeps of all members
 * in each of the three block shapes of its colour kernel (levels whose colours have at most 125
 * nodes: 1, 2 or 4 nodes per block of the point-split kernel; larger levels: 64, 128 or 256 threads
 * per block of the lane kernel) on the members' current coefficients, which it restores, and keeps
 * the fastest shape per level for the next runs.  No shape changes any node's arithmetic.  ms_out
 * (may be NULL) receives 3 mean sweep times per tuned level, coarsest first.  Needs built members. */
int epr_batch_tune(epr_batch *b, int reps, double *ms_out);
/* Sets level's block shape index (0-2; level -1: every level) by hand, in place of the tuner's. */
int epr_batch_set_tile(epr_batch *b, int level, int tile);
/* tiles[l] (l < cap): the block shape index (0-2) level l uses; relax_ms: the last run's relaxation
 * time; launches: kernel launches in the batch's graph. */
int epr_batch_info(epr_batch *b, int *tiles, int cap, double *relax_ms, long long *launches);
void epr_batch_destroy(epr_batch *b);
const char *epr_batch_last_error(epr_batch *b);

/* Synthetic samples generated on the device (the reference's Sample tool: Include/Samples.h shapes,
 * Sample/Sample.cpp:137-199 noise).  Random numbers: Philox4x32-10 keyed by seed, one counter per
 * sample, so the output is a function of (parameters, n, seed) alone. */
#define EPR_SHAPE_TORUS_KNOT 0  /* ((2+cos qt) cos pt, (2+cos qt) sin pt, sin qt); a = p, b = q */
#define EPR_SHAPE_LINK 1        /* unit circles in xy at the origin and in xz at (1,0,0) */
#define EPR_SHAPE_HELIX 2       /* a turns of radius b over height c along z */
#define EPR_SHAPE_CLIFFORD 3    /* 4D: (cos u, sin u, cos v, sin v)/sqrt 2, frame d_u ^ d_v */
typedef struct epr_sampler {
    int shape;           /* EPR_SHAPE_* (curves 3D, with frames dual to the tangent) */
    int regular;         /* torus knot only: parameter t = 2 pi i / n instead of uniform */
    double a, b, c;      /* shape parameters (above) */
    double pos_sigma;    /* Gaussian positional noise in unit-cube units (x largest extent x 1.1) */
    double angle_deg;    /* frames rotated by a N(0, angle) angle in a random 2-plane */
    double spot_frac;    /* round(n spot_frac) extra samples uniform in the box, frames S - S^T, S in U[-1,1] */
    uint64_t seed;
} epr_sampler;

/* n samples (plus the outliers) in world coordinates: pos (total x dim), packed frames
 * (total x dim(dim-1)/2) copied to host buffers; total receives n + round(n spot_frac).  pos and
 * skew may both be NULL to query total. */
int epr_generate_samples(int device, const epr_sampler *sampler, size_t n, double *pos, double *skew, size_t *total);

/* Generates the samples into the context's device memory, maps them to the unit cube there
 * (ExteriorPoisson::ToUnitCube) and sets them as its samples (what epr_set_samples does with host
 * arrays), without a host round trip.  xform (may be NULL) receives the (dim+1)^2 map. */
int epr_set_generated_samples(epr_ctx *ctx, const epr_sampler *sampler, size_t n, double *xform);

/* Hierarchical solution coefficients of one level after epr_solve (what the reference writes to
 * its .tree file: level 0 regular, level d > 0 the residual x[d] - P x[d-1]). */
int epr_get_solution(epr_ctx *ctx, int level, double *x, double *y);

/* The density estimator of a built context (TreeEstimator's splat, GridSamples.h:232-277): for each
 * vertex of level `level` ((2^level+1)^dim, axis 0 slowest; the reference's tree nodes of depth
 * level+1 inside the unit cube) the splatted weight sum, position sum (dim) and covariance sum
 * (dim x dim, row-major): 1 + dim + dim^2 doubles per vertex; vertices the reference's tree never
 * creates hold zeros.  count receives the number of doubles; out may be NULL to query it. */
int epr_get_density(epr_ctx *ctx, int level, double *out, size_t cap, size_t *count);

/* The density tree's structure: out[cell] = 1 where the cell of tree depth t (0 .. depth+1; cells
 * (2^t)^dim, axis 0 most significant) has children.  The root (t = 0) always has children and the
 * cells of depth+1 never do.  count receives (2^t)^dim; out may be NULL to query it. */
int epr_get_density_refined(epr_ctx *ctx, int t, uint8_t *out, size_t cap, size_t *count);

/* Writes the density estimator's tree to `path` in the reference's .density.tree layout: the
 * voxel-to-world transform (voxel_to_world: (dim+1)^2 doubles in the order the .tree stores them,
 * element (column c, row r) at c (dim+1) + r) after one 8-byte zero word, the tree's nodes depth
 * first (each node's 2^dim children as one block before their subtrees; 136-byte nodes in 3D,
 * 208-byte in 4D: u16 depth, u16 offsets, parent and children words, weight, position and
 * covariance sums), then the target samples per cell 2^(dim-2).  Words that hold memory addresses
 * in the reference's file are written as zero (parent) or 1 (children present).  Needs a built
 * context; EPR_ERR_ARG when the file cannot be written. */
int epr_write_density_tree(epr_ctx *ctx, const double *voxel_to_world, const char *path);

/* Writes `path` as the reference's <out>.tree after a solve (ExteriorPoissonRecon.cpp:259-270): u32
 * dim, the u64 type hash of the context's indexer (the regular grid's or the adaptive one's, as
 * libstdc++ computes typeid(...).hash_code(); the reference's Extract selects the indexer by it),
 * the voxel-to-world transform as in epr_write_density_tree, every level's hierarchical x and y
 * coefficients in the indexer's function order (u64 levels, then per level i64 n and n doubles),
 * then the indexer: the regular grid's u32 maximum depth, or the adaptive indexer's node tree (40-byte
 * nodes in 3D, 48-byte in 4D: u16 depth, u16 offsets, parent and children words, u64 function and
 * element index, -1 when none), its active function counts and its function and element node
 * lists (counts, with zero address words).  Needs a solved context; EPR_ERR_ARG when the file
 * cannot be written. */
int epr_write_tree(epr_ctx *ctx, const double *voxel_to_world, const char *path);

/* The finest level's coefficients as the reference's regularCoefficients computes them from a
 * .tree (Hat.adaptive.inl:154-176; Extract's zero set and --grid output use them): the sum of every
 * level's hierarchical coefficients, each prolonged to the finest grid by the regular grid's
 * prolongation.  For the regular grid this is epr_get_coefficients(ctx, depth) after a solve; for
 * the adaptive indexer it also extends the solution beyond the indexed functions.  x and y hold
 * (2^depth+1)^dim doubles.  Needs a solved context. */
int epr_get_regular_coefficients(epr_ctx *ctx, double *x, double *y);

/* The adaptive indexer's tables of one level (adaptive_radius >= 0, after epr_build):
 * counts[0] = functions, counts[1] = active functions (the first counts[1] function indices, the
 * only ones relaxed), counts[2] = elements; fnodes (cap >= counts[0]) receives the grid node
 * (axis 0 most significant) of every function index, enodes (cap >= counts[2]) the grid element
 * of every element index.  Any output may be NULL.  EPR_ERR_STATE for a regular-grid context. */
int epr_get_adaptive_index(epr_ctx *ctx, int level, int64_t *counts, int64_t *fnodes, size_t fcap, int64_t *enodes, size_t ecap);

/* Named internal arrays copied to host memory: "measure", "noise", "depth" (per sample),
 * "S" (per finest element, packed), "leaf_depth", "R", "B" (per level, column stencils), "c".
 * count receives the number of doubles; out may be NULL to query it. */
int epr_get_array(epr_ctx *ctx, const char *name, int level, double *out, size_t cap, size_t *count);

/* Times `reps` launches of one kernel family on the context's stream with CUDA events and returns
 * the mean device time of a single launch in *ms: "gs" (one parity colour of the paired
 * Gauss-Seidel sweep, colour 0), "energy", "quadfit", "prolong", "gn" (Gauss-Newton matvec),
 * "lgs" (one colour of the linear Gauss-Seidel sweep on the alternating y-system, colour-blocked
 * stencil), "residual" (that system's residual), "assemble" (its assembly), "biquad" (the
 * bi-quadratic fit reduction).
 * The level's coefficients are modified by "gs". No counterpart in the reference (a profiling
 * hook for the benchmark). */
int epr_time_kernel(epr_ctx *ctx, const char *kernel, int level, int reps, double *ms);

/* Energy of one level computed without allocating anything, for callers that cannot call
 * cudaMalloc where they need the value (inside a stream capture that must not gain allocation
 * nodes, under an external memory pool or arena, in allocation-free real-time loops).  It has no
 * counterpart in the reference.  All pointers are device memory owned by the caller:
 *   xy    interleaved (x, y) coefficients, 2 (2^level+1)^dim values of the precision's type;
 *   A, B  the level's column stencils R + dWeight K and B, offset-major (value of offset o at
 *         node i at [o * N + i]), 3^dim N values of the precision's type;
 *   out3  3 doubles: fitting energy, regularisation energy, wedge square norm (as epr_energy).
 * The work is enqueued on `stream` (NULL = default stream) of `device`; the caller synchronises.
 * The caller's current device is left as it was.  The block partial sums use a fixed 128 KiB
 * device array inside the library (one copy per GPU, held until exit), which holds the partial
 * sums of any level; the accepted levels are the library's range, 0..10 (3D) / 0..7 (4D), and
 * other levels are rejected.  The first call on a device looks the array's address up and caches
 * it, so make that first call before any stream capture.  Calls that overlap on the GPU share the
 * array and race: serialise them.  Errors: epr_noalloc_last_error(). */
int epr_energy_noalloc(int device, int dim, int level, int precision, const void *xy, const void *A,
                       const void *B, double c, double *out3, void *stream);
const char *epr_noalloc_last_error(void);

/* Linear multigrid on a host system M v = b, M a symmetric column stencil of `level` (N x 3^dim,
 * node-major, entry o of node i holds M(i+off(o), i)), v updated in place.  In EPR_FP32 mode the
 * relaxation runs in float; epr_mg_vcycle then forms the residual and adds each correction in
 * double.
 *   epr_linear_gs:  iters coloured Gauss-Seidel sweeps (colours by per-axis parity, in order);
 *   epr_mg_vcycle:  cycles V-cycles with gs_iters relaxations before and after the coarse
 *                   correction on every level, Galerkin operators P^T M P, exact solve at
 *                   resolution 1. */
int epr_linear_gs(epr_ctx *ctx, int level, const double *M, const double *b, double *v, int iters);
int epr_mg_vcycle(epr_ctx *ctx, int level, const double *M, const double *b, double *v, int gs_iters, int cycles);

/* The linear system of one half-step of the alternating solve at the level's coefficients, as
 * AlternatingSolve forms it: which = 1 solves for y with x fixed, M = 2 (G_x + A), b = 2 B x;
 * which = 0 solves for x with y fixed, M = 2 (G_y + A), b = 2 B^T y; G_f is the wedge Gram matrix
 * (|f ^ v|^2 = v^T G_f v).  M: N x 3^dim node-major column stencil, b: N doubles. */
int epr_alternating_system(epr_ctx *ctx, int level, int which, double *M, double *b);
/* AlternatingSolve on the level's coefficients (in place): iters rounds of (y, then x), each
 * vcycles V-cycles of gs_iters relaxations, or gs_iters * vcycles sweeps when single_level != 0. */
int epr_alternating_solve(epr_ctx *ctx, int level, int iters, int vcycles, int gs_iters, int single_level);

/* q9[3i + j] = coefficient of s^i t^j of E(x + s dx, y + t dy) at the level's coefficients.
 * as_reference != 0 reproduces the reference's biQuadraticFit term by term, which deviates from
 * the exact expansion twice: its s t^2 coefficient is 2 <dx^dy, x^y> (SystemEnergy.h:506) and its
 * stiffness term has weight 1 instead of dWeight (SystemEnergy.h:522-530). */
int epr_biquadratic_fit(epr_ctx *ctx, int level, const double *dx, const double *dy, int as_reference, double *q9);
/* stepSize: the s minimising P(s, s) among the critical points; newtonUpdate: `steps` Newton
 * steps on P from (0, 0), each followed by an exact line search.  Host arithmetic only. */
int epr_step_size(const double *q9, double *s);
int epr_newton_update(const double *q9, int steps, double *st2);

/* Waits for all work of the context. */
int epr_synchronize(epr_ctx *ctx);

/* ---- Learned warm start ------------------------------------------------------------------------
 * No counterpart in the reference, whose solve starts from random coefficients at its coarsest solve
 * level (ExteriorPoisson.h:333-341): a 3D convolutional U-Net (16-32-64-128 channels, 3x3x3
 * kernels, BF16 weights and activations, FP32 accumulation on the tensor cores) predicts the
 * regular (x, y) coefficients of one level L of the cascadic solve (L = 6: 65^3 nodes) from the
 * density and frame splats of that level, and the solve then runs from level L (warm_start = 1,
 * min_solve_depth = L).  The network is trained on the GPU by the library's own forward and
 * backward kernels on solves the method computes.
 *
 * Activation layout of the primitives: BF16, channels-last (value of voxel v, channel c at
 * [v * ld + c]) on an n^3 node grid (voxel index with axis 0 slowest); ld and channel offsets
 * multiples of 8, buffers 16-byte aligned; all pointers device memory; work enqueued on `stream`. */

/* out = relu?(conv3x3x3(in) + bias): cin a multiple of 16, cout in {16, 32, 48, 64, 96, 128, 192};
 * w: cout x 27 cin BF16 (row co, column tap * cin + ci, tap = 9 (dz+1) + 3 (dy+1) + (dx+1));
 * flip != 0 uses the neighbour v - offset instead of v + offset (the data gradient of a
 * convolution is this with the weights transposed: row ci, column tap * cout + co). */
int epr_conv3(int device, int n, int cin, int cout, const void *in, int ldi, const void *w, const float *bias,
              void *out, int ldo, int relu, int flip, void *stream);
/* dw[(tap, ci)][co] = sum_v in[v + offset(tap)][ci] dz[v][co] (FP32, 27 cin x cout, overwritten);
 * scratch: epr_conv3_wgrad_scratch(n, cin, cout) floats of device memory. */
int epr_conv3_wgrad(int device, int n, int cin, int cout, const void *in, int ldi, const void *dz, int ldz, float *dw,
                    float *scratch, size_t scratch_floats, void *stream);
size_t epr_conv3_wgrad_scratch(int n, int cin, int cout);
const char *epr_conv_last_error(void);

typedef struct epr_unet epr_unet;
/* A network for level `level` (3..8) on `device`, He-initialised from `seed`.  NULL on error
 * (epr_unet_last_error(NULL)). */
epr_unet *epr_unet_create(int device, int level, uint64_t seed);
void epr_unet_destroy(epr_unet *net);
const char *epr_unet_last_error(const epr_unet *net);
/* FP32 master parameters (count in *count): copied to host (set = 0) or from host (set != 0). */
int epr_unet_params(epr_unet *net, float *host, size_t cap, size_t *count, int set);
/* nodes per axis of the network's grid, bytes of one input (n^3 x 16 BF16), floats of one target
 * or prediction (n^3 x 2). */
int epr_unet_grid(const epr_unet *net, int *nodes_per_axis, size_t *input_bytes, size_t *target_floats);
/* The network input of a built 3D context (depth >= the network's level), 16 BF16 channels per
 * vertex of the level, all scale-free: the density weight and the frame splat (3) divided by their
 * maximum magnitudes, the splatted samples' mean offset from the vertex in cells (3), the frame's
 * direction (3) and relative magnitude, the vertex coordinates in [-1, 1] (3), log(1 + weight /
 * max) / log 2, and a zero channel; into dev_input (NULL: the network's own input buffer). */
int epr_unet_input(epr_unet *net, epr_ctx *ctx, void *dev_input);
/* The training target of a solved context: its level-L regular (x, y) coefficients as FP32 pairs. */
int epr_unet_target(epr_unet *net, epr_ctx *ctx, float *dev_target);
/* Prediction (n^3 x 2 FP32) for an input (NULL: the network's own); with dev_target, *loss is the
 * training loss 1 - (<p,t>^2 + <p x t>^2) / (|p|^2 |t|^2), invariant under scaling and rotating p. */
int epr_unet_forward(epr_unet *net, const void *dev_input, float *dev_pred, double *loss, const void *dev_target);
/* Loss and the gradient of every parameter (host, count floats, the master layout) for one pair. */
int epr_unet_gradients(epr_unet *net, const void *dev_input, const void *dev_target, float *host_grads, double *loss);
/* One Adam step on the mean loss of `batch` (input, target) pairs in device memory. */
int epr_unet_train_step(epr_unet *net, int batch, const void *const *dev_inputs, const void *const *dev_targets,
                        float lr, double *loss);
/* Warm start of a built context: predicts its level-L coefficients, scales them by the factor that
 * minimises the energy along the prediction (E(s p) is a quartic in s: one energy evaluation gives
 * it), and sets them as the level's coefficients; the prediction's reflection (x, -y), whose wedge
 * is the negated one, is taken instead when its minimum is lower (the same evaluation gives it).
 * Falls back to the reference's random start on that level when the scaled prediction's energy is
 * not below both the random start's and the zero function's.  info (4 doubles, may be NULL): used
 * (1, 2 when reflected, 0 when not used), energy of the scaled prediction, energy of the random
 * start, scale. */
int epr_unet_warm_start(epr_unet *net, epr_ctx *ctx, double *info);

#ifdef __cplusplus
}
#endif
#endif
