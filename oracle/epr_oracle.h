/* CPU restatement of the reference regular-grid reconstruction path (test infrastructure only).
 *
 * This library is the oracle the CUDA path is checked against and the CPU baseline that the
 * benchmark times.  It is never linked into the product library.  Every function restates one
 * step of the reference (file:line cited at its definition in epr_oracle.cpp).
 *
 * Conventions shared with the CUDA path:
 *   - node (function) index: axis 0 most significant, (r+1)^Dim nodes per level (r = 2^depth);
 *   - element index: axis 0 most significant, r^Dim elements;
 *   - packed skew matrices: p[i(i-1)/2 + j] for i > j (Dim(Dim-1)/2 values);
 *   - column stencils: 3^Dim values per node i, entry o holds M(i + off(o), i), where
 *     o = sum_d (off[d]+1) 3^(Dim-1-d).
 */
#ifndef EPR_ORACLE_H
#define EPR_ORACLE_H
#include <stddef.h>
#include <stdint.h>
#ifdef __cplusplus
extern "C" {
#endif

typedef struct epr_oracle epr_oracle;

typedef struct epr_oracle_params {
    double s_weight;      /* --sWeight (screening) */
    double d_weight;      /* --dWeight (Dirichlet) */
    double n_sigma;       /* --nSigma */
    double i_mult;        /* --iMult */
    int t_radius;         /* --tRadius */
    int d_radius;         /* --dRadius */
    int gs_iters;         /* --gsIters */
    int min_solve_depth;  /* --minSolveDepth */
    int max_solve_depth;  /* --maxSolveDepth (-1 = depth) */
    unsigned int seed;    /* --seed */
    int threads;          /* OpenMP threads (0 = all) */
    int single_level;     /* --singleLevel */
    int separate;         /* --separate */
    int alt_rounds;       /* > 0: relax every level with this many AlternatingSolve rounds (one
                             V-cycle of gs_iters relaxations per half-step) instead of paired GS */
    int project;          /* --project: S(E) projected onto its best blade (ExteriorPoisson.h:300-305,
                             411-438) */
    int adaptive_radius;  /* --aRadius: -1 the regular grid; >= 0 the adaptive indexer's function and
                             element sets (Hat.adaptive.inl:342-732) on the same grids */
} epr_oracle_params;

void epr_oracle_default_params(epr_oracle_params *p);

/* world -> unit cube map (ExteriorPoisson.h:100-123); xform is (Dim+1)x(Dim+1) with the same
 * (column, row) element order as the reference SquareMatrix; positions are mapped in place. */
int epr_oracle_unit_cube(int dim, size_t n, double scale, double *pos, double *xform);

epr_oracle *epr_oracle_create(int dim, int depth, const epr_oracle_params *p);
void epr_oracle_destroy(epr_oracle *o);

/* unit-cube positions (n x Dim) and packed skew frames (n x Dim(Dim-1)/2) */
int epr_oracle_set_samples(epr_oracle *o, size_t n, const double *pos, const double *skew);

/* Runs ordered sampling, density estimation, skew splatting, S(E), R, B and the Galerkin
 * hierarchy (ExteriorPoisson.h:126-313). */
int epr_oracle_build(epr_oracle *o);

/* Replaces the system of one level: A = R + dWeight K (column stencil), B (column stencil), c. */
int epr_oracle_set_level_system(epr_oracle *o, int level, const double *R, const double *B, double c);

/* Named arrays: "cells","measure","noise","depth","S","leaf_depth","R","B","A","density","skew",
 * "exists"; with the adaptive indexer also "status" (per node of a level: 0 no function, 1 an
 * indexed function that is not relaxed, 2 an active one), "fnodes" (the node of every function
 * index of a level), "enodes" (the element of every element index) and "nactive". Returns the number of doubles written (out may be NULL to query the size). */
long epr_oracle_get(epr_oracle *o, const char *name, int level, double *out);

size_t epr_oracle_num_nodes(int dim, int level);

/* energies(): out[0] = fit, out[1] = regularisation, out[2] = wedge square norm
 * (SystemEnergy.h:486-497). */
int epr_oracle_energy(epr_oracle *o, int level, const double *x, const double *y, double *out);
/* quadraticFit at every node: out is N x 5 (Q20, Q02, Q11, Q10, Q01), SystemEnergy.h:542-643 */
int epr_oracle_quadfit(epr_oracle *o, int level, const double *x, const double *y, double *out);
/* gradient of the energy: gx, gy (N each) */
/* quadfit / Gauss-Newton product at the nodes idx[0..n) only (row k belongs to node idx[k]) */
int epr_oracle_quadfit_at(epr_oracle *o, int level, const double *x, const double *y, const int64_t *idx, size_t n,
                          double *out);
int epr_oracle_gn_matvec_at(epr_oracle *o, int level, const double *x, const double *y, const double *dx,
                            const double *dy, const int64_t *idx, size_t n, double *ox, double *oy);
int epr_oracle_gradient(epr_oracle *o, int level, const double *x, const double *y, double *gx, double *gy);
/* paired Gauss-Seidel, iters full sweeps over the 2^Dim parity colours (ExteriorPoissonSolvers.h:156-196) */
int epr_oracle_gs(epr_oracle *o, int level, double *x, double *y, int iters);
/* paired Gauss-Seidel on the shifted energy E - <tx, x> - <ty, y> (tx, ty per node) */
int epr_oracle_gs_shifted(epr_oracle *o, int level, double *x, double *y, int iters, const double *tx, const double *ty);
/* one coloured Gauss-Seidel sweep of M x = b with a column-stencil M (GSRelaxer, MG.h:57-72) */
int epr_oracle_linear_gs(epr_oracle *o, int level, const double *M, const double *b, double *x);
/* `cycles` V-cycles (MGSolver::vCycle, MG.h:150-187, iters relaxations per level) of M x = b with the
 * Galerkin hierarchy of the column stencil M of `level`; x is updated in place */
int epr_oracle_mg_vcycle(epr_oracle *o, int level, const double *M, const double *b, double *x, int iters, int cycles);
/* wedge Gram matrix of a fixed field f (column stencil, N x 3^dim): v^T G v = |W(f, v)|^2 */
int epr_oracle_wedge_gram(epr_oracle *o, int level, const double *f, double *G);
/* system of one alternating half-step (ExteriorPoissonSolvers.h:96-131): which 1 -> y free,
 * which 0 -> x free; M (N x 3^dim column stencil) and right-hand side b */
int epr_oracle_alternating_system(epr_oracle *o, int level, const double *x, const double *y, int which, double *M, double *b);
/* AlternatingSolve (ExteriorPoissonSolvers.h:86-154) on (x, y) in place */
int epr_oracle_alternating_solve(epr_oracle *o, int level, double *x, double *y, int iters, int vcycles, int gs_iters, int single_level);
/* q9[i*3+j] = coefficient of s^i t^j of E(x+s dx, y+t dy); as_reference != 0 reproduces the
 * reference's biQuadraticFit (SystemEnergy.h:499-540) including its two deviations */
int epr_oracle_biquadratic_fit(epr_oracle *o, int level, const double *x, const double *y, const double *dx, const double *dy, double *q9,
                               int as_reference);
/* stepSize / newtonUpdate (SystemEnergy.h:256-303) on a bi-quadratic fit */
double epr_oracle_step_size(const double *q9);
void epr_oracle_newton_update(const double *q9, int steps, double *st);
/* restriction coarse = P^T fine of a level-(level+1) vector to level `level` */
int epr_oracle_restrict(epr_oracle *o, int level, const double *fine, double *coarse);
/* prolongation of a level-`level` vector to level+1 (Hat.scalars.inl:1747-1779) */
int epr_oracle_prolong(epr_oracle *o, int level, const double *coarse, double *fine);
/* Gauss-Newton matvec of the energy's quadratic model at (x,y) applied to (dx,dy) */
int epr_oracle_gn_matvec(epr_oracle *o, int level, const double *x, const double *y,
                         const double *dx, const double *dy, double *ox, double *oy);

/* cascadic solve (ExteriorPoisson.h:315-409); x_out,y_out receive the hierarchical coefficients of
 * every level concatenated (level 0 first); energies_out = (E0, fit, reg). */
int epr_oracle_solve(epr_oracle *o, double *x_out, double *y_out, double *energies_out);
/* The same cascadic solve in pieces: begin (random start; returns the schedule's node updates),
 * advance (whole sweeps in order until target node updates are done; 1 when complete), finish
 * (energies as epr_oracle_solve's: c, fit, reg). */
int64_t epr_oracle_solve_begin(epr_oracle *o);
int epr_oracle_solve_advance(epr_oracle *o, int64_t target_node_updates);
int epr_oracle_solve_finish(epr_oracle *o, double *energies_out);

#ifdef __cplusplus
}
#endif
#endif
