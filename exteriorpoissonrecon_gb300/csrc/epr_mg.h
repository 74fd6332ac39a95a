// Host entry points of the linear multigrid and the solvers built on it (epr_mg.cu).
#pragma once
#include "epr_context.h"

namespace epr {

struct MGHierarchy;
void release_mg(Context &c);

// iters coloured Gauss-Seidel sweeps of M x = b (GSRelaxer, MG.h:57-72); M is a host column
// stencil (N x 3^dim, node-major), x is updated in place
bool linear_gs(Context &c, int level, const double *M, const double *b, double *x, int iters);
// cycles V-cycles (MGSolver, MG.h:81-187, iters relaxations per level, Galerkin hierarchy down to
// resolution 1) of M x = b
bool mg_vcycles(Context &c, int level, const double *M, const double *b, double *x, int iters, int cycles);
// half-step system of the alternating solve at the level's coefficients (which 1: y free, 0: x free)
bool alternating_system(Context &c, int level, int which, double *M, double *b);
// AlternatingSolve on the level's coefficients
bool alternating_solve(Context &c, int level, int iters, int vcycles, int gsIters, bool singleLevel);
// relaxation of one level of the multigrid solver: alternating rounds (one V-cycle of gs_iters
// relaxations per half-step) until |grad E| <= tolerance |grad E(start)| or max_cycles rounds
bool relax_alternating(Context &c, int level, bool finest);
// CUDA-event time of one launch of a multigrid kernel family ("lgs", "residual", "assemble", "biquad")
bool time_mg_kernel(Context &c, const char *kernel, int level, int reps, double *ms);
// |grad E| of the level's double coefficients
bool grad_norm(Context &c, int level, double *out);
// bi-quadratic fit along the device direction pairs ddxy (2N doubles)
bool biquadratic_fit(Context &c, int level, const double *ddxy, bool asReference, double *q);

}  // namespace epr
