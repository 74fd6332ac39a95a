"""Parity of the CUDA linear multigrid, the alternating-solve systems and the bi-quadratic fit
(through the C ABI) with the reference's own outputs (golden fixtures) and with the oracle.

Tolerances: FP64 1e-12 relative for single sweeps, systems and fits, 1e-10 for V-cycles (Galerkin
products and a dense coarse solve), 1e-9 for multi-round alternating solves; FP32 1e-5."""
import numpy as np
import pytest

import exteriorpoissonrecon_gb300 as epr
from conftest import GOLDEN_CASES, load_golden
from oracle import oracle as O

pytestmark = pytest.mark.gpu


def rel(a, b):
    a = np.asarray(a, dtype=np.float64).ravel()
    b = np.asarray(b, dtype=np.float64).ravel()
    assert a.shape == b.shape, (a.shape, b.shape)
    return float(np.abs(a - b).max() / max(np.abs(b).max(), 1e-300))


@pytest.fixture(scope="module", params=GOLDEN_CASES)
def built(request):
    g = load_golden(request.param)
    dim = g["pos"].shape[1]
    depth = int(g["depth"])
    r = epr.Reconstructor(dim, depth, g["pos"], g["skew"])
    return g, r, dim, depth


def test_linear_gs_sweep(built):
    g, r, dim, depth = built
    v = r.linear_gs(depth, g["mg_M"], g["mg_b"], np.zeros_like(g["mg_b"]), iters=1)
    assert rel(v, g["mg_gs1"]) < 1e-12


def test_vcycles(built):
    g, r, dim, depth = built
    M, b = g["mg_M"], g["mg_b"]
    v1 = r.mg_vcycle(depth, M, b, np.zeros_like(b), gs_iters=2, cycles=1)
    assert rel(v1, g["mg_v1"]) < 1e-10
    v2 = r.mg_vcycle(depth, M, b, np.zeros_like(b), gs_iters=2, cycles=2)
    assert rel(v2, g["mg_v2"]) < 1e-10


def test_vcycles_fp32(built):
    g, r, dim, depth = built
    r32 = epr.Reconstructor(dim, depth, g["pos"], g["skew"], precision="fp32")
    M, b = g["mg_M"], g["mg_b"]
    assert rel(r32.linear_gs(depth, M, b, np.zeros_like(b), iters=1), g["mg_gs1"]) < 1e-5
    assert rel(r32.mg_vcycle(depth, M, b, np.zeros_like(b), gs_iters=2, cycles=2), g["mg_v2"]) < 1e-5
    # float relaxation with double residuals tracks the double iteration (the V-cycle contracts
    # slowly on these high-contrast operators, ~0.95 per cycle, so rounding would show here)
    v64 = r.mg_vcycle(depth, M, b, np.zeros_like(b), gs_iters=2, cycles=30)
    v32 = r32.mg_vcycle(depth, M, b, np.zeros_like(b), gs_iters=2, cycles=30)
    assert rel(v32, v64) < 1e-5
    A = sparse(M, dim, depth)
    assert np.linalg.norm(A @ v32 - b) < 0.7 * np.linalg.norm(A @ g["mg_v2"] - b)


def sparse(M, dim, level):
    """Sparse matrix of a column stencil (tests only)."""
    from scipy.sparse import csc_matrix
    rr = 1 << level
    N = (rr + 1) ** dim
    idx = np.array(np.unravel_index(np.arange(N), (rr + 1,) * dim)).T
    rows, cols, vals = [], [], []
    for o in range(3 ** dim):
        off = np.array(np.unravel_index(o, (3,) * dim)) - 1
        J = idx + off
        ok = np.all((J >= 0) & (J <= rr), axis=1)
        rows.append(np.ravel_multi_index(J[ok].T, (rr + 1,) * dim))
        cols.append(np.arange(N)[ok])
        vals.append(M[ok, o])
    return csc_matrix((np.concatenate(vals), (np.concatenate(rows), np.concatenate(cols))), shape=(N, N))


def test_wedge_gram_against_reference(built):
    """Half-step systems: u^T (M/2 - A) v equals the reference's <x^u, x^v> (and <u^y, v^y>)."""
    from conftest import stencil_apply
    g, r, dim, depth = built
    x, y = g["qa_x"], g["qa_y"]
    r.set_coefficients(depth, x, y)
    A = r.get("A", depth).reshape(-1, 3 ** dim)
    for which, key in ((1, "qa_gx"), (0, "qa_gy")):
        M, b = r.alternating_system(depth, which)
        G = 0.5 * M - A
        vals = [g["qa_u"][k] @ stencil_apply(G, g["qa_v"][k], dim, depth) for k in range(len(g[key]))]
        assert rel(vals, g[key]) < 1e-11


def test_alternating_system_matches_oracle(built):
    g, r, dim, depth = built
    o = O.Oracle(dim, depth)
    o.set_samples(g["pos"], g["skew"])
    o.build()
    x, y = g["qa_x"], g["qa_y"]
    r.set_coefficients(depth, x, y)
    for which in (0, 1):
        M, b = r.alternating_system(depth, which)
        Mo, bo = o.alternating_system(depth, x, y, which)
        assert rel(M, Mo) < 1e-12
        assert rel(b, bo) < 1e-12


def test_biquadratic_fit(built):
    g, r, dim, depth = built
    r.set_coefficients(depth, g["qa_x"], g["qa_y"])
    q = r.biquadratic_fit(depth, g["qa_dx"], g["qa_dy"], as_reference=True)
    assert rel(q, g["qa_biquad"]) < 1e-12
    assert abs(epr.step_size(q) - g["qa_step"][0]) < 1e-9 * abs(g["qa_step"][0])
    assert np.abs(epr.newton_update(q, 10) - g["qa_newton"]).max() < 1e-9 * np.abs(g["qa_newton"]).max()
    o = O.Oracle(dim, depth)
    o.set_samples(g["pos"], g["skew"])
    o.build()
    qe = r.biquadratic_fit(depth, g["qa_dx"], g["qa_dy"])
    assert rel(qe, o.biquadratic_fit(depth, g["qa_x"], g["qa_y"], g["qa_dx"], g["qa_dy"])) < 1e-12


@pytest.mark.parametrize("single", [False, True])
def test_alternating_solve_matches_oracle(built, single):
    g, r, dim, depth = built
    o = O.Oracle(dim, depth)
    o.set_samples(g["pos"], g["skew"])
    o.build()
    lev = depth - 1
    x0, y0 = 0.01 * g[f"xr_d{lev}"], 0.01 * g[f"yr_d{lev}"]
    r.set_coefficients(lev, x0, y0)
    x, y = r.alternating_solve(lev, iters=2, vcycles=2, gs_iters=2, single_level=single)
    xo, yo = o.alternating_solve(lev, x0, y0, iters=2, vcycles=2, gs_iters=2, single_level=single)
    assert rel(x, xo) < 1e-9
    assert rel(y, yo) < 1e-9


@pytest.mark.parametrize("precision", ["fp64", "fp32"])
def test_multigrid_solver_matches_oracle(precision):
    """EPR_SOLVER_MULTIGRID: the cascadic schedule with every level relaxed by alternating-solve
    rounds (fixed round count: tolerance 0) against the oracle's same schedule."""
    g = load_golden("knot3_d4")
    depth = int(g["depth"])
    r = epr.Reconstructor(3, depth, g["pos"], g["skew"], solver="multigrid", tolerance=0.0, max_cycles=2,
                          gsIters=2, precision=precision)
    st = r.solve()
    assert st["cycles"] == 2 * (depth + 1)
    xs, ys = r.solution()
    o = O.Oracle(3, depth, alt_rounds=2, gs_iters=2)
    o.set_samples(g["pos"], g["skew"])
    o.build()
    xo, yo, eo = o.solve()
    tol = 1e-8 if precision == "fp64" else 1e-4
    for l in range(depth + 1):
        assert rel(xs[l], xo[l]) < tol, l
        assert rel(ys[l], yo[l]) < tol, l
    assert abs(st["fit_energy"] + st["reg_energy"] - (eo[1] + eo[2])) < tol * (eo[1] + eo[2])


@pytest.fixture(scope="module")
def link6():
    pos, fr = epr.samples.make_workload("link", 100000, seed=1)
    pu, _ = epr.unit_cube(pos)
    return pu, epr.pack_skew(fr)


def test_float_levels_track_double(link6):
    """At depth 6 the fine levels relax in float (>= 32768 nodes); V-cycles with double residuals
    track the double V-cycles, and the multigrid solver's float result has the double energy."""
    pu, sk = link6
    depth = 6
    r64 = epr.Reconstructor(3, depth, pu, sk)
    r32 = epr.Reconstructor(3, depth, pu, sk, precision="fp32")
    n = r64.nodes(depth)
    rng = np.random.default_rng(0)
    r64.set_coefficients(depth, rng.uniform(-0.1, 0.1, n), rng.uniform(-0.1, 0.1, n))
    M, b = r64.alternating_system(depth, 1)
    for cycles, tol in ((1, 1e-5), (20, 1e-7)):
        v64 = r64.mg_vcycle(depth, M, b, np.zeros(n), gs_iters=2, cycles=cycles)
        v32 = r32.mg_vcycle(depth, M, b, np.zeros(n), gs_iters=2, cycles=cycles)
        assert rel(v32, v64) < tol
    e = {}
    sol = {}
    for prec in ("fp64", "fp32"):
        r = epr.Reconstructor(3, depth, pu, sk, solver="multigrid", tolerance=0.0, max_cycles=3, gsIters=2, precision=prec)
        st = r.solve()
        e[prec] = st["fit_energy"] + st["reg_energy"]
        sol[prec] = r.solution()[0][depth]
    assert abs(e["fp32"] - e["fp64"]) < 1e-5 * e["fp64"]
    assert np.linalg.norm(sol["fp32"] - sol["fp64"]) < 1e-3 * np.linalg.norm(sol["fp64"])


def test_multigrid_solver_4d_matches_oracle():
    g = load_golden("cliff4_d3")
    depth = int(g["depth"])
    r = epr.Reconstructor(4, depth, g["pos"], g["skew"], solver="multigrid", tolerance=0.0, max_cycles=2, gsIters=2)
    st = r.solve()
    assert st["cycles"] == 2 * (depth + 1)
    xs, ys = r.solution()
    o = O.Oracle(4, depth, alt_rounds=2, gs_iters=2)
    o.set_samples(g["pos"], g["skew"])
    o.build()
    xo, yo, eo = o.solve()
    for l in range(depth + 1):
        assert rel(xs[l], xo[l]) < 1e-8, l
        assert rel(ys[l], yo[l]) < 1e-8, l
