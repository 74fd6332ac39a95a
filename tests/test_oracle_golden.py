"""Pins the CPU restatement (oracle/epr_oracle.cpp) against fixtures written by the reference
implementation itself (tests/golden/make_golden.py).  Tolerances are relative to each array's
largest magnitude; FP64 throughout."""
import numpy as np
import pytest

from conftest import GOLDEN_CASES, load_golden
from oracle import oracle as O


def rel(a, b):
    a = np.asarray(a, dtype=np.float64).ravel()
    b = np.asarray(b, dtype=np.float64).ravel()
    assert a.shape == b.shape
    return float(np.abs(a - b).max() / max(np.abs(b).max(), 1e-300))


@pytest.fixture(scope="module", params=GOLDEN_CASES)
def case(request):
    g = load_golden(request.param)
    dim = g["pos"].shape[1]
    depth = int(g["depth"])
    o = O.Oracle(dim, depth)
    o.set_samples(g["pos"], g["skew"])
    o.build()
    return g, o, dim, depth


def test_unit_cube(case):
    g, o, dim, depth = case
    pos, xf = O.unit_cube(g["world_pos"])
    assert np.array_equal(pos, g["pos"])
    assert np.array_equal(xf, g["world_to_unit"])


def test_ordered_cells(case):
    g, o, dim, depth = case
    assert np.array_equal(o.get("cells").reshape(-1, dim), g["cells"])
    assert np.array_equal(o.get("cell_counts"), g["cell_counts"])


def test_density_tree(case):
    g, o, dim, depth = case
    for l in range(depth + 1):
        assert rel(o.get("density", l), g[f"density_l{l}"]) < 1e-12


def test_estimator(case):
    g, o, dim, depth = case
    assert rel(o.get("measure"), g["est_measure"]) < 1e-12
    assert rel(o.get("depth"), g["est_depth"]) < 1e-12
    # eigenvalues by Jacobi rotations instead of Eigen's solver
    assert rel(o.get("noise"), g["est_noise"]) < 1e-9


def test_skew_splat_and_constraint(case):
    g, o, dim, depth = case
    for l in range(depth + 1):
        assert rel(o.get("skew", l), g[f"skew_l{l}"]) < 1e-12
    assert np.array_equal(o.get("leaf_depth"), g["leaf_depth"])
    assert rel(o.get("S"), g["S"]) < 1e-12
    assert abs(o.get("c")[0] - g["c"][0]) < 1e-12 * g["c"][0]


def test_system_stencils(case):
    g, o, dim, depth = case
    for l in g["stencil_levels"]:
        assert rel(o.get("R", int(l)), g[f"R_d{l}"]) < 1e-10
        assert rel(o.get("B", int(l)), g[f"B_d{l}"]) < 1e-12


def test_energy_levels(case):
    g, o, dim, depth = case
    for l in range(depth + 1):
        e = o.energy(l, g[f"xr_d{l}"], g[f"yr_d{l}"])
        ref = g[f"energies_d{l}"]
        for k in range(3):
            assert abs(e[k] - ref[k]) <= 1e-12 * abs(ref[k]) + 1e-14, (l, k, e, ref)


def test_quadfit_and_gs(case):
    g, o, dim, depth = case
    for key in g:
        if not key.startswith("quadfit_d"):
            continue
        l = int(key[len("quadfit_d"):])
        x, y = g[f"xr_d{l}"], g[f"yr_d{l}"]
        assert rel(o.quadfit(l, x, y), g[key]) < 1e-11
        gx, gy = o.gs(l, x, y, 1)
        assert rel(gx, g[f"gsx_d{l}"]) < 1e-11
        assert rel(gy, g[f"gsy_d{l}"]) < 1e-11


def test_prolongation(case):
    g, o, dim, depth = case
    for l in range(depth):
        assert rel(o.prolong(l, g[f"xr_d{l}"]), g[f"prolong_d{l}"]) < 1e-15


def test_cascadic_solve(case):
    g, o, dim, depth = case
    xs, ys, e = o.solve()
    ref = g["sol_energies"]
    assert abs(e[1] - ref[0]) < 1e-10 * ref[0]
    assert abs(e[2] - ref[1]) < 1e-10 * ref[1]
    for l in range(depth + 1):
        assert rel(xs[l], g[f"solx_d{l}"]) < 1e-9
        assert rel(ys[l], g[f"soly_d{l}"]) < 1e-9


ORACLE_NAMES = {"separate": "separate", "singleLevel": "single_level", "gsIters": "gs_iters", "seed": "seed",
                "minSolveDepth": "min_solve_depth", "iMult": "i_mult"}


@pytest.mark.parametrize("name", ["knot3_d4_separate", "knot3_d4_single", "knot3_d4_seed7_min2"])
def test_solver_variants(name):
    from conftest import variant_params
    g = load_golden(name)
    depth = int(g["depth"])
    kw = {ORACLE_NAMES[k]: v for k, v in variant_params(g["flags"]).items()}
    o = O.Oracle(3, depth, **kw)
    o.set_samples(g["pos"], g["skew"])
    o.build()
    xs, ys, e = o.solve()
    ref = g["sol_energies"]
    assert abs(e[1] - ref[0]) < 1e-10 * ref[0]
    assert abs(e[2] - ref[1]) < 1e-10 * ref[1]
    for l in range(depth + 1):
        assert rel(xs[l], g[f"solx_d{l}"]) < 1e-9
        assert rel(ys[l], g[f"soly_d{l}"]) < 1e-9


def test_linear_multigrid(case):
    """GSRelaxer sweep and MGSolver V-cycles (MG.h:57-72, 150-187) on M = R + dWeight K."""
    g, o, dim, depth = case
    M, b = g["mg_M"], g["mg_b"]
    x = o.linear_gs(depth, M, b, np.zeros_like(b))
    assert rel(x, g["mg_gs1"]) < 1e-12
    x1 = o.mg_vcycle(depth, M, b, np.zeros_like(b), 2, 1)
    assert rel(x1, g["mg_v1"]) < 1e-10
    x2 = o.mg_vcycle(depth, M, b, x1, 2, 1)
    assert rel(x2, g["mg_v2"]) < 1e-10
