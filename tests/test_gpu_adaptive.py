"""The adaptive indexer on the GPU (adaptive_radius / --aRadius K >= 0, the reference command line's
default): its tables, system, probes and cascadic solve against the reference's own outputs
(tests/golden/make_golden.py ADAPTIVE), the command line's .tree / .grid against the reference's
files, and the zero set in the benchmark's precision configuration.

Tolerances: index tables exact; FP64 stencils 1e-12 (R 1e-10, it carries the eigenvalue-based
noise weights), energies 1e-12; whole solves: energies 1e-10, coefficients 1e-8 (the rounding of
the FP64 sums, in another order than the reference's, accumulates over the schedule's sweeps: the
narrow K = 0 band measured 1.6e-9)."""
import os
import subprocess
import tempfile

import numpy as np
import pytest

import exteriorpoissonrecon_gb300 as epr
from conftest import ADAPTIVE_CASES, ADAPTIVE_TREES, load_golden
from exteriorpoissonrecon_gb300 import samples
from oracle import adapted_tree as AT
from oracle import zero_set as Z

pytestmark = pytest.mark.gpu

HEADLINE = ["--precision", "fp32", "--fp64From", "0", "--fp64Levels", "4", "--bandPrecision", "df"]


def rel(a, b):
    a = np.asarray(a, dtype=np.float64).ravel()
    b = np.asarray(b, dtype=np.float64).ravel()
    assert a.shape == b.shape, (a.shape, b.shape)
    return float(np.abs(a - b).max() / max(np.abs(b).max(), 1e-300))


@pytest.fixture(scope="module", params=ADAPTIVE_CASES)
def built(request):
    g = load_golden(request.param)
    dim = g["pos"].shape[1]
    depth = int(g["depth"])
    r = epr.Reconstructor(dim, depth, g["pos"], g["skew"], aRadius=int(g["a_radius"]))
    return g, r, dim, depth


def test_index_tables(built):
    g, r, dim, depth = built
    for l in range(depth + 1):
        t = r.adaptive_index(l)
        assert t["active"] == int(g[f"aact_d{l}"][0])
        assert np.array_equal(t["fnodes"], g[f"afn_d{l}"]), l
        assert np.array_equal(t["enodes"], g[f"ael_d{l}"]), l


def test_system(built):
    g, r, dim, depth = built
    assert abs(r.get("c")[0] - g["c"][0]) < 1e-12 * g["c"][0]
    for l in g["stencil_levels"]:
        assert rel(r.get("R", int(l)), g[f"R_d{l}"]) < 1e-10
        assert rel(r.get("B", int(l)), g[f"B_d{l}"]) < 1e-12


def test_energies_fits_sweep_prolongation(built):
    g, r, dim, depth = built
    for l in range(depth + 1):
        x, y = g[f"xr_d{l}"], g[f"yr_d{l}"]
        e = r.energy(l, x, y)
        ref = g[f"energies_d{l}"]
        for k in range(3):
            assert abs(e[k] - ref[k]) <= 1e-12 * abs(ref[k]) + 1e-14, (l, k, e, ref)
        if f"quadfit_d{l}" in g:
            active = g[f"afn_d{l}"][:int(g[f"aact_d{l}"][0])]
            assert rel(r.quadfit(l, x, y)[active], g[f"quadfit_d{l}"]) < 1e-11
            gx, gy = r.gs(l, x, y, 1)
            assert rel(gx, g[f"gsx_d{l}"]) < 1e-11
            assert rel(gy, g[f"gsy_d{l}"]) < 1e-11
        if l < depth:
            z = np.zeros(r.nodes(l + 1))
            r.set_coefficients(l + 1, z, z)
            r.set_coefficients(l, x, y)
            r.prolong(l)
            px, _ = r.coefficients(l + 1)
            assert rel(px, g[f"prolong_d{l}"]) < 1e-15


def test_cascadic_solve(built):
    g, r, dim, depth = built
    st = r.solve()
    ref = g["sol_energies"]
    assert abs(st["fit_energy"] - ref[0]) < 1e-10 * ref[0]
    assert abs(st["reg_energy"] - ref[1]) < 1e-10 * ref[1]
    xs, ys = r.solution()
    for l in range(depth + 1):
        assert rel(xs[l], g[f"solx_d{l}"]) < 1e-8
        assert rel(ys[l], g[f"soly_d{l}"]) < 1e-8
    # the regular coefficients extend the solution beyond the indexed functions with the regular
    # grid's prolongation (regularCoefficients, Hat.adaptive.inl:154-176)
    X, Y = r.regular_coefficients()
    assert rel(X, Z.regular_finest([g[f"solx_d{l}"] for l in range(depth + 1)], dim)) < 1e-8
    assert rel(Y, Z.regular_finest([g[f"soly_d{l}"] for l in range(depth + 1)], dim)) < 1e-8


def test_mixed_precision_solve():
    """FP32 relaxation with the double-float band on the adaptive indexer: the same schedule's
    FP64-evaluated energy within 1e-5 of the all-FP64 solve's."""
    g = load_golden("link3_d5_a3")
    K = int(g["a_radius"])
    e = []
    for kw in ({}, dict(precision="fp32", fp64_from=0, fp64_levels=4, band_precision="df")):
        r = epr.Reconstructor(3, int(g["depth"]), g["pos"], g["skew"], aRadius=K, **kw)
        st = r.solve()
        e.append(st["fit_energy"] + st["reg_energy"])
        r.close()
    assert abs(e[1] - e[0]) <= 1e-5 * e[0], e


def test_regular_grid_has_no_adaptive_tables():
    g = load_golden("knot3_d4")
    r = epr.Reconstructor(3, 4, g["pos"], g["skew"])
    with pytest.raises(epr.EprError):
        r.adaptive_index(0)


@pytest.fixture(scope="module")
def cli():
    from exteriorpoissonrecon_gb300.build import build_cli
    epr.load()
    return build_cli()


@pytest.mark.parametrize("name", sorted(ADAPTIVE_TREES))
def test_cli_adaptive_tree_matches_reference_file(cli, name):
    """The command line's default indexer: its .tree holds the reference's tree node for node
    (depth, offset, children, function and element index), the same counts, the solution within
    1e-8, and every other byte the reference's reader interprets; its .grid the values the
    reference's Extract writes from the reference's own .tree."""
    g = load_golden(name)
    depth = int(g["depth"])
    with tempfile.TemporaryDirectory() as td:
        ply = os.path.join(td, "in.ply")
        samples.write_ply(ply, g["world_pos"], g["frames"])
        out = os.path.join(td, "out")
        r = subprocess.run([cli, "--in", ply, "--out", out, "--grid", out, "--depth", str(depth)] + list(g["flags"]),
                           capture_output=True, text=True, timeout=300)
        assert r.returncode == 0, r.stderr
        with open(out + ".tree", "rb") as f:
            raw = f.read()
        grids = []
        for c in range(2):
            with open(out + f".{c}.grid", "rb") as f:
                grids.append(f.read())
    ref_raw = g["tree"].tobytes()
    got, ref = AT.parse(raw), AT.parse(ref_raw)
    assert got["hash"] == ref["hash"] == AT.HASH[got["dim"]]
    for k in ("depth", "offset", "has_children", "findex", "eindex", "active", "functions", "elements"):
        assert np.array_equal(got[k], ref[k]), k
    assert np.allclose(got["xform"], ref["xform"], rtol=1e-14, atol=1e-14)
    for a, b in zip(got["x"] + got["y"], ref["x"] + ref["y"]):
        assert a.shape == b.shape
        assert np.abs(a - b).max() <= 1e-8 * max(np.abs(b).max(), 1e-30)
    # every byte outside the coefficients, the transform and the address words agrees
    m_got, m_ref = AT.masked(raw), AT.masked(ref_raw)
    assert len(m_got) == len(m_ref)
    coef = np.zeros(len(m_got), bool)
    o = 12 + 8 + 8 * (got["dim"] + 1) ** 2
    coef[12:o] = True
    for lv in (got["x"], got["y"]):
        o += 8
        for v in lv:
            coef[o + 8:o + 8 + 8 * len(v)] = True
            o += 8 + 8 * len(v)
    assert np.array_equal(m_got[~coef], m_ref[~coef])
    n = (2 ** depth + 1) ** got["dim"]
    for c, mine in enumerate(grids):
        want = g[f"grid{c}"].tobytes()
        assert mine[:-8 * n] == want[:-8 * n]
        a = np.frombuffer(mine[-8 * n:], "<f8")
        b = np.frombuffer(want[-8 * n:], "<f8")
        assert np.abs(a - b).max() <= 1e-8 * np.abs(b).max()


@pytest.mark.parametrize("flags,bound", [([], 1e-6), (HEADLINE, 0.1)])
def test_adaptive_zero_set_matches_reference(cli, flags, bound):
    """The zero curve of the command line's adaptive .tree (the reference's Extract computation:
    regular coefficients, marching simplices) against the reference Extract's zero set of the
    reference's own adaptive .tree, in FP64 and in the benchmark's precision configuration."""
    g = load_golden("link3_d5_a3_tree")
    simp = load_golden("cube_simplices")["simplices3"]
    with tempfile.TemporaryDirectory() as td:
        ply = os.path.join(td, "in.ply")
        samples.write_ply(ply, g["world_pos"], g["frames"])
        out = os.path.join(td, "out")
        r = subprocess.run([cli, "--in", ply, "--out", out, "--depth", str(int(g["depth"]))] + list(g["flags"]) + flags,
                           capture_output=True, text=True, timeout=300)
        assert r.returncode == 0, r.stderr
        with open(out + ".tree", "rb") as f:
            segs, cell = Z.tree_zero_set(f.read(), simp)
    ref = g["zero_vertices"][g["zero_simplices"]]
    d = Z.curve_hausdorff(segs, ref, cell / 10)
    assert d / cell <= bound, (d / cell, len(segs), len(ref))


@pytest.mark.parametrize("dim,depth,workload,n,K,solve", [(3, 6, "link", 60000, 2, True), (4, 4, "clifford", 60000, 1, False)])
def test_adaptive_against_oracle_larger(dim, depth, workload, n, K, solve):
    """The adaptive indexer beyond the fixtures' sizes against the oracle's restatement: index
    tables exactly, c and the system, two sweeps of the finest level, and (3D; the oracle's 4D
    solve takes minutes) the whole cascadic solve."""
    from oracle import oracle as O
    pos, frames = epr.samples.make_workload(workload, n, seed=11)
    pu, _ = epr.unit_cube(pos)
    sk = epr.pack_skew(frames)
    o = O.Oracle(dim, depth, adaptive_radius=K)
    o.set_samples(pu, sk)
    o.build()
    r = epr.Reconstructor(dim, depth, pu, sk, aRadius=K)
    for l in range(depth + 1):
        t = r.adaptive_index(l)
        assert t["active"] == int(o.get("nactive", l)[0])
        assert np.array_equal(t["fnodes"], o.get("fnodes", l).astype(np.int64)), l
        assert np.array_equal(t["enodes"], o.get("enodes", l).astype(np.int64)), l
    assert abs(r.get("c")[0] - o.get("c")[0]) < 1e-12 * o.get("c")[0]
    for l in (depth, depth - 1, 0):
        assert rel(r.get("B", l), o.get("B", l)) < 1e-11
        assert rel(r.get("R", l), o.get("R", l)) < 1e-10
    rng = np.random.default_rng(1)
    x = rng.uniform(-1, 1, o.nodes(depth))
    y = rng.uniform(-1, 1, o.nodes(depth))
    gx, gy = r.gs(depth, x, y, 2)
    ox, oy = o.gs(depth, x, y, 2)
    assert rel(gx, ox) < 1e-10 and rel(gy, oy) < 1e-10
    if not solve:
        return
    st = r.solve()
    xs, ys, e = o.solve()
    assert abs(st["fit_energy"] - e[1]) < 1e-10 * e[1]
    assert abs(st["reg_energy"] - e[2]) < 1e-10 * e[2]
    gxs, gys = r.solution()
    for l in range(depth + 1):
        assert rel(gxs[l], xs[l]) < 1e-8
        assert rel(gys[l], ys[l]) < 1e-8
