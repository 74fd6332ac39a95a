"""Pins the adaptive indexer of the CPU restatement (the function and element sets of
Hat::HierarchicalAdaptedIndexer, Hat.adaptive.inl:342-732, on the dense level grids) against fixtures
the reference wrote: its index tables, system, energies, fits, one sweep, prolongation and cascadic
solve (tests/golden/make_golden.py ADAPTIVE), and its command line's own adaptive .tree files."""
import numpy as np
import pytest

from conftest import ADAPTIVE_CASES, ADAPTIVE_TREES, load_golden
from oracle import adapted_tree as AT
from oracle import density_tree as DT
from oracle import oracle as O


def rel(a, b):
    a = np.asarray(a, dtype=np.float64).ravel()
    b = np.asarray(b, dtype=np.float64).ravel()
    assert a.shape == b.shape
    return float(np.abs(a - b).max() / max(np.abs(b).max(), 1e-300))


_BUILT = {}


def _built(name):
    if name not in _BUILT:
        g = load_golden(name)
        dim = g["pos"].shape[1]
        depth = int(g["depth"])
        o = O.Oracle(dim, depth, adaptive_radius=int(g["a_radius"]))
        o.set_samples(g["pos"], g["skew"])
        o.build()
        _BUILT[name] = (g, o, dim, depth)
    return _BUILT[name]


@pytest.fixture(scope="module", params=ADAPTIVE_CASES)
def case(request):
    return _built(request.param)


def test_index_tables(case):
    """active functions in the tree's depth-first (Morton) order, then the inactive indexed ones and
    the elements in the order the indexer's finalisation discovers them"""
    g, o, dim, depth = case
    for l in range(depth + 1):
        assert int(o.get("nactive", l)[0]) == int(g[f"aact_d{l}"][0])
        assert np.array_equal(o.get("fnodes", l).astype(np.int64), g[f"afn_d{l}"]), l
        assert np.array_equal(o.get("enodes", l).astype(np.int64), g[f"ael_d{l}"]), l
        st = o.get("status", l)
        fn = g[f"afn_d{l}"]
        na = int(g[f"aact_d{l}"][0])
        assert (st[fn[:na]] == 2).all() and (st[fn[na:]] == 1).all()
        assert int((st > 0).sum()) == len(fn)


def test_system(case):
    g, o, dim, depth = case
    assert abs(o.get("c")[0] - g["c"][0]) < 1e-12 * g["c"][0]
    for l in g["stencil_levels"]:
        # R carries the noise weights, whose eigenvalues come from a different solver
        assert rel(o.get("R", int(l)), g[f"R_d{l}"]) < 1e-10
        assert rel(o.get("B", int(l)), g[f"B_d{l}"]) < 1e-12


def test_energies_fits_sweep_prolongation(case):
    g, o, dim, depth = case
    for l in range(depth + 1):
        x, y = g[f"xr_d{l}"], g[f"yr_d{l}"]
        e = o.energy(l, x, y)
        ref = g[f"energies_d{l}"]
        for k in range(3):
            assert abs(e[k] - ref[k]) <= 1e-12 * abs(ref[k]) + 1e-14, (l, k, e, ref)
        if l < depth:
            assert rel(o.prolong(l, x), g[f"prolong_d{l}"]) < 1e-15
        if f"quadfit_d{l}" in g:
            na = int(g[f"aact_d{l}"][0])
            active = g[f"afn_d{l}"][:na]
            assert rel(o.quadfit(l, x, y)[active], g[f"quadfit_d{l}"]) < 1e-11
            gx, gy = o.gs(l, x, y, 1)
            assert rel(gx, g[f"gsx_d{l}"]) < 1e-11
            assert rel(gy, g[f"gsy_d{l}"]) < 1e-11


def test_cascadic_solve(case):
    g, o, dim, depth = case
    xs, ys, e = o.solve()
    ref = g["sol_energies"]
    assert abs(e[1] - ref[0]) < 1e-10 * ref[0]
    assert abs(e[2] - ref[1]) < 1e-10 * ref[1]
    for l in range(depth + 1):
        assert rel(xs[l], g[f"solx_d{l}"]) < 1e-9
        assert rel(ys[l], g[f"soly_d{l}"]) < 1e-9


@pytest.mark.parametrize("name", sorted(ADAPTIVE_TREES))
def test_reference_tree_file(name):
    """The reference command line's adaptive .tree: its header, the indexer's tree (every node's
    depth, offset, children and function / element index), the per-level counts and the solution in
    the indexer's order all follow from the restatement."""
    import exteriorpoissonrecon_gb300 as epr
    g = load_golden(name)
    t = AT.parse(g["tree"].tobytes())
    dim, depth, K = t["dim"], int(g["depth"]), ADAPTIVE_TREES[name]
    assert t["hash"] == AT.HASH[dim]
    pos, _ = O.unit_cube(g["world_pos"])
    flags = [str(f) for f in g["flags"]]
    kw = {"gs_iters": int(flags[flags.index("--gsIters") + 1])} if "--gsIters" in flags else {}
    o = O.Oracle(dim, depth, adaptive_radius=K, **kw)
    o.set_samples(pos, epr.pack_skew(g["frames"]))
    o.build()
    fn = [o.get("fnodes", l).astype(np.int64) for l in range(depth + 1)]
    en = [o.get("enodes", l).astype(np.int64) for l in range(depth + 1)]
    na = [int(o.get("nactive", l)[0]) for l in range(depth + 1)]
    assert t["active"].tolist() == na
    assert t["functions"].tolist() == [len(f) for f in fn]
    assert t["elements"].tolist() == [len(e) for e in en]
    cells = o.get("cells").astype(np.int64).reshape(-1, dim)
    d, off, has = DT.nodes(dim, AT.refinement(dim, depth, K, cells, fn, na))
    assert np.array_equal(d, t["depth"]) and np.array_equal(off, t["offset"]) and np.array_equal(has, t["has_children"])
    fi, ei = AT.node_indices(dim, d, off, fn, en)
    assert np.array_equal(fi, t["findex"]) and np.array_equal(ei, t["eindex"])
    xs, ys, _ = o.solve()
    for l in range(depth + 1):
        assert rel(xs[l][fn[l]], t["x"][l]) < 1e-9
        assert rel(ys[l][fn[l]], t["y"][l]) < 1e-9
