"""Parity of the CUDA path (through the C ABI) against the reference's own outputs (golden
fixtures) and against the CPU oracle at larger sizes.

Tolerances: FP64 path 1e-12 relative for energies and stencils (1e-9 for the eigenvalue-based
noise and for quantities accumulated over whole solves); FP32 path 1e-5 relative."""
import numpy as np
import pytest

import exteriorpoissonrecon_gb300 as epr
from conftest import SOLVE_CASES, VARIANT_CASES, load_golden
from oracle import oracle as O

pytestmark = pytest.mark.gpu


def rel(a, b):
    a = np.asarray(a, dtype=np.float64).ravel()
    b = np.asarray(b, dtype=np.float64).ravel()
    assert a.shape == b.shape, (a.shape, b.shape)
    return float(np.abs(a - b).max() / max(np.abs(b).max(), 1e-300))


@pytest.fixture(scope="module", params=SOLVE_CASES)
def built(request):
    g = load_golden(request.param)
    dim = g["pos"].shape[1]
    depth = int(g["depth"])
    r = epr.Reconstructor(dim, depth, g["pos"], g["skew"])
    return g, r, dim, depth


def test_estimator(built):
    g, r, dim, depth = built
    assert rel(r.get("measure"), g["est_measure"]) < 1e-12
    assert rel(r.get("depth"), g["est_depth"]) < 1e-12
    assert rel(r.get("noise"), g["est_noise"]) < 1e-9


def test_density_estimator(built):
    """epr_get_density: the estimator's splatted weight, position and covariance sums at every
    level against the reference's tree (TreeEstimator, GridSamples.inl:740-771)."""
    g, r, dim, depth = built
    for l in range(depth + 1):
        assert rel(r.density(l), g[f"density_l{l}"]) < 1e-12, l


def test_frame_field(built):
    g, r, dim, depth = built
    assert np.array_equal(r.get("leaf_depth"), g["leaf_depth"])
    assert rel(r.get("S"), g["S"]) < 1e-12
    assert abs(r.get("c")[0] - g["c"][0]) < 1e-12 * g["c"][0]


def test_stencils(built):
    g, r, dim, depth = built
    for l in g["stencil_levels"]:
        assert rel(r.get("R", int(l)), g[f"R_d{l}"]) < 1e-10
        assert rel(r.get("B", int(l)), g[f"B_d{l}"]) < 1e-12


def test_energy_every_level(built):
    g, r, dim, depth = built
    for l in range(depth + 1):
        e = r.energy(l, g[f"xr_d{l}"], g[f"yr_d{l}"])
        ref = g[f"energies_d{l}"]
        for k in range(3):
            assert abs(e[k] - ref[k]) <= 1e-12 * abs(ref[k]) + 1e-14, (l, k, e, ref)


def test_quadfit_and_gs(built):
    g, r, dim, depth = built
    for key in g:
        if not key.startswith("quadfit_d"):
            continue
        l = int(key[len("quadfit_d"):])
        x, y = g[f"xr_d{l}"], g[f"yr_d{l}"]
        assert rel(r.quadfit(l, x, y), g[key]) < 1e-11
        gx, gy = r.gs(l, x, y, 1)
        assert rel(gx, g[f"gsx_d{l}"]) < 1e-11
        assert rel(gy, g[f"gsy_d{l}"]) < 1e-11


def test_gradient(built):
    """epr_gradient against the linear terms of the reference's quadraticFit (SystemEnergy.h:542-643):
    1e-11 in FP64; the FP32 context's float kernel within 1e-5."""
    g, r, dim, depth = built
    r32 = epr.Reconstructor(dim, depth, g["pos"], g["skew"], precision="fp32")
    for key in g:
        if not key.startswith("quadfit_d"):
            continue
        l = int(key[len("quadfit_d"):])
        x, y = g[f"xr_d{l}"], g[f"yr_d{l}"]
        gx, gy = r.gradient(l, x, y)
        assert rel(gx, g[key][:, 3]) < 1e-11 and rel(gy, g[key][:, 4]) < 1e-11
        fx, fy = r32.gradient(l, x, y)
        assert rel(fx, g[key][:, 3]) < 1e-5 and rel(fy, g[key][:, 4]) < 1e-5
    r32.close()


def test_cascadic_solve_matches_reference(built):
    g, r, dim, depth = built
    st = r.solve()
    ref = g["sol_energies"]
    assert abs(st["fit_energy"] - ref[0]) < 1e-10 * ref[0]
    assert abs(st["reg_energy"] - ref[1]) < 1e-10 * ref[1]
    xs, ys = r.solution()
    for l in range(depth + 1):
        assert rel(xs[l], g[f"solx_d{l}"]) < 1e-9
        assert rel(ys[l], g[f"soly_d{l}"]) < 1e-9


def test_fp32_operators(built):
    """FP32 smoothing path: energy and quadratic fits within 1e-5 of the reference."""
    g, _, dim, depth = built
    r = epr.Reconstructor(dim, depth, g["pos"], g["skew"], precision="fp32")
    l = depth
    x, y = g[f"xr_d{l}"], g[f"yr_d{l}"]
    e = r.energy(l, x, y)
    ref = g[f"energies_d{l}"]
    assert abs(e[2] - ref[2]) < 1e-5 * abs(ref[2])
    assert abs(e[0] + e[1] - ref[0] - ref[1]) < 1e-5 * abs(ref[0] + ref[1])
    assert rel(r.quadfit(l, x, y), g[f"quadfit_d{l}"]) < 1e-5


def test_system_upload_path():
    """epr_set_level_system + operators on an uploaded system (isolates the solve kernels)."""
    g = load_golden("knot3_d4")
    depth = int(g["depth"])
    r = epr.Reconstructor(3, depth)
    l = depth
    r.set_level_system(l, g[f"R_d{l}"], g[f"B_d{l}"], g["c"][0])
    e = r.energy(l, g[f"xr_d{l}"], g[f"yr_d{l}"])
    ref = g[f"energies_d{l}"]
    assert abs(e[0] - ref[0]) < 1e-12 * abs(ref[0])
    assert abs(e[1] - ref[1]) < 1e-12 * abs(ref[1])


@pytest.mark.parametrize("dim,depth,workload,n", [(3, 6, "link", 60000), (4, 4, "clifford", 60000)])
def test_against_oracle_larger(dim, depth, workload, n):
    """Build, energy, fits, gradient, sweeps and the Gauss-Newton product against the oracle on
    inputs larger than the fixtures: FP64 to 1e-10 - 1e-12, the FP32 kernels to 1e-5."""
    pos, frames = epr.samples.make_workload(workload, n, seed=11)
    pu, _ = epr.unit_cube(pos)
    sk = epr.pack_skew(frames)
    o = O.Oracle(dim, depth)
    o.set_samples(pu, sk)
    o.build()
    r = epr.Reconstructor(dim, depth, pu, sk)
    assert rel(r.get("measure"), o.get("measure")) < 1e-12
    assert rel(r.get("S"), o.get("S")) < 1e-11
    for l in (depth, depth - 1, 0):
        assert rel(r.get("B", l), o.get("B", l)) < 1e-11
        assert rel(r.get("R", l), o.get("R", l)) < 1e-10
    rng = np.random.default_rng(1)
    x = rng.uniform(-1, 1, o.nodes(depth))
    y = rng.uniform(-1, 1, o.nodes(depth))
    e = r.energy(depth, x, y)
    eo = o.energy(depth, x, y)
    assert rel(e, eo) < 1e-12
    q = r.quadfit(depth, x, y)
    assert rel(q, o.quadfit(depth, x, y)) < 1e-11
    gx, gy = r.gs(depth, x, y, 2)
    ox, oy = o.gs(depth, x, y, 2)
    assert rel(gx, ox) < 1e-10 and rel(gy, oy) < 1e-10
    dx = rng.uniform(-1, 1, o.nodes(depth))
    dy = rng.uniform(-1, 1, o.nodes(depth))
    r.set_coefficients(depth, x, y)
    mx, my = r.gn_matvec(depth, dx, dy)
    omx, omy = o.gn_matvec(depth, x, y, dx, dy)
    assert rel(mx, omx) < 1e-11 and rel(my, omy) < 1e-11
    ogx, ogy = o.gradient(depth, x, y)
    gx, gy = r.gradient(depth, x, y)
    assert rel(gx, ogx) < 1e-11 and rel(gy, ogy) < 1e-11
    # the float kernels (gradient = the fit's linear terms, Gauss-Newton product) within 1e-5
    r32 = epr.Reconstructor(dim, depth, pu, sk, precision="fp32")
    fx, fy = r32.gradient(depth, x, y)
    assert rel(fx, ogx) < 1e-5 and rel(fy, ogy) < 1e-5
    r32.set_coefficients(depth, x, y)
    fmx, fmy = r32.gn_matvec(depth, dx, dy)
    assert rel(fmx, omx) < 1e-5 and rel(fmy, omy) < 1e-5
    e32 = r32.energy(depth, x, y)
    # evaluated in double from the float context's coefficients (x, y rounded to float on upload)
    assert rel(e32, eo) < 1e-6
    r32.close()


def test_against_oracle_4d_depth5():
    """4D at depth 5 (33^4 = 1,185,921 nodes, 81-point stencils), the largest 4D size whose oracle
    comparison fits test time: the build (measure, S, B, R on three levels) and the energy in full,
    the quadratic fits, gradient and Gauss-Newton product at 3,000 sampled nodes (the oracle's
    per-node arithmetic; a whole 4D fit there takes minutes on the CPU).  FP64 to 1e-10 - 1e-12,
    the FP32 kernels to 1e-5."""
    dim, depth = 4, 5
    pos, frames = epr.samples.make_workload("clifford", 100000, seed=11)
    pu, _ = epr.unit_cube(pos)
    sk = epr.pack_skew(frames)
    o = O.Oracle(dim, depth)
    o.set_samples(pu, sk)
    o.build()
    r = epr.Reconstructor(dim, depth, pu, sk)
    assert rel(r.get("measure"), o.get("measure")) < 1e-12
    assert rel(r.get("S"), o.get("S")) < 1e-11
    for l in (depth, depth - 1, 0):
        assert rel(r.get("B", l), o.get("B", l)) < 1e-11
        assert rel(r.get("R", l), o.get("R", l)) < 1e-10
    rng = np.random.default_rng(1)
    N = o.nodes(depth)
    x, y = rng.uniform(-1, 1, N), rng.uniform(-1, 1, N)
    dx, dy = rng.uniform(-1, 1, N), rng.uniform(-1, 1, N)
    eo = o.energy(depth, x, y)
    assert rel(r.energy(depth, x, y), eo) < 1e-12
    idx = np.sort(rng.choice(N, 3000, replace=False))
    qo = o.quadfit_at(depth, x, y, idx)
    assert rel(r.quadfit(depth, x, y)[idx], qo) < 1e-11
    omx, omy = o.gn_matvec_at(depth, x, y, dx, dy, idx)
    r.set_coefficients(depth, x, y)
    mx, my = r.gn_matvec(depth, dx, dy)
    assert rel(mx[idx], omx) < 1e-11 and rel(my[idx], omy) < 1e-11
    r32 = epr.Reconstructor(dim, depth, pu, sk, precision="fp32")
    fx, fy = r32.gradient(depth, x, y)
    assert rel(fx[idx], qo[:, 3]) < 1e-5 and rel(fy[idx], qo[:, 4]) < 1e-5
    r32.set_coefficients(depth, x, y)
    fmx, fmy = r32.gn_matvec(depth, dx, dy)
    assert rel(fmx[idx], omx) < 1e-5 and rel(fmy[idx], omy) < 1e-5
    r32.close()
    r.close()


@pytest.mark.parametrize("name", VARIANT_CASES)
def test_solver_variants(name):
    """--separate, --singleLevel and seed/minSolveDepth/iMult schedules against the reference, on the
    regular grid and with the adaptive indexer (whose narrow bands accumulate the different order of
    the FP64 sums a little further: coefficients at 1e-8)."""
    from conftest import variant_params
    g = load_golden(name)
    depth = int(g["depth"])
    r = epr.Reconstructor(3, depth, g["pos"], g["skew"], **variant_params(g["flags"]))
    st = r.solve()
    ref = g["sol_energies"]
    assert abs(st["fit_energy"] - ref[0]) < 1e-10 * ref[0]
    assert abs(st["reg_energy"] - ref[1]) < 1e-10 * ref[1]
    tol = 1e-8 if "--aRadius" in [str(f) for f in g["flags"]] else 1e-9
    xs, ys = r.solution()
    for l in range(depth + 1):
        assert rel(xs[l], g[f"solx_d{l}"]) < tol
        assert rel(ys[l], g[f"soly_d{l}"]) < tol


@pytest.mark.parametrize("precision", ["fp64", "fp32"])
def test_repeated_solves_are_identical(precision):
    """The first solve of a context launches directly, the second captures the relaxation sequence
    into a CUDA graph and later ones replay it: all give bitwise the same solution."""
    g = load_golden("link3_d4")
    r = epr.Reconstructor(3, int(g["depth"]), g["pos"], g["skew"], precision=precision)
    sols = []
    for _ in range(3):
        st = r.solve()
        xs, ys = r.solution()
        sols.append((np.concatenate(xs), np.concatenate(ys), st["fit_energy"], st["reg_energy"]))
    for s in sols[1:]:
        assert np.array_equal(s[0], sols[0][0]) and np.array_equal(s[1], sols[0][1])
        assert s[2] == sols[0][2] and s[3] == sols[0][3]


def test_double_band_keeps_the_double_minimum():
    """Float relaxation with levels 2-3 in double reaches the double run's energy (the cascadic
    solve leaves the zero stationary point on those levels, where float rounding would pick another
    local minimum)."""
    pos, fr = epr.samples.make_workload("link", 100000, seed=1)
    pu, _ = epr.unit_cube(pos)
    sk = epr.pack_skew(fr)
    e = {}
    for name, kw in [("fp64", dict(precision="fp64")), ("band", dict(precision="fp32", fp64_from=2, fp64_levels=4))]:
        r = epr.Reconstructor(3, 6, pu, sk, **kw)
        st = r.solve()
        e[name] = st["fit_energy"] + st["reg_energy"]
        r.close()
    assert abs(e["band"] - e["fp64"]) < 1e-6 * e["fp64"]


def _xy_rel_l2(x, y, X, Y):
    return float(np.sqrt(((x - X) ** 2 + (y - Y) ** 2).sum() / (X * X + Y * Y).sum()))


@pytest.mark.parametrize("band", ["df", "fp64"])
def test_full_size_mixed_precision_matches_double_run(band):
    """The benchmark's full size (3D link, 1.1M samples, depth 8, 257^3 nodes): FP32 relaxation
    with levels 0-3 in double-float (the benchmark's band) or in FP64 ends at the all-double run's
    energy to 1e-6 (both evaluated in FP64) and its finest grid within 1e-5 relative L2 of the
    double run's, every coarser level too; a repeated solve (graph replay) gives the same bits.
    Size-independent checks, as the oracle cannot run this size in test time."""
    pos, fr = epr.samples.make_workload("link", 1_000_000, seed=0)
    pu, _ = epr.unit_cube(pos)
    sk = epr.pack_skew(fr)
    r64 = epr.Reconstructor(3, 8, pu, sk, precision="fp64")
    s64 = r64.solve()
    e64 = s64["fit_energy"] + s64["reg_energy"]
    ref = [r64.coefficients(l) for l in range(9)]
    r64.close()
    r = epr.Reconstructor(3, 8, pu, sk, precision="fp32", fp64_from=0, fp64_levels=4, band_precision=band)
    s1 = r.solve()
    x1 = r.coefficients(8)
    s2 = r.solve()
    x2 = r.coefficients(8)
    e = s2["fit_energy"] + s2["reg_energy"]
    assert abs(e - e64) < 1e-6 * e64, (e, e64)
    assert s1["fit_energy"] == s2["fit_energy"] and np.array_equal(x1[0], x2[0]) and np.array_equal(x1[1], x2[1])
    assert s2["initial_energy"] == s64["initial_energy"]
    for l in range(9):
        xl = r.coefficients(l)
        assert _xy_rel_l2(xl[0], xl[1], *ref[l]) < 1e-5, l
    r.close()


def _edge_case(name):
    rng = np.random.default_rng(0)

    def frames(n):
        return epr.pack_skew(epr.samples.curve_frames(rng.normal(size=(n, 3))))

    if name == "one_sample":
        return np.array([[0.31, 0.52, 0.47]]), frames(1)
    if name == "two_in_one_cell":
        return np.array([[0.31, 0.52, 0.47], [0.312, 0.521, 0.471]]), frames(2)
    # samples on the faces and the far corner of the cube (keys clamped to the last cell)
    p = rng.uniform(0, 1, (200, 3))
    p[:20, 0] = 0.0
    p[20:40, 1] = 1.0
    p[40:50] = 1.0
    return p, frames(200)


@pytest.mark.parametrize("name", ["one_sample", "two_in_one_cell", "faces"])
def test_edge_inputs_match_oracle(name):
    """Inputs at the edges of the reference's sample handling: a single sample, coincident samples
    in one cell, samples on the cube's faces.  With one or two coincident samples the covariance is
    rank-deficient and its smallest eigenvalues are rounding noise, so the noise value itself is
    not reproducible across machines (the oracle gives 2.5 on x86 and -4.7e7 on Arm for the single
    sample); what the solve uses is the weight exp(-noise^2 / (2 nSigma^2)), which saturates there
    (0 and 1), and that is compared."""
    pu, sk = _edge_case(name)
    depth = 4
    o = O.Oracle(3, depth)
    o.set_samples(pu, sk)
    o.build()
    r = epr.Reconstructor(3, depth, pu, sk)
    assert rel(r.get("measure"), o.get("measure")) < 1e-12
    weight = lambda v: np.exp(-v * v / (2 * 0.25 * 0.25))
    if name == "faces":
        assert rel(r.get("noise"), o.get("noise")) < 1e-9
    with np.errstate(over="ignore"):
        assert np.abs(weight(r.get("noise")) - weight(o.get("noise"))).max() < 1e-10
    assert rel(r.get("S"), o.get("S")) < 1e-11
    for l in (depth, 0):
        assert rel(r.get("B", l), o.get("B", l)) < 1e-11
        # R is read back as A - dWeight K: where the weights vanish it is a rounding residue of A
        Rg, Ro = r.get("R", l), o.get("R", l)
        assert np.abs(Rg - Ro).max() <= 1e-10 * np.abs(Ro).max() + 1e-14
    st = r.solve()
    _, _, eo = o.solve()
    assert abs(st["fit_energy"] - eo[1]) < 1e-9 * eo[1] and abs(st["reg_energy"] - eo[2]) < 1e-9 * eo[2]


@pytest.mark.parametrize("name,tol", [("knot3_d4_project", 1e-12), ("cliff4_d3_project", 2e-5)])
def test_blade_projection(name, tol):
    """--project: S(E) on the GPU against the reference's FitBlade of every element, and the whole
    solve on the projected system against the oracle's.  (The reference's own solve with --project
    is not comparable: its projection draws random start vectors from rand() inside a parallel loop
    before the solve's random start is drawn from the same generator.)"""
    g = load_golden(name)
    dim, depth = g["pos"].shape[1], int(g["depth"])
    r = epr.Reconstructor(dim, depth, g["pos"], g["skew"], project=1)
    assert rel(r.get("S"), g["S_project"]) < tol
    if dim == 3:
        st = r.solve()
        o = O.Oracle(dim, depth, project=1)
        o.set_samples(g["pos"], g["skew"])
        o.build()
        xs, ys, e = o.solve()
        assert abs(st["fit_energy"] - e[1]) < 1e-10 * e[1]
        assert abs(st["reg_energy"] - e[2]) < 1e-10 * e[2]
        gx, gy = r.solution()
        for l in range(depth + 1):
            assert rel(gx[l], xs[l]) < 1e-9 and rel(gy[l], ys[l]) < 1e-9
    r.close()
