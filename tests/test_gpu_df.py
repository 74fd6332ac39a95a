"""Double-float coarse levels (band_precision = EPR_BAND_DF): the 3D levels up to 3 of a float
solve's band relax in pairs of floats with a power-of-two exponent per level.  They must track the
double path to far below float rounding, keep double's exponent range, and leave the cascadic solve
at the double band's energy.

Tolerances: a double-float sweep against the double sweep 1e-11 relative (48-bit arithmetic);
whole solves against the double band 1e-8 relative in energy."""
import numpy as np
import pytest

import exteriorpoissonrecon_gb300 as epr
from conftest import load_golden
from oracle import oracle as O

pytestmark = pytest.mark.gpu

DF = dict(precision="fp32", fp64_from=0, fp64_levels=4, band_precision="df")


def rel(a, b):
    a = np.asarray(a, dtype=np.float64).ravel()
    b = np.asarray(b, dtype=np.float64).ravel()
    return float(np.abs(a - b).max() / max(np.abs(b).max(), 1e-300))


@pytest.fixture(scope="module")
def link():
    g = load_golden("link3_d4")
    depth = int(g["depth"])
    r64 = epr.Reconstructor(3, depth, g["pos"], g["skew"], precision="fp64")
    rdf = epr.Reconstructor(3, depth, g["pos"], g["skew"], **DF)
    o = O.Oracle(3, depth)
    o.set_samples(g["pos"], g["skew"])
    o.build()
    return g, depth, r64, rdf, o


@pytest.mark.parametrize("level", [0, 1, 2, 3])
def test_df_sweeps_track_double(link, level):
    """Two paired-GS sweeps of a double-float level against the double kernels and the oracle."""
    g, depth, r64, rdf, o = link
    rng = np.random.default_rng(level)
    n = o.nodes(level)
    x, y = rng.uniform(-1, 1, n), rng.uniform(-1, 1, n)
    dx, dy = rdf.gs(level, x, y, 2)
    ex, ey = r64.gs(level, x, y, 2)
    ox, oy = o.gs(level, x, y, 2)
    assert rel(dx, ex) < 1e-11 and rel(dy, ey) < 1e-11
    assert rel(dx, ox) < 1e-11 and rel(dy, oy) < 1e-11
    # energies of a double-float level are evaluated in double from its coefficients
    e_df = rdf.energy(level, x, y)
    e_64 = r64.energy(level, x, y)
    assert rel(e_df, e_64) < 1e-12


@pytest.mark.parametrize("scale", [1e-30, 1e-45, 1e-60])
def test_df_exponent_keeps_tiny_coefficients(link, scale):
    """Coefficients far below float's range (the cascadic schedule drives coarse levels to 1e-59)
    keep their digits: the level's exponent carries the magnitude."""
    g, depth, r64, rdf, o = link
    level = 2
    rng = np.random.default_rng(7)
    n = o.nodes(level)
    x, y = scale * rng.uniform(-1, 1, n), scale * rng.uniform(-1, 1, n)
    dx, dy = rdf.gs(level, x, y, 3)
    ex, ey = r64.gs(level, x, y, 3)
    assert np.abs(ex).max() > 0
    assert rel(dx, ex) < 1e-11 and rel(dy, ey) < 1e-11


def test_df_band_solve_matches_double_band():
    """The cascadic solve with levels 2-3 in double-float ends at the double band's energy."""
    pos, fr = epr.samples.make_workload("link", 100000, seed=1)
    pu, _ = epr.unit_cube(pos)
    sk = epr.pack_skew(fr)
    e = {}
    for name, kw in [("fp64", dict(precision="fp64")),
                     ("band", dict(precision="fp32", fp64_from=2, fp64_levels=4)),
                     ("df", dict(precision="fp32", fp64_from=2, fp64_levels=4, band_precision="df"))]:
        r = epr.Reconstructor(3, 6, pu, sk, **kw)
        for _ in range(2):  # the second solve replays the captured graph
            st = r.solve()
        e[name] = st["fit_energy"] + st["reg_energy"]
        r.close()
    assert abs(e["df"] - e["band"]) < 1e-8 * e["band"]
    assert abs(e["df"] - e["fp64"]) < 1e-6 * e["fp64"]


def test_df_band_is_cascadic_3d_only():
    """Other solvers and 4D keep the band in double (the parameter is accepted and ignored there)."""
    g = load_golden("link3_d4")
    r = epr.Reconstructor(3, int(g["depth"]), g["pos"], g["skew"], solver="multigrid", max_cycles=2, **DF)
    st = r.solve()
    assert np.isfinite(st["fit_energy"])
    with pytest.raises(epr.EprError):
        epr.Reconstructor(3, 3, band_precision=7)

