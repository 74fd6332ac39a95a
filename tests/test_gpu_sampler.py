"""Samples generated on the GPU (epr_generate_samples / epr_set_generated_samples): the shapes are
the host generator's formulas, the noise has the requested statistics, the output is a function of
the seed, and samples set on the device give the build the host path gives for the same points.

Tolerances: shapes against the host formulas 1e-13 absolute (unit-size coordinates); noise
statistics 2 % (1e5 samples)."""
import numpy as np
import pytest

import exteriorpoissonrecon_gb300 as epr

pytestmark = pytest.mark.gpu


def test_regular_knot_matches_host_formulas():
    n = 4096
    pos, skew = epr.generate_samples(epr.sampler("knot", 2, 3, regular=True), n)
    hp, hf = epr.samples.torus_knot(n, 2, 3, regular=True)
    assert np.abs(pos - hp).max() < 1e-13
    assert np.abs(skew - epr.pack_skew(hf)).max() < 1e-13


def test_clifford_points_and_frames():
    pos, skew = epr.generate_samples(epr.sampler("clifford", seed=4), 20000)
    assert np.abs(pos[:, 0] ** 2 + pos[:, 1] ** 2 - 0.5).max() < 1e-14
    assert np.abs(pos[:, 2] ** 2 + pos[:, 3] ** 2 - 0.5).max() < 1e-14
    z = np.zeros(len(pos))
    du = np.stack([-pos[:, 1], pos[:, 0], z, z], axis=1)
    dv = np.stack([z, z, -pos[:, 3], pos[:, 2]], axis=1)
    assert np.abs(skew - epr.pack_skew(epr.samples.bivector_frames(du, dv))).max() < 1e-13


def test_seeded_and_launch_independent():
    sp = epr.sampler("helix", 5.0, pos_sigma=0.01, angle_deg=10.0, spot_frac=0.1, seed=7)
    a = epr.generate_samples(sp, 10000)
    b = epr.generate_samples(sp, 10000)
    assert np.array_equal(a[0], b[0]) and np.array_equal(a[1], b[1])
    sp.seed = 8
    c = epr.generate_samples(sp, 10000)
    assert not np.array_equal(a[0], c[0])
    # sample i does not depend on how many samples are drawn (before the outliers, whose box moves)
    sp.seed = 7
    sp.spot_frac = 0.0
    sp.pos_sigma = 0.0
    d = epr.generate_samples(sp, 5000)
    e = epr.generate_samples(sp, 10000)
    assert np.array_equal(d[0], e[0][:5000]) and np.array_equal(d[1], e[1][:5000])


def test_noise_statistics():
    n = 100000
    clean = epr.generate_samples(epr.sampler("link", seed=3), n)
    sigma = 0.005
    noisy = epr.generate_samples(epr.sampler("link", pos_sigma=sigma, angle_deg=5.0, seed=3), n)
    scale = (clean[0].max(axis=0) - clean[0].min(axis=0)).max() * 1.1
    d = noisy[0] - clean[0]
    assert np.all(np.abs(d.mean(axis=0)) < 0.02 * sigma * scale)
    assert np.all(np.abs(d.std(axis=0) / (sigma * scale) - 1) < 0.02)
    # rotations keep the frames' norms; the frame changes are of the requested angle's size
    nc = np.linalg.norm(clean[1], axis=1)
    nn = np.linalg.norm(noisy[1], axis=1)
    assert np.abs(nn - nc).max() < 1e-13
    rel = np.linalg.norm(noisy[1] - clean[1], axis=1) / nc
    assert 0.3 * np.radians(5.0) < np.median(rel) < 3 * np.radians(5.0)
    # outliers: inside the noisy samples' box, frames S - S^T of entries in [-1, 1]
    sp = epr.sampler("link", pos_sigma=sigma, spot_frac=0.1, seed=3)
    pos, skew = epr.generate_samples(sp, n)
    assert len(pos) == n + n // 10
    lo, hi = pos[:n].min(axis=0), pos[:n].max(axis=0)
    assert np.all(pos[n:] >= lo) and np.all(pos[n:] <= hi)
    assert np.abs(skew[n:]).max() <= 2.0 and np.abs(skew[n:]).max() > 1.5


def test_generated_samples_build_like_host_samples():
    """On-device generation + unit-cube map gives the build of the same samples mapped on the host."""
    sp = epr.sampler("link", pos_sigma=0.005, angle_deg=5.0, spot_frac=0.1, seed=11)
    n = 50000
    pos, skew = epr.generate_samples(sp, n)
    pu, xf_host = epr.unit_cube(pos)
    r_host = epr.Reconstructor(3, 5, pu, skew)
    r_dev = epr.Reconstructor(3, 5)
    xf_dev = r_dev.set_generated_samples(sp, n)
    r_dev.build()
    assert np.array_equal(xf_dev, xf_host)
    assert np.array_equal(r_dev.get("measure"), r_host.get("measure"))
    assert np.array_equal(r_dev.get("B", 5), r_host.get("B", 5))
    s1, s2 = r_dev.solve(), r_host.solve()
    assert s1["fit_energy"] == s2["fit_energy"] and s1["reg_energy"] == s2["reg_energy"]
    with pytest.raises(epr.EprError, match="4D"):
        epr.Reconstructor(3, 3).set_generated_samples(epr.sampler("clifford"), 100)
