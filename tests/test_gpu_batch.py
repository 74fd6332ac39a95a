"""Batched reconstructions (epr_batch_solve): several independent reconstructions of uneven
sizes, depths, dims and precisions built and solved concurrently on one GPU give exactly what each
gives alone, and a reconstruction inside a batch still matches the reference's golden solve."""
import numpy as np
import pytest

import exteriorpoissonrecon_gb300 as epr
from conftest import load_golden

pytestmark = pytest.mark.gpu


def _inputs():
    """A small mix: knots and helices of the batched workload at depths 3-5, a 4D Clifford torus,
    an FP32 run with the double band, and the golden knot of the reference."""
    items = []
    for w in epr.samples.batch_workloads(6, seed=3, n_range=(2000, 40000), depths=(3, 4, 5)):
        pu, _ = epr.unit_cube(w["pos"])
        items.append(dict(dim=3, depth=w["depth"], pos=pu, skew=epr.pack_skew(w["frames"]), kw={}))
    pos, fr = epr.samples.make_workload("clifford", 20000, seed=5)
    pu, _ = epr.unit_cube(pos)
    items.append(dict(dim=4, depth=3, pos=pu, skew=epr.pack_skew(fr), kw={}))
    items.append(dict(items[0], kw=dict(precision="fp32", fp64_from=2, fp64_levels=4)))
    items.append(dict(items[1], kw=dict(precision="fp32", fp64_from=0, fp64_levels=4, band_precision="df")))
    g = load_golden("knot3_d4")
    items.append(dict(dim=3, depth=int(g["depth"]), pos=g["pos"], skew=g["skew"], kw={}))
    return items, g


def _recon(it, build):
    return epr.Reconstructor(it["dim"], it["depth"], it["pos"], it["skew"], build=build, **it["kw"])


def _result(r, st):
    xs, ys = r.solution()
    return np.concatenate(xs), np.concatenate(ys), st["fit_energy"], st["reg_energy"]


def test_batch_matches_individual_solves():
    items, g = _inputs()
    alone = []
    for it in items:
        r = _recon(it, True)
        alone.append(_result(r, r.solve()))
        r.close()
    recons = [_recon(it, False) for it in items]
    # the first batch solve launches directly, the second captures every context's graph
    for rnd in range(2):
        stats = epr.batch_solve(recons, build=(rnd == 0), threads=4)
        for k, (r, st) in enumerate(zip(recons, stats)):
            got = _result(r, st)
            assert np.array_equal(got[0], alone[k][0]) and np.array_equal(got[1], alone[k][1]), (rnd, k)
            assert got[2] == alone[k][2] and got[3] == alone[k][3], (rnd, k)
    # the golden member against the reference's own solve
    ref = g["sol_energies"]
    st = recons[-1].stats.as_dict()
    assert abs(st["fit_energy"] - ref[0]) < 1e-10 * ref[0]
    assert abs(st["reg_energy"] - ref[1]) < 1e-10 * ref[1]
    for r in recons:
        r.close()


@pytest.mark.parametrize("threads", [1, 3, 16])
def test_batch_thread_counts(threads):
    """The schedule does not change the results: any number of workers gives the same bits."""
    items, _ = _inputs()
    items = items[:4]
    outs = []
    for t in (threads, 2):
        recons = [_recon(it, False) for it in items]
        stats = epr.batch_solve(recons, build=True, threads=t)
        outs.append([_result(r, s) for r, s in zip(recons, stats)])
        for r in recons:
            r.close()
    for a, b in zip(*outs):
        assert np.array_equal(a[0], b[0]) and np.array_equal(a[1], b[1]) and a[2:] == b[2:]


def test_batch_reports_the_failing_context():
    """A context without samples fails its build with EPR_ERR_STATE; the others still solve."""
    items, _ = _inputs()
    good = [_recon(it, False) for it in items[:2]]
    bad = epr.Reconstructor(3, 3)
    recons = [good[0], bad, good[1]]
    with pytest.raises(epr.EprError, match=r"context 1: .*before epr_set_samples"):
        epr.batch_solve(recons, build=True)
    for r in good:
        assert r.stats.fit_energy > 0
    handles = [good[0], good[0]]
    with pytest.raises(epr.EprError, match="twice"):
        epr.batch_solve(handles, build=False)
    for r in recons:
        r.close()


def test_rebuild_gives_the_same_system():
    """epr_build may run again on the same samples (it frees its earlier products first)."""
    items, _ = _inputs()
    it = items[1]
    r = _recon(it, True)
    b0, s0 = r.get("B", it["depth"]), r.get("S")
    r.build()
    assert np.array_equal(r.get("B", it["depth"]), b0) and np.array_equal(r.get("S"), s0)
    r.close()


# ---------------------------------------------------------------------------------------------
# lockstep batches (epr_batch_*): one launch per level colour for all members, one graph, tuned tiles
# ---------------------------------------------------------------------------------------------

def _lockstep_inputs(kw):
    """3D members of uneven depths (3-6, so that levels 2-6 run per-colour launches with members
    dropping out as their schedules end), sample counts and sweep counts, in one precision
    configuration, plus the reference's golden knot."""
    items = []
    for w in epr.samples.batch_workloads(7, seed=11, n_range=(2000, 60000), depths=(3, 4, 5, 6)):
        pu, _ = epr.unit_cube(w["pos"])
        items.append(dict(dim=3, depth=w["depth"], pos=pu, skew=epr.pack_skew(w["frames"]), kw=dict(kw)))
    items[1]["kw"]["gs_iters"] = 7  # another sweep count on every level
    items[2]["kw"]["separate"] = 1
    g = load_golden("knot3_d4")
    items.append(dict(dim=3, depth=int(g["depth"]), pos=g["pos"], skew=g["skew"], kw=dict(kw)))
    return items


@pytest.mark.parametrize("kw", [dict(precision="fp32", fp64_from=0, fp64_levels=4, band_precision="df"),
                                dict(precision="fp32", fp64_from=2, fp64_levels=4),
                                dict()], ids=["df_band", "fp64_band", "fp64"])
def test_lockstep_batch_matches_individual_solves(kw):
    items = _lockstep_inputs(kw)
    alone = []
    for it in items:
        r = _recon(it, True)
        alone.append(_result(r, r.solve()))
        r.close()
    recons = [_recon(it, False) for it in items]
    b = epr.LockstepBatch(recons, threads=4)
    try:
        # the first run builds and captures the graph, the second replays it, the third runs the
        # tuned block shapes (a new graph)
        for rnd in range(3):
            if rnd == 2:
                times = b.tune(reps=2)
                assert times.shape[1] == 3 and len(times) >= 1 and (times > 0).all()
                assert all(0 <= t <= 2 for t in b.info()["tiles"])
            stats = b.run(build=(rnd == 0))
            for k, (r, st) in enumerate(zip(recons, stats)):
                got = _result(r, st)
                assert np.array_equal(got[0], alone[k][0]) and np.array_equal(got[1], alone[k][1]), (rnd, k)
                assert got[2] == alone[k][2] and got[3] == alone[k][3], (rnd, k)
        info = b.info()
        assert info["relax_ms"] > 0 and info["graph_launches"] > 0
    finally:
        b.close()
        for r in recons:
            r.close()


def test_lockstep_batch_every_block_shape_gives_the_same_bits():
    """Each of the three block shapes of every per-colour level, forced by hand, gives the solo bits."""
    kw = dict(precision="fp32", fp64_from=0, fp64_levels=4, band_precision="df")
    items = _lockstep_inputs(kw)[:4]
    alone = []
    for it in items:
        r = _recon(it, True)
        alone.append(_result(r, r.solve()))
        r.close()
    lib = epr.load()
    for shape in range(3):
        recons = [_recon(it, True) for it in items]
        b = epr.LockstepBatch(recons, threads=2)
        b.set_tile(-1, shape)
        stats = b.run()
        assert all(t == shape for t in b.info()["tiles"]), b.info()
        for k, (r, st) in enumerate(zip(recons, stats)):
            got = _result(r, st)
            assert np.array_equal(got[0], alone[k][0]) and np.array_equal(got[1], alone[k][1]), (shape, k)
        b.close()
        for r in recons:
            r.close()
    with pytest.raises(epr.EprError):
        epr.LockstepBatch([_recon(items[0], True)]).set_tile(0, 3)
    assert lib is not None


def test_lockstep_batch_rejects_members_it_cannot_share():
    items = _lockstep_inputs({})[:2]
    pos, fr = epr.samples.make_workload("clifford", 3000, seed=5)
    pu, _ = epr.unit_cube(pos)
    four = epr.Reconstructor(4, 2, pu, epr.pack_skew(fr))
    three = _recon(items[0], True)
    mg = _recon(dict(items[1], kw=dict(solver="multigrid")), True)
    mixed = _recon(dict(items[1], kw=dict(precision="fp32")), True)
    try:
        for bad, msg in (([three, four], "3D"), ([three, mg], "cascadic"), ([three, mixed], "arithmetic")):
            b = epr.LockstepBatch(bad)
            with pytest.raises(epr.EprError, match=msg):
                b.run()
            b.close()
        with pytest.raises(epr.EprError, match="twice"):
            epr.LockstepBatch([three, three])
    finally:
        for r in (four, three, mg, mixed):
            r.close()
