"""Failure handling through the C ABI (GPU): invalid arguments and out-of-order calls return the
documented status codes with a message, and the context stays usable afterwards.  Nothing here
faults the device: every rejection happens on the host before a launch."""
import ctypes

import numpy as np
import pytest

import exteriorpoissonrecon_gb300 as epr
from conftest import load_golden

pytestmark = pytest.mark.gpu

EPR_ERR_ARG, EPR_ERR_STATE = -1, -3


def code(exc):
    return int(str(exc).split("]")[0].strip("["))


def test_create_rejects_bad_configurations():
    L = epr.load()
    for dim, depth, kw in [(2, 4, {}), (3, 11, {}), (4, 8, {}), (3, 0, {}), (3, 4, {"tRadius": 5}),
                           (3, 4, {"precision": 7}), (3, 4, {"solver": 9}), (3, 4, {"solver": "multigrid", "max_cycles": -1})]:
        p = epr.default_params(**kw)
        h = L.epr_create(dim, depth, ctypes.byref(p))
        assert not h, (dim, depth, kw)
        assert L.epr_global_error().decode()


def test_bad_samples_and_order_of_calls():
    g = load_golden("knot3_d4")
    r = epr.Reconstructor(3, 4)
    with pytest.raises(epr.EprError) as e:
        r.build()
    assert code(e.value) == EPR_ERR_STATE
    with pytest.raises(epr.EprError) as e:
        r.solve()
    assert code(e.value) == EPR_ERR_STATE
    pos = g["pos"].copy()
    pos[5, 1] = np.nan
    with pytest.raises(epr.EprError) as e:
        r.set_samples(pos, g["skew"])
    assert code(e.value) == EPR_ERR_ARG and "non-finite" in str(e.value)
    sk = g["skew"].copy()
    sk[3, 0] = np.inf
    with pytest.raises(epr.EprError) as e:
        r.set_samples(g["pos"], sk)
    assert code(e.value) == EPR_ERR_ARG
    with pytest.raises(ValueError):
        r.set_samples(g["pos"][:, :2], g["skew"])
    # the context is still usable: the valid samples build and solve
    r.set_samples(g["pos"], g["skew"])
    r.build()
    st = r.solve()
    assert st["fit_energy"] + st["reg_energy"] < st["initial_energy"]
    with pytest.raises(epr.EprError) as e:
        r.energy(5)
    assert code(e.value) == EPR_ERR_ARG and "out of range" in str(e.value)
    with pytest.raises(epr.EprError) as e:
        r.prolong(4)
    assert code(e.value) == EPR_ERR_ARG
    with pytest.raises(epr.EprError) as e:
        r.time_kernel("nope", 4)
    assert code(e.value) == EPR_ERR_ARG


def test_degenerate_inputs():
    # all samples at one point: the unit-cube map divides by a zero extent, and the non-finite
    # positions are rejected before anything reaches the device
    pos = np.tile(np.array([[0.3, 0.4, 0.5]]), (10, 1))
    frames = np.zeros((10, 3, 3))
    frames[:, 0, 1], frames[:, 1, 0] = 1.0, -1.0
    try:
        with np.errstate(divide="ignore", invalid="ignore"):
            pu, _ = epr.unit_cube(pos)
    except ZeroDivisionError:
        pu = np.full_like(pos, np.nan)
    assert not np.isfinite(pu).all()
    r = epr.Reconstructor(3, 3)
    with pytest.raises(epr.EprError) as e:
        r.set_samples(pu, epr.pack_skew(frames))
    assert code(e.value) == EPR_ERR_ARG


def test_allocation_cap_fails_like_out_of_memory(monkeypatch):
    """Host-side fault injection of device out-of-memory: with EPR_ALLOC_CAP_BYTES set, the context
    whose allocations exceed the cap fails with EPR_ERR_NOMEM and a message, nothing is left
    half-built, and a context created without the cap works."""
    import exteriorpoissonrecon_gb300 as epr
    g = load_golden("knot3_d4")
    monkeypatch.setenv("EPR_ALLOC_CAP_BYTES", str(3 << 20))  # the context fits (2.7 MB), its build does not
    r = epr.Reconstructor(3, 4)
    r.set_samples(g["pos"], g["skew"])
    with pytest.raises(epr.EprError) as e:
        r.build()
    assert "[-5]" in str(e.value) and "allocation cap" in str(e.value)
    r.close()
    monkeypatch.setenv("EPR_ALLOC_CAP_BYTES", "1000")  # below what the context itself needs
    with pytest.raises(epr.EprError) as e:
        epr.Reconstructor(3, 4)
    assert "allocation cap" in str(e.value)
    monkeypatch.delenv("EPR_ALLOC_CAP_BYTES")
    r = epr.Reconstructor(3, 4, g["pos"], g["skew"])
    st = r.solve()
    assert abs(st["fit_energy"] - g["sol_energies"][0]) < 1e-10 * g["sol_energies"][0]
