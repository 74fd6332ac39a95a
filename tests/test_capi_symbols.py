"""CPU-side checks of the C ABI: the library builds for sm_103a, loads, and exports every function
that include/epr.h declares (no CUDA calls are made)."""
import ctypes

import exteriorpoissonrecon_gb300 as epr


def test_header_declares_the_boundary():
    names = epr.header_symbols()
    for required in ["epr_create", "epr_set_samples", "epr_build", "epr_solve", "epr_energy", "epr_quadfit",
                     "epr_gradient", "epr_gs", "epr_gn_matvec", "epr_get_solution", "epr_destroy", "epr_last_error"]:
        assert required in names


def test_library_exports_every_declared_symbol():
    lib = epr.load()
    missing = [n for n in epr.header_symbols() if not hasattr(lib, n)]
    assert not missing, missing


def test_params_struct_matches_defaults():
    p = epr.default_params()
    assert p.s_weight == 100.0 and p.d_weight == 0.00625 and p.n_sigma == 0.25 and p.i_mult == 2.0
    assert p.t_radius == 1 and p.d_radius == 1 and p.gs_iters == 10 and p.seed == 0
    assert p.max_solve_depth == -1 and p.precision == epr.EPR_FP64
    q = epr.default_params(sWeight=50, gsIters=20, precision="fp32")
    assert q.s_weight == 50 and q.gs_iters == 20 and q.precision == epr.EPR_FP32
    assert p.band_precision == epr.EPR_BAND_FP64
    assert epr.default_params(band_precision="df").band_precision == epr.EPR_BAND_DF
    assert ctypes.sizeof(epr.Params) == 128  # warm start, extra-sweep cap, target energy and projection after band_precision


def test_line_searches_host_only():
    """stepSize / newtonUpdate are host arithmetic in the library (no CUDA call): they reproduce the
    reference's values for the reference's own bi-quadratic fits."""
    import numpy as np
    from conftest import GOLDEN_CASES, load_golden
    for name in GOLDEN_CASES:
        g = load_golden(name)
        q = g["qa_biquad"]
        assert abs(epr.step_size(q) - g["qa_step"][0]) <= 1e-10 * abs(g["qa_step"][0])
        assert np.abs(epr.newton_update(q, 10) - g["qa_newton"]).max() <= 1e-10 * np.abs(g["qa_newton"]).max()
    # a cubic derivative with a single real root and one whose constant term vanishes
    q = np.zeros((3, 3))
    q[2, 2], q[1, 0] = 1.0, -1.0
    assert abs(epr.step_size(q) - 0.25 ** (1 / 3)) < 1e-14  # argmin of s^4 - s
    q = np.zeros((3, 3))
    q[2, 0], q[0, 2] = 1.0, 1.0
    assert epr.step_size(q) == 0.0


def test_batch_argument_checks_host_only():
    """epr_batch_solve validates its arguments before touching a context or the GPU."""
    import ctypes
    lib = epr.load()
    st = (epr.Stats * 2)()
    status = (ctypes.c_int * 2)()
    assert lib.epr_batch_solve(None, 0, 1, 0, st, status) == epr.EPR_OK
    assert lib.epr_batch_solve(None, 2, 1, 0, st, status) == -1
    assert lib.epr_batch_solve(None, -1, 1, 0, st, status) == -1
    handles = (ctypes.c_void_p * 2)(None, None)
    assert lib.epr_batch_solve(handles, 2, 1, 0, st, status) == -1
    assert b"null context" in lib.epr_global_error()


def test_sampler_arguments_host_only():
    """epr_generate_samples checks its arguments and reports the output size without the GPU."""
    import ctypes
    lib = epr.load()
    total = ctypes.c_size_t(0)
    sp = epr.sampler("link", pos_sigma=0.005, spot_frac=0.1)
    assert lib.epr_generate_samples(0, ctypes.byref(sp), 1000, None, None, ctypes.byref(total)) == epr.EPR_OK
    assert total.value == 1100
    assert lib.epr_generate_samples(0, None, 1000, None, None, ctypes.byref(total)) == -1
    assert lib.epr_generate_samples(0, ctypes.byref(sp), 0, None, None, ctypes.byref(total)) == -1
    bad = epr.sampler("knot")
    bad.shape = 9
    assert lib.epr_generate_samples(0, ctypes.byref(bad), 10, None, None, ctypes.byref(total)) == -1
    neg = epr.sampler("helix", pos_sigma=-1.0)
    assert lib.epr_generate_samples(0, ctypes.byref(neg), 10, None, None, ctypes.byref(total)) == -1
    assert b"non-negative" in lib.epr_global_error()
