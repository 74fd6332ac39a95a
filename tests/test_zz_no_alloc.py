"""The allocation-free energy entry point (epr_energy_noalloc) against the context's epr_energy.

Callers that cannot allocate device memory where they need an energy value (stream captures that
must stay free of allocation nodes, hosts whose memory belongs to an external pool, real-time
loops) pass their own device buffers; the library's reduction scratch is a fixed device array.
This file is collected last so that a failure here leaves every other test already run; it also
passes when run alone in a fresh process.  Tolerance: 1e-12 relative (FP64), as the other
energy parity tests."""
import ctypes

import numpy as np
import pytest

from conftest import load_golden

pytestmark = pytest.mark.gpu


def _device_stencil(torch, host_node_major, N, S):
    # node-major (N x S) host copy -> offset-major device buffer
    a = np.ascontiguousarray(host_node_major.reshape(N, S).T)
    return torch.tensor(a.ravel(), dtype=torch.float64, device="cuda")


def test_energy_noalloc_matches_context_energy_on_two_calls():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    import exteriorpoissonrecon_gb300 as epr

    g = load_golden("knot3_d4")
    depth = int(g["depth"])
    r = epr.Reconstructor(3, depth, g["pos"], g["skew"])
    lib = epr.load()
    c = float(r.get("c")[0])
    torch.cuda.init()
    stream = torch.cuda.current_stream().cuda_stream
    for level in (depth, depth - 2):  # two calls in a row, different sizes, same fixed scratch
        N = (2 ** level + 1) ** 3
        x, y = g[f"xr_d{level}"], g[f"yr_d{level}"]
        ref = r.energy(level, x, y)
        A = _device_stencil(torch, r.get("A", level), N, 27)
        B = _device_stencil(torch, r.get("B", level), N, 27)
        xy = torch.tensor(np.stack([x, y], axis=1).ravel(), dtype=torch.float64, device="cuda")
        out = torch.full((3,), float("nan"), dtype=torch.float64, device="cuda")
        rc = lib.epr_energy_noalloc(torch.cuda.current_device(), 3, level, epr.EPR_FP64, ctypes.c_void_p(xy.data_ptr()),
                                    ctypes.c_void_p(A.data_ptr()), ctypes.c_void_p(B.data_ptr()), c,
                                    ctypes.c_void_p(out.data_ptr()), ctypes.c_void_p(stream))
        assert rc == 0, lib.epr_noalloc_last_error().decode()
        torch.cuda.synchronize()
        got = out.cpu().numpy()
        for k in range(3):
            assert abs(got[k] - ref[k]) <= 1e-12 * abs(ref[k]) + 1e-14, (level, k, got, ref)


def test_energy_noalloc_rejects_bad_sizes():
    import exteriorpoissonrecon_gb300 as epr
    lib = epr.load()
    null = ctypes.c_void_p(0)
    rc = lib.epr_energy_noalloc(0, 3, 11, 0, null, null, null, 0.0, null, null)
    assert rc != 0 and b"level out of range" in lib.epr_noalloc_last_error()
    rc = lib.epr_energy_noalloc(0, 5, 3, 0, null, null, null, 0.0, null, null)
    assert rc != 0 and b"dim" in lib.epr_noalloc_last_error()
