"""The allocation-free energy entry point (epr_energy_noalloc) against the reference's energies.

Callers that cannot allocate device memory where they need an energy value (stream captures that
must stay free of allocation nodes, hosts whose memory belongs to an external pool, real-time
loops) pass their own device buffers; the library's reduction scratch is a fixed device array.
Each case makes two calls in a row on levels of different sizes (the fixed array keeps the first
call's contents) and compares both with the energies the reference computed on the same
coefficients (golden fixtures written by the reference's own code), and with the context's
epr_energy.  Tolerances: 1e-12 relative in FP64, 1e-5 in FP32, as the other energy parity tests.
This file is collected last so that a failure here leaves every other test already run; it also
passes when run alone in a fresh process."""
import ctypes

import numpy as np
import pytest

from conftest import load_golden

pytestmark = pytest.mark.gpu


def _device(torch, host, dtype):
    return torch.tensor(np.ascontiguousarray(host).ravel(), dtype=dtype, device="cuda")


@pytest.mark.parametrize("case,precision", [("knot3_d4", "fp64"), ("knot3_d4", "fp32"),
                                            ("cliff4_d3", "fp64"), ("cliff4_d3", "fp32")])
def test_energy_noalloc_matches_reference_on_two_calls(case, precision):
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    import exteriorpoissonrecon_gb300 as epr

    g = load_golden(case)
    dim = g["pos"].shape[1]
    depth = int(g["depth"])
    S = 3 ** dim
    r = epr.Reconstructor(dim, depth, g["pos"], g["skew"])
    lib = epr.load()
    c = float(r.get("c")[0])
    fp32 = precision == "fp32"
    dtype = torch.float32 if fp32 else torch.float64
    tol = 1e-5 if fp32 else 1e-12
    torch.cuda.init()
    device = torch.cuda.current_device()
    stream = torch.cuda.current_stream().cuda_stream
    for level in (depth, depth - 2):
        N = (2 ** level + 1) ** dim
        x, y = g[f"xr_d{level}"], g[f"yr_d{level}"]
        ref = g[f"energies_d{level}"]
        ctx = r.energy(level, x, y)
        # node-major host stencils -> offset-major device buffers
        A = _device(torch, r.get("A", level).reshape(N, S).T, dtype)
        B = _device(torch, r.get("B", level).reshape(N, S).T, dtype)
        xy = _device(torch, np.stack([x, y], axis=1), dtype)
        out = torch.full((3,), float("nan"), dtype=torch.float64, device="cuda")
        rc = lib.epr_energy_noalloc(device, dim, level, epr.EPR_FP32 if fp32 else epr.EPR_FP64,
                                    ctypes.c_void_p(xy.data_ptr()), ctypes.c_void_p(A.data_ptr()),
                                    ctypes.c_void_p(B.data_ptr()), c, ctypes.c_void_p(out.data_ptr()),
                                    ctypes.c_void_p(stream))
        assert rc == 0, lib.epr_noalloc_last_error().decode()
        assert torch.cuda.current_device() == device
        torch.cuda.synchronize()
        got = out.cpu().numpy()
        for k in range(3):
            assert abs(got[k] - ref[k]) <= tol * abs(ref[k]) + 1e-14, (level, k, got, ref)
            assert abs(got[k] - ctx[k]) <= tol * abs(ctx[k]) + 1e-14, (level, k, got, ctx)


def test_energy_noalloc_rejects_bad_sizes():
    import exteriorpoissonrecon_gb300 as epr
    lib = epr.load()
    null = ctypes.c_void_p(0)
    rc = lib.epr_energy_noalloc(0, 3, 11, 0, null, null, null, 0.0, null, null)
    assert rc != 0 and b"level out of range" in lib.epr_noalloc_last_error()
    rc = lib.epr_energy_noalloc(0, 4, 8, 0, null, null, null, 0.0, null, null)
    assert rc != 0 and b"level out of range" in lib.epr_noalloc_last_error()
    rc = lib.epr_energy_noalloc(0, 5, 3, 0, null, null, null, 0.0, null, null)
    assert rc != 0 and b"dim" in lib.epr_noalloc_last_error()
