"""The learned warm start's tensor-core kernels and network against the CPU oracle
(oracle/unet_oracle.py), through the C ABI.

Tolerances: the convolution primitives take BF16 operands exactly and accumulate in FP32, so the
forward and data-gradient outputs (stored in BF16) are within one BF16 rounding (2^-8 relative) of
the oracle's float64 sums of the same operands, and the FP32 weight gradient within 1e-4 relative;
the whole network's loss and parameter gradients, with the oracle rounding to BF16 where the GPU
stores BF16, within 2e-2 relative in norm per layer's weights and 5e-2 per layer's biases (bias
gradients are sums of cancelling BF16 values; rounding-boundary flips of BF16 intermediates move
individual values by one BF16 step)."""
import ctypes

import numpy as np
import pytest

from oracle import unet_oracle as U

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def torch():
    t = pytest.importorskip("torch")
    if not t.cuda.is_available():
        pytest.skip("no CUDA device")
    t.cuda.init()
    return t


def _dev_bf16(torch, a):
    return torch.tensor(np.ascontiguousarray(a, dtype=np.float32), device="cuda").to(torch.bfloat16).contiguous()


def _ptr(t):
    return ctypes.c_void_p(t.data_ptr())


def _kmajor(W):
    """(27, Cin, Cout) -> (Cout, 27 Cin) with column t * Cin + ci."""
    return np.ascontiguousarray(W.transpose(2, 0, 1).reshape(W.shape[2], -1))


@pytest.mark.parametrize("n,cin,cout", [(9, 16, 16), (17, 32, 64), (9, 192, 64), (9, 64, 192), (5, 48, 96), (17, 16, 128)])
def test_conv_forward_and_data_gradient(torch, n, cin, cout):
    import exteriorpoissonrecon_gb300 as epr
    lib = epr.load()
    rng = np.random.default_rng(n + cin + cout)
    x = U.bf16(rng.normal(size=(n, n, n, cin)))
    W = U.bf16(rng.normal(size=(27, cin, cout)) / np.sqrt(27 * cin))
    b = rng.normal(size=cout).astype(np.float32)
    ref = U.conv3(x, W, b.astype(np.float64), relu=True)
    dx, dw, db = _dev_bf16(torch, x.reshape(-1, cin)), _dev_bf16(torch, _kmajor(W)), torch.tensor(b, device="cuda")
    out = torch.zeros((n ** 3, cout), dtype=torch.bfloat16, device="cuda")
    s = torch.cuda.current_stream().cuda_stream
    rc = lib.epr_conv3(0, n, cin, cout, _ptr(dx), cin, _ptr(dw), _ptr(db), _ptr(out), cout, 1, 0, ctypes.c_void_p(s))
    assert rc == 0, lib.epr_conv_last_error()
    torch.cuda.synchronize()
    got = out.float().cpu().numpy().reshape(ref.shape)
    assert np.abs(got - ref).max() <= 2 ** -8 * np.abs(ref).max() + 1e-6
    assert np.linalg.norm(got - ref) <= 4e-3 * np.linalg.norm(ref)
    # data gradient: the same kernel with flipped taps and the transposed weights
    dz = U.bf16(rng.normal(size=(n, n, n, cout)))
    refd = U.conv3_dgrad(dz, W)
    Wt = np.ascontiguousarray(W.transpose(1, 0, 2).reshape(cin, 27 * cout))  # row ci, column t * cout + co
    ddz, dwt = _dev_bf16(torch, dz.reshape(-1, cout)), _dev_bf16(torch, Wt)
    outd = torch.zeros((n ** 3, cin), dtype=torch.bfloat16, device="cuda")
    if cin in (16, 32, 48, 64, 96, 128, 192) and cout % 16 == 0:
        rc = lib.epr_conv3(0, n, cout, cin, _ptr(ddz), cout, _ptr(dwt), None, _ptr(outd), cin, 0, 1, ctypes.c_void_p(s))
        assert rc == 0, lib.epr_conv_last_error()
        torch.cuda.synchronize()
        gd = outd.float().cpu().numpy().reshape(refd.shape)
        assert np.abs(gd - refd).max() <= 2 ** -8 * np.abs(refd).max() + 1e-6
        assert np.linalg.norm(gd - refd) <= 4e-3 * np.linalg.norm(refd)


@pytest.mark.parametrize("n,cin,cout", [(9, 16, 16), (17, 32, 64), (9, 192, 64), (9, 64, 128)])
def test_conv_weight_gradient(torch, n, cin, cout):
    import exteriorpoissonrecon_gb300 as epr
    lib = epr.load()
    rng = np.random.default_rng(7 * n + cin + cout)
    x = U.bf16(rng.normal(size=(n, n, n, cin)))
    dz = U.bf16(rng.normal(size=(n, n, n, cout)))
    ref = U.conv3_wgrad(x, dz).reshape(27 * cin, cout)
    dx, ddz = _dev_bf16(torch, x.reshape(-1, cin)), _dev_bf16(torch, dz.reshape(-1, cout))
    dw = torch.zeros((27 * cin, cout), dtype=torch.float32, device="cuda")
    ns = lib.epr_conv3_wgrad_scratch(n, cin, cout)
    scratch = torch.zeros(ns, dtype=torch.float32, device="cuda")
    s = torch.cuda.current_stream().cuda_stream
    rc = lib.epr_conv3_wgrad(0, n, cin, cout, _ptr(dx), cin, _ptr(ddz), cout, _ptr(dw), _ptr(scratch), ns, ctypes.c_void_p(s))
    assert rc == 0, lib.epr_conv_last_error()
    torch.cuda.synchronize()
    got = dw.cpu().numpy()
    assert np.abs(got - ref).max() <= 1e-4 * np.abs(ref).max()


def _net(epr, level, seed=0):
    lib = epr.load()
    h = lib.epr_unet_create(0, level, seed)
    assert h, lib.epr_unet_last_error(None)
    cnt = ctypes.c_size_t(0)
    assert lib.epr_unet_params(h, None, 0, ctypes.byref(cnt), 0) == 0
    return lib, h, cnt.value


def test_network_gradients_match_oracle(torch):
    """Loss and every layer's weight and bias gradients of the whole U-Net (level 4: 17^3 nodes)
    against the oracle's forward and backward with BF16 rounding at the GPU's storage points."""
    import exteriorpoissonrecon_gb300 as epr
    level = 4
    lib, h, cnt = _net(epr, level, seed=3)
    try:
        params = np.zeros(cnt, np.float32)
        assert lib.epr_unet_params(h, params.ctypes.data_as(ctypes.POINTER(ctypes.c_float)), cnt, None, 0) == 0
        # non-zero biases, so that their gradients and the ReLU masks are exercised
        lay, total = U.layout(level)
        assert total == cnt
        rng = np.random.default_rng(5)
        for name, (wo, bo, cin, cout, lv, relu) in lay.items():
            params[bo:bo + cout] = 0.05 * rng.normal(size=cout) * (1 if name != "head" else 0)
        assert lib.epr_unet_params(h, params.ctypes.data_as(ctypes.POINTER(ctypes.c_float)), cnt, None, 1) == 0
        n = 2 ** level + 1
        x = np.zeros((n, n, n, 16))
        x[..., :15] = rng.uniform(-1, 1, size=(n, n, n, 15))
        x = U.bf16(x)
        t = rng.normal(size=(n, n, n, 2))
        dx = _dev_bf16(torch, x.reshape(-1, 16))
        dt = torch.tensor(t.reshape(-1, 2).astype(np.float32), device="cuda")
        grads = np.zeros(cnt, np.float32)
        loss = ctypes.c_double(0)
        rc = lib.epr_unet_gradients(h, _ptr(dx), _ptr(dt), grads.ctypes.data_as(ctypes.POINTER(ctypes.c_float)), ctypes.byref(loss))
        assert rc == 0, lib.epr_unet_last_error(h)
        net = U.UNet(params.astype(np.float64), level, round_bf16=True)
        L, g = net.gradients(x, t.astype(np.float32).astype(np.float64))
        assert abs(loss.value - L) <= 2e-2 * abs(L), (loss.value, L)
        for name, (wo, bo, cin, cout, lv, relu) in lay.items():
            gw, rw = grads[wo:wo + 27 * cin * cout], g[wo:wo + 27 * cin * cout]
            gb, rb = grads[bo:bo + cout], g[bo:bo + cout]
            assert np.linalg.norm(gw - rw) <= 2e-2 * np.linalg.norm(rw) + 1e-12, name
            # a bias gradient is a sum over all voxels of BF16 values that largely cancel
            assert np.linalg.norm(gb - rb) <= 5e-2 * np.linalg.norm(rb) + 1e-12, name
        # the prediction itself
        pred = torch.zeros((n ** 3, 2), dtype=torch.float32, device="cuda")
        assert lib.epr_unet_forward(h, _ptr(dx), _ptr(pred), None, None) == 0
        p_ref, _ = net.forward(x)
        p = pred.cpu().numpy().reshape(p_ref.shape)
        assert np.linalg.norm(p - p_ref) <= 1e-2 * np.linalg.norm(p_ref)
    finally:
        lib.epr_unet_destroy(h)


def test_training_steps_reduce_the_loss(torch):
    """A few Adam steps on a fixed small batch (level 4) lower the loss; the steps are deterministic
    (two networks from the same seed take the same steps bit for bit)."""
    import exteriorpoissonrecon_gb300 as epr
    level, n = 4, 17
    rng = np.random.default_rng(9)
    ins, tgts = [], []
    for k in range(4):
        x = np.zeros((n, n, n, 16))
        x[..., :15] = rng.uniform(-1, 1, size=(n, n, n, 15))
        ins.append(_dev_bf16(torch, x.reshape(-1, 16)))
        # a smooth target field
        g = np.linspace(0, 1, n)
        zz, yy, xx = np.meshgrid(g, g, g, indexing="ij")
        t = np.stack([np.sin(3 * xx + k) * yy, np.cos(2 * zz - k) * xx], axis=-1)
        tgts.append(torch.tensor(t.reshape(-1, 2).astype(np.float32), device="cuda"))
    arr_in = (ctypes.c_void_p * 4)(*[t.data_ptr() for t in ins])
    arr_t = (ctypes.c_void_p * 4)(*[t.data_ptr() for t in tgts])
    losses = []
    for rep in range(2):
        lib, h, cnt = _net(epr, level, seed=11)
        try:
            ls = []
            for step in range(30):
                l = ctypes.c_double(0)
                assert lib.epr_unet_train_step(h, 4, arr_in, arr_t, 3e-3, ctypes.byref(l)) == 0, lib.epr_unet_last_error(h)
                ls.append(l.value)
            p = np.zeros(cnt, np.float32)
            lib.epr_unet_params(h, p.ctypes.data_as(ctypes.POINTER(ctypes.c_float)), cnt, None, 0)
            losses.append((ls, p))
        finally:
            lib.epr_unet_destroy(h)
    ls = losses[0][0]
    assert ls[-1] < 0.7 * ls[0], ls
    assert losses[0][0] == losses[1][0] and np.array_equal(losses[0][1], losses[1][1])
