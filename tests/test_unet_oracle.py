"""The network oracle itself (oracle/unet_oracle.py), on the CPU: its data and weight gradients
are the adjoints of its convolution, its restriction is the adjoint of its prolongation, and the
whole backward pass agrees with central differences of the float64 loss."""
import numpy as np

from oracle import unet_oracle as U


def test_convolution_adjoints():
    rng = np.random.default_rng(0)
    n, cin, cout = 5, 3, 4
    x = rng.normal(size=(n, n, n, cin))
    W = rng.normal(size=(27, cin, cout))
    dz = rng.normal(size=(n, n, n, cout))
    y = U.conv3(x, W)
    lhs = float((y * dz).sum())
    assert abs(lhs - float((x * U.conv3_dgrad(dz, W)).sum())) < 1e-10 * abs(lhs)
    assert abs(lhs - float((W * U.conv3_wgrad(x, dz)).sum())) < 1e-10 * abs(lhs)
    # the data gradient is the flipped convolution with transposed weights
    assert np.allclose(U.conv3_dgrad(dz, W), U.conv3(dz, W.transpose(0, 2, 1), flip=True))


def test_transfer_adjoints():
    rng = np.random.default_rng(1)
    f = rng.normal(size=(9, 9, 9, 2))
    c = rng.normal(size=(5, 5, 5, 2))
    assert abs(float((U.restrict(f, 1.0) * c).sum()) - float((f * U.prolong(c, 1.0)).sum())) < 1e-10
    # prolongation reproduces multilinear functions
    g = np.linspace(0, 1, 5)
    zz, yy, xx = np.meshgrid(g, g, g, indexing="ij")
    lin = (1 + 2 * zz - yy + 3 * xx)[..., None]
    gf = np.linspace(0, 1, 9)
    zf, yf, xf = np.meshgrid(gf, gf, gf, indexing="ij")
    assert np.allclose(U.prolong(lin, 1.0)[..., 0], 1 + 2 * zf - yf + 3 * xf)


def test_bf16_rounding():
    a = np.array([1.0, 1.00390625, 1.01171875, -3.14159, 65504.0, 1e-30])
    r = U.bf16(a)
    # halfway cases go to the even significand: 1 + 2^-8 -> 1, 1 + 3 2^-8 -> 1 + 2^-6
    assert r[0] == 1.0 and r[1] == 1.0 and r[2] == 1.015625
    assert np.array_equal(U.from_bf16_bits(U.to_bf16_bits(a)), r)
    assert np.all(np.abs(r - a) <= 2 ** -8 * np.abs(a))


def test_network_backward_matches_central_differences():
    level = 3
    lay, total = U.layout(level)
    rng = np.random.default_rng(2)
    p = np.zeros(total)
    for name, (wo, bo, cin, cout, lv, relu) in lay.items():
        p[wo:wo + 27 * cin * cout] = rng.normal(size=27 * cin * cout) * np.sqrt(2 / (27 * cin))
        p[bo:bo + cout] = 0.05 * rng.normal(size=cout)
    n = 2 ** level + 1
    x = np.zeros((n, n, n, 16))
    x[..., :15] = rng.uniform(-1, 1, size=(n, n, n, 15))
    t = rng.normal(size=(n, n, n, 2))
    L, g = U.UNet(p, level).gradients(x, t)

    def loss(q):
        pred, _ = U.UNet(q, level).forward(x)
        return U.loss_and_grad(pred, t)[0]

    h = 1e-6
    # a few parameters of every layer (weights with real input channels and the bias)
    picks = []
    for name, (wo, bo, cin, cout, lv, relu) in lay.items():
        creal = 15 if name == "enc0" else cin
        coutr = 2 if name == "head" else cout
        for _ in range(3):
            t_, ci, co = rng.integers(27), rng.integers(creal), rng.integers(coutr)
            picks.append(wo + (t_ * cin + ci) * cout + co)
        picks.append(bo + rng.integers(coutr))
    scale = np.abs(g).max()
    for i in picks:
        q1, q2 = p.copy(), p.copy()
        q1[i] += h
        q2[i] -= h
        fd = (loss(q1) - loss(q2)) / (2 * h)
        assert abs(fd - g[i]) <= 1e-5 * scale, (i, fd, g[i])
