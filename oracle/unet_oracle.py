"""CPU oracle of the learned warm start's network (test infrastructure only; nothing here is
shipped or timed).

The library's U-Net (exteriorpoissonrecon_gb300/csrc/epr_unet.cu) restated in float64 numpy: the
3x3x3 convolutions on node grids (zero padding), their data and weight gradients, the grid
transfers between network levels (full-weighting restriction with the multilinear weights,
1/8-normalised, and multilinear prolongation: the solver's own transfer, Hat.scalars.inl:370-386),
the scale- and rotation-invariant loss, and the whole forward and backward pass over the flat
parameter layout the library uses (per layer: weights [27 Cin][Cout] with row tap * Cin + ci,
then the bias [Cout]).

With bf16=True the activations, weights and gradients are rounded to BF16 where the GPU stores
them in BF16 (the products and sums stay in float64), so that the comparison isolates the
accumulation order; finite differences of the float64 model check the backward pass itself.
"""
from __future__ import annotations

import numpy as np

TAPS = [(t // 9 - 1, (t // 3) % 3 - 1, t % 3 - 1) for t in range(27)]

# layers: (GEMM input channels, real input channels, output channels, network level, relu)
LAYERS = [("enc0", 16, 15, 16, 0, True), ("enc1", 16, 16, 32, 1, True), ("enc2", 32, 32, 64, 2, True),
          ("bott", 64, 64, 128, 3, True), ("dec2", 192, 192, 64, 2, True), ("dec1", 96, 96, 32, 1, True),
          ("dec0", 48, 48, 16, 0, True), ("head", 16, 16, 16, 0, False)]


def bf16(a):
    """Round to the nearest BF16 (ties to even), returned as float64."""
    a32 = np.ascontiguousarray(np.asarray(a, dtype=np.float32))
    u = a32.view(np.uint32).astype(np.uint64)
    u = ((u + 0x7FFF + ((u >> 16) & 1)) >> 16) << 16
    return (u.astype(np.uint32)).view(np.float32).astype(np.float64)


def to_bf16_bits(a) -> np.ndarray:
    """The BF16 bit patterns (uint16) of a (round to nearest even)."""
    a32 = np.ascontiguousarray(np.asarray(a, dtype=np.float32))
    u = a32.view(np.uint32).astype(np.uint64)
    return (((u + 0x7FFF + ((u >> 16) & 1)) >> 16) & 0xFFFF).astype(np.uint16)


def from_bf16_bits(b) -> np.ndarray:
    return (np.asarray(b, dtype=np.uint32) << 16).view(np.float32).astype(np.float64)


def shift(x, off):
    """y[v] = x[v + off] on an (n, n, n, C) grid, zero outside."""
    n = x.shape[0]
    y = np.zeros_like(x)
    src = tuple(slice(max(o, 0), n + min(o, 0)) for o in off)
    dst = tuple(slice(max(-o, 0), n + min(-o, 0)) for o in off)
    y[dst] = x[src]
    return y


def conv3(x, W, b=None, relu=False, flip=False):
    """x (n, n, n, Cin), W (27, Cin, Cout) -> (n, n, n, Cout): sum_t x[v + s off(t)] W[t] + b."""
    s = -1 if flip else 1
    out = sum(shift(x, tuple(s * o for o in TAPS[t])) @ W[t] for t in range(27))
    if b is not None:
        out = out + b
    return np.maximum(out, 0) if relu else out


def conv3_dgrad(dz, W):
    """Gradient with respect to the input of conv3 (without bias and activation)."""
    return sum(shift(dz, tuple(-o for o in TAPS[t])) @ W[t].T for t in range(27))


def conv3_wgrad(x, dz):
    """(27, Cin, Cout): dW[t] = sum_v x[v + off(t)] dz[v]^T."""
    cin, cout = x.shape[-1], dz.shape[-1]
    return np.stack([shift(x, TAPS[t]).reshape(-1, cin).T @ dz.reshape(-1, cout) for t in range(27)])


def _w(o):
    return np.prod([1.0 if d == 0 else 0.5 for d in o])


def restrict(f, scale):
    """coarse[I] = scale * sum_o w(o) f[2I + o] (n_fine = 2 n_coarse - 1)."""
    nf = f.shape[0]
    nc = (nf + 1) // 2
    out = np.zeros((nc, nc, nc, f.shape[-1]))
    for o in TAPS:
        sh = shift(f, o)  # sh[v] = f[v + o]
        out += scale * _w(o) * sh[::2, ::2, ::2]
    return out


def prolong(c, scale):
    """fine[f] = scale * multilinear interpolation of c."""
    nc = c.shape[0]
    nf = 2 * nc - 1
    out = np.zeros((nf, nf, nf, c.shape[-1]))
    out[::2, ::2, ::2] = c
    for ax in range(3):
        sl_odd = [slice(None)] * 3
        sl_lo = [slice(None)] * 3
        sl_hi = [slice(None)] * 3
        sl_odd[ax] = slice(1, nf, 2)
        sl_lo[ax] = slice(0, nf - 1, 2)
        sl_hi[ax] = slice(2, nf, 2)
        out[tuple(sl_odd)] = 0.5 * (out[tuple(sl_lo)] + out[tuple(sl_hi)])
    return scale * out


def loss_and_grad(p, t):
    """1 - (a^2 + b^2) / (P T) with a = <p, t>, b = <p x t> over nodes' (x, y) pairs; and dL/dp."""
    px, py, tx, ty = p[..., 0], p[..., 1], t[..., 0], t[..., 1]
    a = float((px * tx + py * ty).sum())
    b = float((px * ty - py * tx).sum())
    P = float((px * px + py * py).sum())
    T = float((tx * tx + ty * ty).sum())
    nrm = a * a + b * b
    L = 1.0 - nrm / (P * T)
    gx = -((2 * a * tx + 2 * b * ty) * P - nrm * 2 * px) / (P * P * T)
    gy = -((2 * a * ty - 2 * b * tx) * P - nrm * 2 * py) / (P * P * T)
    return L, np.stack([gx, gy], axis=-1)


def layout(level):
    """Offsets of each layer's weights and bias in the flat parameter vector; total count."""
    off, out = 0, {}
    for name, cin, _, cout, lv, relu in LAYERS:
        out[name] = (off, off + 27 * cin * cout, cin, cout, lv, relu)
        off += 27 * cin * cout + cout
    return out, off


def unpack(params, level):
    lay, _ = layout(level)
    W, B = {}, {}
    for name, (wo, bo, cin, cout, _, _) in lay.items():
        W[name] = np.asarray(params[wo:wo + 27 * cin * cout], np.float64).reshape(27, cin, cout)
        B[name] = np.asarray(params[bo:bo + cout], np.float64)
    return W, B


class UNet:
    """Forward and backward of the library's network in float64 (optionally BF16-rounded where the
    GPU stores BF16)."""

    def __init__(self, params, level, round_bf16=False):
        self.level = level
        self.r = bf16 if round_bf16 else (lambda a: np.asarray(a, np.float64))
        W, self.B = unpack(params, level)
        self.W = {k: self.r(v) for k, v in W.items()}

    def forward(self, x):
        """x: (n, n, n, 16) input; returns the (n, n, n, 2) prediction and the saved activations."""
        r, W, B = self.r, self.W, self.B
        s = {}
        s["in"] = r(x)
        s["e0"] = r(conv3(s["in"], W["enc0"], B["enc0"], True))
        s["d0"] = r(restrict(s["e0"], 1 / 8))
        s["e1"] = r(conv3(s["d0"], W["enc1"], B["enc1"], True))
        s["d1"] = r(restrict(s["e1"], 1 / 8))
        s["e2"] = r(conv3(s["d1"], W["enc2"], B["enc2"], True))
        s["d2"] = r(restrict(s["e2"], 1 / 8))
        s["b3"] = r(conv3(s["d2"], W["bott"], B["bott"], True))
        s["c2"] = np.concatenate([r(prolong(s["b3"], 1.0)), s["e2"]], axis=-1)
        s["u2"] = r(conv3(s["c2"], W["dec2"], B["dec2"], True))
        s["c1"] = np.concatenate([r(prolong(s["u2"], 1.0)), s["e1"]], axis=-1)
        s["u1"] = r(conv3(s["c1"], W["dec1"], B["dec1"], True))
        s["c0"] = np.concatenate([r(prolong(s["u1"], 1.0)), s["e0"]], axis=-1)
        s["u0"] = r(conv3(s["c0"], W["dec0"], B["dec0"], True))
        out = conv3(s["u0"], W["head"], B["head"], False)
        return out[..., :2], s

    def gradients(self, x, target):
        """Loss and the flat gradient of every parameter (the library's layout)."""
        r, W = self.r, self.W
        pred, s = self.forward(x)
        L, gp = loss_and_grad(pred, target)
        dh = np.zeros(pred.shape[:3] + (16,))
        dh[..., :2] = gp
        dh = r(dh)
        g = {}

        def wg(name, xin, dz):
            g[name] = (conv3_wgrad(xin, dz), dz.reshape(-1, dz.shape[-1]).sum(axis=0))

        wg("head", s["u0"], dh)
        dz0 = r(conv3_dgrad(dh, W["head"]) * (s["u0"] > 0))
        wg("dec0", s["c0"], dz0)
        dc0 = r(conv3_dgrad(dz0, W["dec0"]))
        dz1 = r(restrict(dc0[..., :32], 1.0) * (s["u1"] > 0))
        wg("dec1", s["c1"], dz1)
        dc1 = r(conv3_dgrad(dz1, W["dec1"]))
        dz2 = r(restrict(dc1[..., :64], 1.0) * (s["u2"] > 0))
        wg("dec2", s["c2"], dz2)
        dc2 = r(conv3_dgrad(dz2, W["dec2"]))
        dzb = r(restrict(dc2[..., :128], 1.0) * (s["b3"] > 0))
        wg("bott", s["d2"], dzb)
        dd2 = r(conv3_dgrad(dzb, W["bott"]))
        dze2 = r((dc2[..., 128:] + prolong(dd2, 1 / 8)) * (s["e2"] > 0))
        wg("enc2", s["d1"], dze2)
        dd1 = r(conv3_dgrad(dze2, W["enc2"]))
        dze1 = r((dc1[..., 64:] + prolong(dd1, 1 / 8)) * (s["e1"] > 0))
        wg("enc1", s["d0"], dze1)
        dd0 = r(conv3_dgrad(dze1, W["enc1"]))
        dze0 = r((dc0[..., 32:] + prolong(dd0, 1 / 8)) * (s["e0"] > 0))
        wg("enc0", s["in"], dze0)
        lay, total = layout(self.level)
        flat = np.zeros(total)
        for name, (wo, bo, cin, cout, _, _) in lay.items():
            flat[wo:wo + 27 * cin * cout] = g[name][0].reshape(-1)
            flat[bo:bo + cout] = g[name][1]
        return L, flat
