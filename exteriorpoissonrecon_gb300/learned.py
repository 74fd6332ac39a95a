"""The learned warm start: a U-Net on the GPU (libepr_cuda's tensor-core kernels) that predicts the
level-L coefficients of the cascadic solve from the splatted density and frame field of level L,
trained on solves the method itself computes.

    net = WarmStartNet.load()                       # the trained network shipped with the package
    r = Reconstructor(3, 8, pos, skew, precision="fp32", minSolveDepth=6, warm_start=1)
    info = net.warm_start(r)                        # predicted start on level 6 (or the random one)
    r.solve()                                       # levels 6-8 of the schedule

Training (``python -m exteriorpoissonrecon_gb300.learned train``): random closed Fourier curves
(3-8 harmonics, coefficient vectors N(0, 1/k^2)), torus knots with coprime (p, q) in [2, 7],
helices (1-8 turns) and perturbed two-circle links, 64K-1M samples each (log-uniform), positional
noise sigma in [0, 0.01] (unit-cube units), angular noise in [0, 10] degrees and up to 10% spot
outliers; each is built at depth 8 and solved by the reference's schedule through level L (FP32
relaxation, levels 0-3 in double-float, the configuration whose result matches the FP64 run), and
the level-L regular coefficients are the target.  Device memory for the data set comes from
PyTorch (plumbing); every kernel that touches the network is the library's.
"""
from __future__ import annotations

import argparse
import ctypes
import json
import math
import os
import time

import numpy as np

from . import EprError, Reconstructor, load, pack_skew, samples, unit_cube

HERE = os.path.dirname(os.path.abspath(__file__))
WEIGHTS = os.path.join(HERE, "weights", "warm_start_level6.npz")

# the precision configuration the training solves use (the benchmark's)
SOLVE_KW = dict(precision="fp32", fp64_from=0, fp64_levels=4, band_precision="df")


class WarmStartNet:
    """Handle of an epr_unet (a network for one level) on one device."""

    def __init__(self, level: int = 6, seed: int = 0, device: int = 0, params: np.ndarray | None = None):
        L = load()
        self.level, self.device = int(level), int(device)
        self._h = L.epr_unet_create(self.device, self.level, int(seed))
        if not self._h:
            raise EprError(L.epr_unet_last_error(None).decode())
        cnt = ctypes.c_size_t(0)
        self._check(L.epr_unet_params(self._h, None, 0, ctypes.byref(cnt), 0))
        self.nparams = cnt.value
        n = ctypes.c_int(0)
        ib, tf = ctypes.c_size_t(0), ctypes.c_size_t(0)
        self._check(L.epr_unet_grid(self._h, ctypes.byref(n), ctypes.byref(ib), ctypes.byref(tf)))
        self.n, self.input_bytes, self.target_floats = n.value, ib.value, tf.value
        if params is not None:
            self.set_params(params)

    def _check(self, rc):
        if rc != 0:
            raise EprError(f"[{rc}] " + load().epr_unet_last_error(self._h).decode())

    def close(self):
        if getattr(self, "_h", None):
            load().epr_unet_destroy(self._h)
            self._h = None

    def __del__(self):
        self.close()

    # ---------------------------------------------------------------- parameters
    def params(self) -> np.ndarray:
        p = np.zeros(self.nparams, np.float32)
        self._check(load().epr_unet_params(self._h, p.ctypes.data_as(ctypes.POINTER(ctypes.c_float)), self.nparams, None, 0))
        return p

    def set_params(self, p: np.ndarray):
        p = np.ascontiguousarray(p, np.float32)
        if p.size != self.nparams:
            raise ValueError(f"expected {self.nparams} parameters, got {p.size}")
        self._check(load().epr_unet_params(self._h, p.ctypes.data_as(ctypes.POINTER(ctypes.c_float)), self.nparams, None, 1))

    def save(self, path: str, meta: dict | None = None):
        os.makedirs(os.path.dirname(os.path.abspath(path)), exist_ok=True)
        np.savez_compressed(path, params=self.params(), level=np.array(self.level),
                            meta=np.array(json.dumps(meta or {})))

    @classmethod
    def load(cls, path: str = WEIGHTS, device: int = 0) -> "WarmStartNet":
        d = np.load(path)
        return cls(level=int(d["level"]), device=device, params=d["params"])

    # ---------------------------------------------------------------- data
    def input(self, r: Reconstructor, dev_ptr: int | None = None):
        """The network input of a built reconstruction into dev_ptr (device address) or the
        network's own input buffer."""
        self._check(load().epr_unet_input(self._h, r._h, ctypes.c_void_p(dev_ptr) if dev_ptr else None))

    def target(self, r: Reconstructor, dev_ptr: int):
        self._check(load().epr_unet_target(self._h, r._h, ctypes.c_void_p(dev_ptr)))

    def loss(self, dev_input: int, dev_target: int) -> float:
        l = ctypes.c_double(0)
        self._check(load().epr_unet_forward(self._h, ctypes.c_void_p(dev_input), None, ctypes.byref(l), ctypes.c_void_p(dev_target)))
        return l.value

    def predict(self, dev_input: int | None = None):
        """One forward pass on dev_input (device address) or the network's own input buffer; the
        prediction stays in the network's device memory."""
        self._check(load().epr_unet_forward(self._h, ctypes.c_void_p(dev_input) if dev_input else None, None, None, None))

    def train_step(self, inputs, targets, lr: float) -> float:
        b = len(inputs)
        ai = (ctypes.c_void_p * b)(*inputs)
        at = (ctypes.c_void_p * b)(*targets)
        l = ctypes.c_double(0)
        self._check(load().epr_unet_train_step(self._h, b, ai, at, ctypes.c_float(lr), ctypes.byref(l)))
        return l.value

    # ---------------------------------------------------------------- use
    def warm_start(self, r: Reconstructor) -> dict:
        """Sets the predicted (energy-optimally scaled) start on the network's level of r, or the
        reference's random start there when the prediction does not lower the energy."""
        info = np.zeros(4)
        self._check(load().epr_unet_warm_start(self._h, r._h, info.ctypes.data_as(ctypes.POINTER(ctypes.c_double))))
        return {"used": bool(info[0]), "reflected": bool(info[0] == 2), "energy_predicted": float(info[1]),
                "energy_random_start": float(info[2]), "scale": float(info[3])}


# ---------------------------------------------------------------------------------------------
# synthetic training shapes
# ---------------------------------------------------------------------------------------------

def fourier_curve(n: int, rng, harmonics: int):
    """Closed curve sum_k a_k cos(k t) + b_k sin(k t), a_k, b_k ~ N(0, I / k^2) in R^3; t uniform."""
    k = np.arange(1, harmonics + 1)
    a = rng.normal(size=(harmonics, 3)) / k[:, None]
    b = rng.normal(size=(harmonics, 3)) / k[:, None]
    t = rng.uniform(0.0, 2.0 * math.pi, n)
    ct, st = np.cos(np.outer(t, k)), np.sin(np.outer(t, k))
    pos = ct @ a + st @ b
    tan = (-st * k) @ a + (ct * k) @ b
    return pos, samples.curve_frames(tan)


def _random_rotation(rng):
    q, r = np.linalg.qr(rng.normal(size=(3, 3)))
    return q * np.sign(np.diag(r))


def perturbed_link(n: int, rng):
    """Two interlocking circles with random radii ratio, offset and tilt."""
    r2 = rng.uniform(0.6, 1.4)
    off = rng.uniform(0.6, 1.2) * r2
    tilt = rng.uniform(-0.4, 0.4)
    t = rng.uniform(0.0, 2.0 * math.pi, n)
    which = rng.integers(0, 2, n)
    c, s = np.cos(t), np.sin(t)
    ct, sn = math.cos(tilt), math.sin(tilt)
    p0 = np.stack([c, s, np.zeros(n)], axis=1)
    t0 = np.stack([-s, c, np.zeros(n)], axis=1)
    # second circle in a plane through the x axis tilted by `tilt` from xz
    e1, e2 = np.array([1.0, 0.0, 0.0]), np.array([0.0, sn, ct])
    p1 = np.array([off, 0.0, 0.0]) + r2 * (np.outer(c, e1) + np.outer(s, e2))
    t1 = np.outer(-s, e1) + np.outer(c, e2)
    pos = np.where(which[:, None] == 0, p0, p1)
    tan = np.where(which[:, None] == 0, t0, t1)
    R = _random_rotation(rng)
    return pos @ R.T, samples.curve_frames(tan @ R.T)


def random_shape(seed: int):
    """(name, world positions, frames) of the training / evaluation distribution for one seed."""
    rng = np.random.default_rng(seed)
    n = int(round(math.exp(rng.uniform(math.log(65536), math.log(1_048_576)))))
    kind = rng.choice(["fourier", "knot", "helix", "link"], p=[0.4, 0.2, 0.2, 0.2])
    if kind == "fourier":
        h = int(rng.integers(3, 9))
        pos, fr = fourier_curve(n, rng, h)
        name = f"fourier{h}"
    elif kind == "knot":
        while True:
            p, q = (int(v) for v in rng.integers(2, 8, 2))
            if math.gcd(p, q) == 1:
                break
        pos, fr = samples.torus_knot(n, p, q, regular=False, rng=rng)
        name = f"knot_{p}_{q}"
    elif kind == "helix":
        turns = float(rng.uniform(1.0, 8.0))
        pos, fr = samples.helix(n, turns, rng)
        name = f"helix_{turns:.1f}"
    else:
        pos, fr = perturbed_link(n, rng)
        name = "link"
    sigma, ang, spot = float(rng.uniform(0, 0.01)), float(rng.uniform(0, 10)), float(rng.uniform(0, 0.1))
    pos, fr = samples.add_noise(pos, fr, rng, sigma, ang, spot)
    return name, pos, fr


def build_pair(net: WarmStartNet, seed: int, depth: int = 8, device: int = 0, dev_input: int = 0, dev_target: int = 0):
    """Builds one training shape at `depth`, solves its schedule through the network's level and
    writes the (input, target) pair to the given device addresses."""
    name, pos, fr = random_shape(seed)
    pu, _ = unit_cube(pos)
    r = Reconstructor(3, depth, pu, pack_skew(fr), device=device, max_solve_depth=net.level, **SOLVE_KW)
    r.solve()
    net.input(r, dev_input)
    net.target(r, dev_target)
    r.close()
    return name


def train(count: int = 512, epochs: int = 40, batch: int = 8, lr: float = 1e-3, level: int = 6, seed: int = 0,
          holdout: int = 16, device: int = 0, log=print):
    """Generates `count` training pairs and `holdout` held-out pairs (seeds disjoint), trains with
    Adam (cosine-decayed learning rate) and returns (net, history)."""
    import torch  # device memory for the data set

    net = WarmStartNet(level=level, seed=seed, device=device)
    dev = torch.device("cuda", device)
    nv = net.n ** 3

    def alloc_pairs(k):
        ins = torch.zeros((k, nv * 16), dtype=torch.bfloat16, device=dev)
        tg = torch.zeros((k, nv * 2), dtype=torch.float32, device=dev)
        return ins, tg

    t0 = time.perf_counter()
    tr_in, tr_t = alloc_pairs(count)
    ho_in, ho_t = alloc_pairs(holdout)
    names = []
    for i in range(count):
        names.append(build_pair(net, 1000 + i, device=device, dev_input=tr_in[i].data_ptr(), dev_target=tr_t[i].data_ptr()))
    for i in range(holdout):
        build_pair(net, 10_000_000 + i, device=device, dev_input=ho_in[i].data_ptr(), dev_target=ho_t[i].data_ptr())
    gen_s = time.perf_counter() - t0
    log(f"data: {count} training + {holdout} held-out pairs in {gen_s:.1f} s")

    def holdout_loss():
        return float(np.mean([net.loss(ho_in[i].data_ptr(), ho_t[i].data_ptr()) for i in range(holdout)]))

    hist = {"holdout_loss": [holdout_loss()], "train_loss": [], "data_s": gen_s}
    rng = np.random.default_rng(seed)
    steps_per_epoch = max(count // batch, 1)
    total = epochs * steps_per_epoch
    step = 0
    t1 = time.perf_counter()
    for ep in range(epochs):
        order = rng.permutation(count)
        ls = []
        for b in range(steps_per_epoch):
            idx = order[b * batch:(b + 1) * batch]
            cur = lr * 0.5 * (1 + math.cos(math.pi * step / total))
            ls.append(net.train_step([tr_in[i].data_ptr() for i in idx], [tr_t[i].data_ptr() for i in idx], cur))
            step += 1
        hist["train_loss"].append(float(np.mean(ls)))
        hist["holdout_loss"].append(holdout_loss())
        log(f"epoch {ep + 1}/{epochs}: train {hist['train_loss'][-1]:.4f} held-out {hist['holdout_loss'][-1]:.4f}")
    hist["train_s"] = time.perf_counter() - t1
    kinds = [n.split("_")[0].rstrip("0123456789") for n in names]
    hist["shapes"] = {k: kinds.count(k) for k in sorted(set(kinds))}
    return net, hist


def time_to_target(net: WarmStartNet | None, pu, sk, depth: int, target: float, cap: int, mode: str, device: int = 0,
                   repeats: int = 2):
    """One solve that ends once the finest level's FP64 energy is <= target (or cap extra sweeps
    were added), in one of three modes:
      "plain":   the reference's schedule from its random start at level 0 (benchmark precision);
      "learned": the network's start on its level, then the schedule from there (FP32);
      "random":  the reference's random start on the network's level, then the same schedule as
                 "learned" (the method without the network at the learned path's cost).
    The last of `repeats` solves counts (the earlier ones build the context's CUDA graph).
    Returns time (warm start wall time + solve device time), energy, reached, extra sweeps."""
    kw = dict(SOLVE_KW) if mode == "plain" else dict(precision="fp32")
    if mode != "plain":
        kw.update(min_solve_depth=net.level, warm_start=1 if mode == "learned" else 0)
    r = Reconstructor(3, depth, pu, sk, device=device, target_energy=target, max_extra_sweeps=cap, **kw)
    res = {}
    for _ in range(repeats):
        ws_s, info = 0.0, None
        if mode == "learned":
            t0 = time.perf_counter()
            info = net.warm_start(r)
            ws_s = time.perf_counter() - t0
        st = r.solve()
        res = {"time_s": ws_s + st["solve_ms"] / 1e3, "warm_start_s": ws_s, "solve_s": st["solve_ms"] / 1e3,
               "energy": st["fit_energy"] + st["reg_energy"], "reached": bool(st["reached_target"]),
               "extra_sweeps": int(st["extra_sweeps"]), "start": info}
    r.close()
    return res


def evaluate(net: WarmStartNet, seeds, depth: int = 8, cap: int = 200, device: int = 0, inputs=None, log=print):
    """For each held-out input: the FP64 run's energy as the target (1 + 1e-6), then the time to
    reach it from the plain schedule, the learned start and the random start on the network's level."""
    out = []
    items = inputs if inputs is not None else [random_shape(s) for s in seeds]
    for name, pos, fr in items:
        pu, _ = unit_cube(pos)
        sk = pack_skew(fr)
        r64 = Reconstructor(3, depth, pu, sk, device=device, precision="fp64")
        s64 = r64.solve()
        e64 = s64["fit_energy"] + s64["reg_energy"]
        r64.close()
        target = e64 * (1 + 1e-6)
        row = {"name": name, "samples": int(len(pu)), "energy_fp64": e64, "fp64_solve_s": s64["solve_ms"] / 1e3}
        for mode in ("plain", "learned", "random"):
            row[mode] = time_to_target(net, pu, sk, depth, target, cap, mode, device)
        out.append(row)
        log(json.dumps(row))
    return out


def main():
    ap = argparse.ArgumentParser()
    sub = ap.add_subparsers(dest="cmd", required=True)
    t = sub.add_parser("train")
    t.add_argument("--count", type=int, default=512)
    t.add_argument("--epochs", type=int, default=40)
    t.add_argument("--batch", type=int, default=8)
    t.add_argument("--lr", type=float, default=1e-3)
    t.add_argument("--holdout", type=int, default=16)
    t.add_argument("--seed", type=int, default=0)
    t.add_argument("--out", default=WEIGHTS)
    t.add_argument("--eval", type=int, default=0, help="held-out inputs evaluated after training")
    e = sub.add_parser("eval")
    e.add_argument("--weights", default=WEIGHTS)
    e.add_argument("--count", type=int, default=4)
    e.add_argument("--cap", type=int, default=200)
    a = ap.parse_args()
    if a.cmd == "eval":
        net = WarmStartNet.load(a.weights)
        rows = evaluate(net, [20_000_000 + i for i in range(a.count)], cap=a.cap)
        print(json.dumps({"eval": rows}))
        return
    if a.cmd == "train":
        net, hist = train(a.count, a.epochs, a.batch, a.lr, seed=a.seed, holdout=a.holdout)
        meta = {"count": a.count, "epochs": a.epochs, "batch": a.batch, "lr": a.lr, "seed": a.seed,
                "holdout_loss_first": hist["holdout_loss"][0], "holdout_loss_last": hist["holdout_loss"][-1],
                "train_loss_last": hist["train_loss"][-1], "data_s": hist["data_s"], "train_s": hist["train_s"]}
        net.save(a.out, meta)
        print(json.dumps({"saved": a.out, **meta, "history": hist}))
        if a.eval:
            rows = evaluate(net, [20_000_000 + i for i in range(a.eval)])
            print(json.dumps({"eval": rows}))


if __name__ == "__main__":
    main()
