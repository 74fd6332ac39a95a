"""ctypes front end of the CPU restatement (oracle/epr_oracle.cpp).

TEST INFRASTRUCTURE ONLY: imported by tests/, by __graft_entry__.smoke() as the checker and by
bench.py's CPU-baseline leg.  The product package never imports this module.
"""
from __future__ import annotations

import ctypes
import os
import subprocess

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_LIB_PATH = os.path.join(_HERE, "_build", "libepr_oracle.so")
_lib = None


class Params(ctypes.Structure):
    _fields_ = [
        ("s_weight", ctypes.c_double),
        ("d_weight", ctypes.c_double),
        ("n_sigma", ctypes.c_double),
        ("i_mult", ctypes.c_double),
        ("t_radius", ctypes.c_int),
        ("d_radius", ctypes.c_int),
        ("gs_iters", ctypes.c_int),
        ("min_solve_depth", ctypes.c_int),
        ("max_solve_depth", ctypes.c_int),
        ("seed", ctypes.c_uint),
        ("threads", ctypes.c_int),
        ("single_level", ctypes.c_int),
        ("separate", ctypes.c_int),
        ("alt_rounds", ctypes.c_int),
        ("project", ctypes.c_int),
        ("adaptive_radius", ctypes.c_int),
    ]


def build() -> str:
    """Compiles the restatement (make -C oracle port)."""
    subprocess.run(["make", "-s", "-C", _HERE, "port"], check=True)
    return _LIB_PATH


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(_LIB_PATH) or os.path.getmtime(_LIB_PATH) < os.path.getmtime(
                os.path.join(_HERE, "epr_oracle.cpp")):
            build()
        L = ctypes.CDLL(_LIB_PATH)
        P = ctypes.POINTER(ctypes.c_double)
        L.epr_oracle_create.restype = ctypes.c_void_p
        L.epr_oracle_create.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.POINTER(Params)]
        L.epr_oracle_destroy.argtypes = [ctypes.c_void_p]
        L.epr_oracle_default_params.argtypes = [ctypes.POINTER(Params)]
        L.epr_oracle_unit_cube.argtypes = [ctypes.c_int, ctypes.c_size_t, ctypes.c_double, P, P]
        L.epr_oracle_set_samples.argtypes = [ctypes.c_void_p, ctypes.c_size_t, P, P]
        L.epr_oracle_build.argtypes = [ctypes.c_void_p]
        L.epr_oracle_set_level_system.argtypes = [ctypes.c_void_p, ctypes.c_int, P, P, ctypes.c_double]
        L.epr_oracle_get.restype = ctypes.c_long
        L.epr_oracle_get.argtypes = [ctypes.c_void_p, ctypes.c_char_p, ctypes.c_int, P]
        L.epr_oracle_num_nodes.restype = ctypes.c_size_t
        L.epr_oracle_num_nodes.argtypes = [ctypes.c_int, ctypes.c_int]
        L.epr_oracle_energy.argtypes = [ctypes.c_void_p, ctypes.c_int, P, P, P]
        L.epr_oracle_quadfit.argtypes = [ctypes.c_void_p, ctypes.c_int, P, P, P]
        L.epr_oracle_gradient.argtypes = [ctypes.c_void_p, ctypes.c_int, P, P, P, P]
        I64 = ctypes.POINTER(ctypes.c_int64)
        L.epr_oracle_quadfit_at.argtypes = [ctypes.c_void_p, ctypes.c_int, P, P, I64, ctypes.c_size_t, P]
        L.epr_oracle_gn_matvec_at.argtypes = [ctypes.c_void_p, ctypes.c_int, P, P, P, P, I64, ctypes.c_size_t, P, P]
        L.epr_oracle_gs.argtypes = [ctypes.c_void_p, ctypes.c_int, P, P, ctypes.c_int]
        L.epr_oracle_prolong.argtypes = [ctypes.c_void_p, ctypes.c_int, P, P]
        L.epr_oracle_gs_shifted.argtypes = [ctypes.c_void_p, ctypes.c_int, P, P, ctypes.c_int, P, P]
        L.epr_oracle_restrict.argtypes = [ctypes.c_void_p, ctypes.c_int, P, P]
        L.epr_oracle_linear_gs.argtypes = [ctypes.c_void_p, ctypes.c_int, P, P, P]
        L.epr_oracle_wedge_gram.argtypes = [ctypes.c_void_p, ctypes.c_int, P, P]
        L.epr_oracle_alternating_system.argtypes = [ctypes.c_void_p, ctypes.c_int, P, P, ctypes.c_int, P, P]
        L.epr_oracle_alternating_solve.argtypes = [ctypes.c_void_p, ctypes.c_int, P, P, ctypes.c_int, ctypes.c_int,
                                                   ctypes.c_int, ctypes.c_int]
        L.epr_oracle_biquadratic_fit.argtypes = [ctypes.c_void_p, ctypes.c_int, P, P, P, P, P, ctypes.c_int]
        L.epr_oracle_step_size.argtypes = [P]
        L.epr_oracle_step_size.restype = ctypes.c_double
        L.epr_oracle_newton_update.argtypes = [P, ctypes.c_int, P]
        L.epr_oracle_mg_vcycle.argtypes = [ctypes.c_void_p, ctypes.c_int, P, P, P, ctypes.c_int, ctypes.c_int]
        L.epr_oracle_gn_matvec.argtypes = [ctypes.c_void_p, ctypes.c_int, P, P, P, P, P, P]
        L.epr_oracle_solve.argtypes = [ctypes.c_void_p, P, P, P]
        L.epr_oracle_solve_begin.restype = ctypes.c_int64
        L.epr_oracle_solve_begin.argtypes = [ctypes.c_void_p]
        L.epr_oracle_solve_advance.argtypes = [ctypes.c_void_p, ctypes.c_int64]
        L.epr_oracle_solve_finish.argtypes = [ctypes.c_void_p, P]
        _lib = L
    return _lib


def _p(a: np.ndarray):
    assert a.dtype == np.float64 and a.flags["C_CONTIGUOUS"]
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_double))


def default_params(**kw) -> Params:
    p = Params()
    lib().epr_oracle_default_params(ctypes.byref(p))
    for k, v in kw.items():
        setattr(p, k, v)
    return p


def num_nodes(dim: int, level: int) -> int:
    return (2 ** level + 1) ** dim


def unit_cube(pos: np.ndarray, scale: float = 1.1):
    pos = np.ascontiguousarray(pos, dtype=np.float64).copy()
    n, dim = pos.shape
    xf = np.zeros((dim + 1) * (dim + 1))
    rc = lib().epr_oracle_unit_cube(dim, n, scale, _p(pos), _p(xf))
    if rc:
        raise ValueError(f"unit_cube failed ({rc})")
    return pos, xf.reshape(dim + 1, dim + 1)


class Oracle:
    """One reconstruction problem (dimension, depth, parameters) on the CPU."""

    def __init__(self, dim: int, depth: int, **params):
        self.dim, self.depth = dim, depth
        self.params = default_params(**params)
        self._h = lib().epr_oracle_create(dim, depth, ctypes.byref(self.params))
        if not self._h:
            raise ValueError("invalid oracle configuration")

    def __del__(self):
        if getattr(self, "_h", None):
            lib().epr_oracle_destroy(self._h)
            self._h = None

    def set_samples(self, pos_unit: np.ndarray, skew_packed: np.ndarray):
        pos = np.ascontiguousarray(pos_unit, dtype=np.float64)
        sk = np.ascontiguousarray(skew_packed, dtype=np.float64)
        if lib().epr_oracle_set_samples(self._h, pos.shape[0], _p(pos), _p(sk)):
            raise ValueError("set_samples failed")

    def build(self):
        if lib().epr_oracle_build(self._h):
            raise RuntimeError("build failed")

    def set_level_system(self, level, R, B, c):
        R = np.ascontiguousarray(R, dtype=np.float64)
        B = np.ascontiguousarray(B, dtype=np.float64)
        lib().epr_oracle_set_level_system(self._h, level, _p(R), _p(B), float(c))

    def get(self, name: str, level: int = 0) -> np.ndarray:
        n = lib().epr_oracle_get(self._h, name.encode(), level, None)
        if n < 0:
            raise KeyError(name)
        out = np.zeros(n)
        lib().epr_oracle_get(self._h, name.encode(), level, _p(out))
        return out

    def nodes(self, level):
        return num_nodes(self.dim, level)

    def energy(self, level, x, y):
        out = np.zeros(3)
        lib().epr_oracle_energy(self._h, level, _p(np.ascontiguousarray(x, np.float64)),
                                _p(np.ascontiguousarray(y, np.float64)), _p(out))
        return out

    def quadfit(self, level, x, y):
        out = np.zeros((self.nodes(level), 5))
        lib().epr_oracle_quadfit(self._h, level, _p(np.ascontiguousarray(x, np.float64)),
                                 _p(np.ascontiguousarray(y, np.float64)), _p(out))
        return out

    def quadfit_at(self, level, x, y, idx):
        """quadfit rows of the nodes idx only."""
        idx = np.ascontiguousarray(idx, np.int64)
        out = np.zeros((len(idx), 5))
        lib().epr_oracle_quadfit_at(self._h, level, _p(np.ascontiguousarray(x, np.float64)),
                                    _p(np.ascontiguousarray(y, np.float64)),
                                    idx.ctypes.data_as(ctypes.POINTER(ctypes.c_int64)), len(idx), _p(out))
        return out

    def gn_matvec_at(self, level, x, y, dx, dy, idx):
        """Gauss-Newton product at the nodes idx only."""
        idx = np.ascontiguousarray(idx, np.int64)
        ox = np.zeros(len(idx))
        oy = np.zeros(len(idx))
        a = [np.ascontiguousarray(v, np.float64) for v in (x, y, dx, dy)]
        lib().epr_oracle_gn_matvec_at(self._h, level, *[_p(v) for v in a],
                                      idx.ctypes.data_as(ctypes.POINTER(ctypes.c_int64)), len(idx), _p(ox), _p(oy))
        return ox, oy

    def gradient(self, level, x, y):
        gx = np.zeros(self.nodes(level))
        gy = np.zeros(self.nodes(level))
        lib().epr_oracle_gradient(self._h, level, _p(np.ascontiguousarray(x, np.float64)),
                                  _p(np.ascontiguousarray(y, np.float64)), _p(gx), _p(gy))
        return gx, gy

    def gs(self, level, x, y, iters=1):
        x = np.array(x, dtype=np.float64)
        y = np.array(y, dtype=np.float64)
        lib().epr_oracle_gs(self._h, level, _p(x), _p(y), iters)
        return x, y

    def gs_shifted(self, level, x, y, tx, ty, iters=1):
        x = np.array(x, dtype=np.float64)
        y = np.array(y, dtype=np.float64)
        lib().epr_oracle_gs_shifted(self._h, level, _p(x), _p(y), iters,
                                    _p(np.ascontiguousarray(tx, np.float64)), _p(np.ascontiguousarray(ty, np.float64)))
        return x, y

    def linear_gs(self, level, M, b, x):
        x = np.array(x, dtype=np.float64)
        lib().epr_oracle_linear_gs(self._h, level, _p(np.ascontiguousarray(M, np.float64)),
                                   _p(np.ascontiguousarray(b, np.float64)), _p(x))
        return x

    def mg_vcycle(self, level, M, b, x, iters=2, cycles=1):
        x = np.array(x, dtype=np.float64)
        lib().epr_oracle_mg_vcycle(self._h, level, _p(np.ascontiguousarray(M, np.float64)),
                                   _p(np.ascontiguousarray(b, np.float64)), _p(x), iters, cycles)
        return x

    def wedge_gram(self, level, f):
        N = int(((1 << level) + 1) ** self.dim)
        G = np.zeros((N, 3 ** self.dim))
        lib().epr_oracle_wedge_gram(self._h, level, _p(np.ascontiguousarray(f, np.float64)), _p(G))
        return G

    def alternating_system(self, level, x, y, which):
        N = int(((1 << level) + 1) ** self.dim)
        M = np.zeros((N, 3 ** self.dim))
        b = np.zeros(N)
        lib().epr_oracle_alternating_system(self._h, level, _p(np.ascontiguousarray(x, np.float64)),
                                            _p(np.ascontiguousarray(y, np.float64)), which, _p(M), _p(b))
        return M, b

    def alternating_solve(self, level, x, y, iters=1, vcycles=1, gs_iters=2, single_level=False):
        x = np.array(x, dtype=np.float64)
        y = np.array(y, dtype=np.float64)
        lib().epr_oracle_alternating_solve(self._h, level, _p(x), _p(y), iters, vcycles, gs_iters, int(single_level))
        return x, y

    def biquadratic_fit(self, level, x, y, dx, dy, as_reference=False):
        q = np.zeros((3, 3))
        c = lambda v: _p(np.ascontiguousarray(v, np.float64))  # noqa: E731
        lib().epr_oracle_biquadratic_fit(self._h, level, c(x), c(y), c(dx), c(dy), _p(q), int(as_reference))
        return q

    @staticmethod
    def step_size(q):
        return float(lib().epr_oracle_step_size(_p(np.ascontiguousarray(q, np.float64))))

    @staticmethod
    def newton_update(q, steps=10):
        st = np.zeros(2)
        lib().epr_oracle_newton_update(_p(np.ascontiguousarray(q, np.float64)), steps, _p(st))
        return st

    def restrict(self, level, vf):
        out = np.zeros(self.nodes(level))
        lib().epr_oracle_restrict(self._h, level, _p(np.ascontiguousarray(vf, np.float64)), _p(out))
        return out

    def prolong(self, level, xc):
        out = np.zeros(self.nodes(level + 1))
        lib().epr_oracle_prolong(self._h, level, _p(np.ascontiguousarray(xc, np.float64)), _p(out))
        return out

    def gn_matvec(self, level, x, y, dx, dy):
        ox = np.zeros(self.nodes(level))
        oy = np.zeros(self.nodes(level))
        a = [np.ascontiguousarray(v, np.float64) for v in (x, y, dx, dy)]
        lib().epr_oracle_gn_matvec(self._h, level, *[_p(v) for v in a], _p(ox), _p(oy))
        return ox, oy

    def solve(self):
        tot = sum(self.nodes(l) for l in range(self.depth + 1))
        x = np.zeros(tot)
        y = np.zeros(tot)
        e = np.zeros(3)
        lib().epr_oracle_solve(self._h, _p(x), _p(y), _p(e))
        xs, ys, off = [], [], 0
        for l in range(self.depth + 1):
            n = self.nodes(l)
            xs.append(x[off:off + n])
            ys.append(y[off:off + n])
            off += n
        return xs, ys, e

    def solve_begin(self) -> int:
        """Starts the cascadic solve (random start); returns its total node updates."""
        return int(lib().epr_oracle_solve_begin(self._h))

    def solve_advance(self, target_node_updates: int) -> bool:
        """Relaxes whole sweeps in schedule order until target node updates are done; True when the
        schedule is complete."""
        return bool(lib().epr_oracle_solve_advance(self._h, int(target_node_updates)))

    def solve_finish(self):
        """(c, fit energy, regularisation energy) of the stepped solve."""
        e = np.zeros(3)
        lib().epr_oracle_solve_finish(self._h, _p(e))
        return e
