"""GB300-native implementation of ExteriorPoissonRecon's regular-grid solve path.

The compute path is libepr_cuda.so (CUDA, sm_103a) behind the C ABI of include/epr.h.  This
module is the Python host side: a ctypes binding of that ABI and a `Reconstructor` that mirrors
the reference's interface (ExteriorPoissonRecon/ExteriorPoisson.h:56-94):

    r = Reconstructor(dim, depth, positions_unit_cube, skew_packed, sWeight=..., ...)
    r.solve()                 # Reconstructor::solve
    r.x(level), r.y(level)    # Reconstructor::x / y (hierarchical coefficients)

There is no CPU fallback: if the library is missing or no GPU is present the calls raise.
"""
from __future__ import annotations

import ctypes
import os
import re

import numpy as np

from . import samples  # noqa: F401  (re-exported helper module)

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libepr_cuda.so")
HEADER = os.path.join(os.path.dirname(HERE), "include", "epr.h")

EPR_OK = 0
EPR_FP64, EPR_FP32 = 0, 1
EPR_SOLVER_CASCADIC, EPR_SOLVER_MULTIGRID = 0, 1
EPR_BAND_FP64, EPR_BAND_DF = 0, 1

_lib = None


class EprError(RuntimeError):
    pass


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
        ("precision", ctypes.c_int),
        ("solver", ctypes.c_int),
        ("tolerance", ctypes.c_double),
        ("max_cycles", ctypes.c_int),
        ("verbose", ctypes.c_int),
        ("device", ctypes.c_int),
        ("fp64_levels", ctypes.c_int),
        ("single_level", ctypes.c_int),
        ("separate", ctypes.c_int),
        ("fp64_from", ctypes.c_int),
        ("band_precision", ctypes.c_int),
        ("warm_start", ctypes.c_int),
        ("max_extra_sweeps", ctypes.c_int),
        ("target_energy", ctypes.c_double),
        ("project", ctypes.c_int),
        ("adaptive_radius", ctypes.c_int),
    ]


class Sampler(ctypes.Structure):
    """epr_sampler: a shape of the reference's Sample tool with its noise, generated on the GPU."""
    _fields_ = [
        ("shape", ctypes.c_int),
        ("regular", ctypes.c_int),
        ("a", ctypes.c_double),
        ("b", ctypes.c_double),
        ("c", ctypes.c_double),
        ("pos_sigma", ctypes.c_double),
        ("angle_deg", ctypes.c_double),
        ("spot_frac", ctypes.c_double),
        ("seed", ctypes.c_uint64),
    ]


SHAPES = {"knot": 0, "link": 1, "helix": 2, "clifford": 3}


def sampler(shape: str, a: float = 0.0, b: float = 0.0, c: float = 0.0, pos_sigma: float = 0.0,
            angle_deg: float = 0.0, spot_frac: float = 0.0, seed: int = 0, regular: bool = False) -> Sampler:
    """knot: a, b = p, q (defaults 2, 3); helix: a turns, radius b (0.3), height c (1)."""
    if shape == "knot":
        a, b = a or 2.0, b or 3.0
    if shape == "helix":
        b, c = b or 0.3, c or 1.0
    return Sampler(SHAPES[shape], int(regular), a, b, c, pos_sigma, angle_deg, spot_frac, seed)


def generate_samples(sp: Sampler, n: int, device: int = 0):
    """World positions (total x dim) and packed frames of n generated samples plus the outliers."""
    L = load()
    total = ctypes.c_size_t(0)
    rc = L.epr_generate_samples(device, ctypes.byref(sp), n, None, None, ctypes.byref(total))
    if rc != EPR_OK:
        raise EprError(f"[{rc}] " + L.epr_global_error().decode())
    dim = 4 if sp.shape == SHAPES["clifford"] else 3
    pos = np.zeros((total.value, dim))
    skew = np.zeros((total.value, dim * (dim - 1) // 2))
    rc = L.epr_generate_samples(device, ctypes.byref(sp), n, _p(pos), _p(skew), ctypes.byref(total))
    if rc != EPR_OK:
        raise EprError(f"[{rc}] " + L.epr_global_error().decode())
    return pos, skew


class Stats(ctypes.Structure):
    _fields_ = [
        ("initial_energy", ctypes.c_double),
        ("fit_energy", ctypes.c_double),
        ("reg_energy", ctypes.c_double),
        ("solve_ms", ctypes.c_double),
        ("build_ms", ctypes.c_double),
        ("grad_norm0", ctypes.c_double),
        ("grad_norm", ctypes.c_double),
        ("cycles", ctypes.c_int),
        ("node_updates", ctypes.c_int64),
        ("kernel_launches", ctypes.c_int64),
        ("extra_sweeps", ctypes.c_int),
        ("reached_target", ctypes.c_int),
    ]

    def as_dict(self):
        return {k: getattr(self, k) for k, _ in self._fields_}


# reference flag names -> epr_params fields
_FLAG_NAMES = {
    "sWeight": "s_weight", "dWeight": "d_weight", "nSigma": "n_sigma", "iMult": "i_mult",
    "tRadius": "t_radius", "dRadius": "d_radius", "gsIters": "gs_iters",
    "minSolveDepth": "min_solve_depth", "maxSolveDepth": "max_solve_depth", "seed": "seed",
    "singleLevel": "single_level", "separate": "separate", "project": "project", "aRadius": "adaptive_radius",
}


def header_symbols() -> list[str]:
    """Names of the functions include/epr.h declares."""
    with open(HEADER) as f:
        txt = f.read()
    return sorted(set(re.findall(r"\b(epr_[a-z_0-9]+)\s*\(", txt)))


def load():
    """Loads libepr_cuda.so (building it first if only the sources are present)."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB_PATH):
        from .build import build
        build()
    L = ctypes.CDLL(LIB_PATH)
    P = ctypes.POINTER(ctypes.c_double)
    vp = ctypes.c_void_p
    L.epr_default_params.argtypes = [ctypes.POINTER(Params)]
    L.epr_create.restype = vp
    L.epr_create.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.POINTER(Params)]
    L.epr_destroy.argtypes = [vp]
    L.epr_last_error.restype = ctypes.c_char_p
    L.epr_last_error.argtypes = [vp]
    L.epr_global_error.restype = ctypes.c_char_p
    L.epr_set_samples.argtypes = [vp, ctypes.c_size_t, P, P]
    L.epr_build.argtypes = [vp]
    L.epr_set_level_system.argtypes = [vp, ctypes.c_int, P, P, ctypes.c_double]
    L.epr_set_coefficients.argtypes = [vp, ctypes.c_int, P, P]
    L.epr_get_coefficients.argtypes = [vp, ctypes.c_int, P, P]
    L.epr_energy.argtypes = [vp, ctypes.c_int, P]
    L.epr_quadfit.argtypes = [vp, ctypes.c_int, P]
    L.epr_gradient.argtypes = [vp, ctypes.c_int, P, P]
    L.epr_gs.argtypes = [vp, ctypes.c_int, ctypes.c_int]
    L.epr_prolong.argtypes = [vp, ctypes.c_int]
    L.epr_gn_matvec.argtypes = [vp, ctypes.c_int, P, P, P, P]
    L.epr_solve.argtypes = [vp, ctypes.POINTER(Stats)]
    L.epr_generate_samples.argtypes = [ctypes.c_int, ctypes.POINTER(Sampler), ctypes.c_size_t, P, P,
                                       ctypes.POINTER(ctypes.c_size_t)]
    L.epr_set_generated_samples.argtypes = [vp, ctypes.POINTER(Sampler), ctypes.c_size_t, P]
    L.epr_batch_solve.argtypes = [ctypes.POINTER(vp), ctypes.c_int, ctypes.c_int, ctypes.c_int,
                                  ctypes.POINTER(Stats), ctypes.POINTER(ctypes.c_int)]
    L.epr_batch_create.restype = vp
    L.epr_batch_create.argtypes = [ctypes.POINTER(vp), ctypes.c_int, ctypes.c_int]
    L.epr_batch_run.argtypes = [vp, ctypes.c_int, vp, vp]
    L.epr_batch_tune.argtypes = [vp, ctypes.c_int, vp]
    L.epr_batch_info.argtypes = [vp, vp, ctypes.c_int, vp, vp]
    L.epr_batch_set_tile.argtypes = [vp, ctypes.c_int, ctypes.c_int]
    L.epr_batch_destroy.argtypes = [vp]
    L.epr_batch_destroy.restype = None
    L.epr_batch_last_error.argtypes = [vp]
    L.epr_batch_last_error.restype = ctypes.c_char_p
    L.epr_get_solution.argtypes = [vp, ctypes.c_int, P, P]
    L.epr_get_array.argtypes = [vp, ctypes.c_char_p, ctypes.c_int, P, ctypes.c_size_t,
                                ctypes.POINTER(ctypes.c_size_t)]
    L.epr_synchronize.argtypes = [vp]
    L.epr_get_density.argtypes = [vp, ctypes.c_int, P, ctypes.c_size_t, ctypes.POINTER(ctypes.c_size_t)]
    L.epr_get_density_refined.argtypes = [vp, ctypes.c_int, vp, ctypes.c_size_t, ctypes.POINTER(ctypes.c_size_t)]
    L.epr_write_density_tree.argtypes = [vp, P, ctypes.c_char_p]
    L.epr_write_tree.argtypes = [vp, P, ctypes.c_char_p]
    L.epr_get_regular_coefficients.argtypes = [vp, P, P]
    I64 = ctypes.POINTER(ctypes.c_int64)
    L.epr_get_adaptive_index.argtypes = [vp, ctypes.c_int, I64, I64, ctypes.c_size_t, I64, ctypes.c_size_t]
    L.epr_time_kernel.argtypes = [vp, ctypes.c_char_p, ctypes.c_int, ctypes.c_int, P]
    L.epr_energy_noalloc.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_int, vp, vp, vp,
                                     ctypes.c_double, vp, vp]
    L.epr_noalloc_last_error.restype = ctypes.c_char_p
    L.epr_linear_gs.argtypes = [vp, ctypes.c_int, P, P, P, ctypes.c_int]
    L.epr_mg_vcycle.argtypes = [vp, ctypes.c_int, P, P, P, ctypes.c_int, ctypes.c_int]
    L.epr_alternating_system.argtypes = [vp, ctypes.c_int, ctypes.c_int, P, P]
    L.epr_alternating_solve.argtypes = [vp, ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_int]
    L.epr_biquadratic_fit.argtypes = [vp, ctypes.c_int, P, P, ctypes.c_int, P]
    L.epr_step_size.argtypes = [P, P]
    L.epr_newton_update.argtypes = [P, ctypes.c_int, P]
    # learned warm start (tensor-core U-Net)
    F = ctypes.POINTER(ctypes.c_float)
    L.epr_conv3.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_int, vp, ctypes.c_int, vp, vp, vp,
                            ctypes.c_int, ctypes.c_int, ctypes.c_int, vp]
    L.epr_conv3_wgrad.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_int, vp, ctypes.c_int, vp,
                                  ctypes.c_int, vp, vp, ctypes.c_size_t, vp]
    L.epr_conv3_wgrad_scratch.restype = ctypes.c_size_t
    L.epr_conv3_wgrad_scratch.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_int]
    L.epr_conv_last_error.restype = ctypes.c_char_p
    L.epr_unet_create.restype = vp
    L.epr_unet_create.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_uint64]
    L.epr_unet_destroy.argtypes = [vp]
    L.epr_unet_last_error.restype = ctypes.c_char_p
    L.epr_unet_last_error.argtypes = [vp]
    L.epr_unet_params.argtypes = [vp, F, ctypes.c_size_t, ctypes.POINTER(ctypes.c_size_t), ctypes.c_int]
    L.epr_unet_grid.argtypes = [vp, ctypes.POINTER(ctypes.c_int), ctypes.POINTER(ctypes.c_size_t),
                                ctypes.POINTER(ctypes.c_size_t)]
    L.epr_unet_input.argtypes = [vp, vp, vp]
    L.epr_unet_target.argtypes = [vp, vp, vp]
    L.epr_unet_forward.argtypes = [vp, vp, vp, P, vp]
    L.epr_unet_gradients.argtypes = [vp, vp, vp, F, P]
    L.epr_unet_train_step.argtypes = [vp, ctypes.c_int, ctypes.POINTER(vp), ctypes.POINTER(vp), ctypes.c_float, P]
    L.epr_unet_warm_start.argtypes = [vp, vp, P]
    _lib = L
    return L


def _p(a: np.ndarray):
    assert a.dtype == np.float64 and a.flags["C_CONTIGUOUS"]
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_double))


def step_size(q) -> float:
    """stepSize (SystemEnergy.h:256-270) on a 3 x 3 bi-quadratic fit."""
    s = np.zeros(1)
    rc = load().epr_step_size(_p(np.ascontiguousarray(q, np.float64)), _p(s))
    if rc != EPR_OK:
        raise EprError(f"[{rc}] step size")
    return float(s[0])


def newton_update(q, steps=10) -> np.ndarray:
    """newtonUpdate (SystemEnergy.h:272-303) on a 3 x 3 bi-quadratic fit."""
    st = np.zeros(2)
    rc = load().epr_newton_update(_p(np.ascontiguousarray(q, np.float64)), steps, _p(st))
    if rc != EPR_OK:
        raise EprError(f"[{rc}] newton update")
    return st


def default_params(**kw) -> Params:
    p = Params()
    load().epr_default_params(ctypes.byref(p))
    for k, v in kw.items():
        k = _FLAG_NAMES.get(k, k)
        if k == "precision" and isinstance(v, str):
            v = {"fp64": EPR_FP64, "fp32": EPR_FP32}[v.lower()]
        if k == "band_precision" and isinstance(v, str):
            v = {"fp64": EPR_BAND_FP64, "df": EPR_BAND_DF}[v.lower()]
        if k == "solver" and isinstance(v, str):
            v = {"cascadic": EPR_SOLVER_CASCADIC, "multigrid": EPR_SOLVER_MULTIGRID}[v.lower()]
        setattr(p, k, v)
    return p


def unit_cube(pos_world: np.ndarray, scale: float = 1.1):
    """ExteriorPoisson::ToUnitCube (ExteriorPoisson.h:100-123): centre the bounding box, scale by
    1/(max extent * scale), shift by 1/2.  Returns (mapped positions, (Dim+1)^2 matrix in the
    reference's (column, row) layout)."""
    pos = np.asarray(pos_world, dtype=np.float64)
    if pos.shape[0] == 0:
        raise ValueError("Expected some samples: 0")
    dim = pos.shape[1]
    lo, hi = pos.min(axis=0), pos.max(axis=0)
    ext = float((hi - lo).max())
    k = 1.0 / (ext * scale)
    t = (-(lo + hi) / 2.0) * k + 0.5
    xf = np.zeros((dim + 1, dim + 1))
    for d in range(dim):
        xf[d, d] = k
        xf[dim, d] = t[d]
    xf[dim, dim] = 1.0
    return pos * k + t, xf


def pack_skew(frames: np.ndarray) -> np.ndarray:
    return samples.pack_skew(frames)


class Reconstructor:
    """One reconstruction problem on the GPU (mirrors ExteriorPoisson::Reconstructor)."""

    def __init__(self, dim: int, depth: int, pos_unit=None, skew_packed=None, build: bool = True, **params):
        L = load()
        self.dim, self.depth = int(dim), int(depth)
        self.params = default_params(**params)
        self._h = L.epr_create(self.dim, self.depth, ctypes.byref(self.params))
        if not self._h:
            raise EprError(L.epr_global_error().decode())
        self.stats = Stats()
        if pos_unit is not None:
            self.set_samples(pos_unit, skew_packed)
            if build:
                self.build()

    def close(self):
        if getattr(self, "_h", None):
            load().epr_destroy(self._h)
            self._h = None

    def __del__(self):
        self.close()

    def _check(self, rc):
        if rc != EPR_OK:
            raise EprError(f"[{rc}] " + load().epr_last_error(self._h).decode())

    def nodes(self, level: int) -> int:
        return (2 ** level + 1) ** self.dim

    # ---------------------------------------------------------------- setup
    def set_samples(self, pos_unit, skew_packed):
        pos = np.ascontiguousarray(pos_unit, dtype=np.float64)
        sk = np.ascontiguousarray(skew_packed, dtype=np.float64)
        if pos.ndim != 2 or pos.shape[1] != self.dim or sk.shape != (pos.shape[0], self.dim * (self.dim - 1) // 2):
            raise ValueError("positions must be n x dim and frames n x dim(dim-1)/2")
        self._check(load().epr_set_samples(self._h, pos.shape[0], _p(pos), _p(sk)))

    def build(self):
        self._check(load().epr_build(self._h))

    def set_generated_samples(self, sp: Sampler, n: int):
        """Samples generated on the GPU and mapped to the unit cube there; returns the map."""
        xf = np.zeros((self.dim + 1) * (self.dim + 1))
        self._check(load().epr_set_generated_samples(self._h, ctypes.byref(sp), n, _p(xf)))
        return xf.reshape(self.dim + 1, self.dim + 1)

    def set_level_system(self, level, R, B, c):
        R = np.ascontiguousarray(R, dtype=np.float64)
        B = np.ascontiguousarray(B, dtype=np.float64)
        self._check(load().epr_set_level_system(self._h, level, _p(R), _p(B), float(c)))

    def get(self, name: str, level: int = 0) -> np.ndarray:
        n = ctypes.c_size_t(0)
        self._check(load().epr_get_array(self._h, name.encode(), level, None, 0, ctypes.byref(n)))
        out = np.zeros(n.value)
        self._check(load().epr_get_array(self._h, name.encode(), level, _p(out), n.value, ctypes.byref(n)))
        return out

    def density(self, level: int) -> np.ndarray:
        """The density estimator's data at the vertices of `level`: (nodes, 1 + dim + dim^2) =
        weight sum, position sum, covariance sum (TreeEstimator, GridSamples.h:232-277)."""
        n = ctypes.c_size_t(0)
        self._check(load().epr_get_density(self._h, level, None, 0, ctypes.byref(n)))
        out = np.zeros(n.value)
        self._check(load().epr_get_density(self._h, level, _p(out), n.value, ctypes.byref(n)))
        return out.reshape(self.nodes(level), -1)

    def density_refined(self, t: int) -> np.ndarray:
        """1 where the density tree's depth-t cell has children ((2^t)^dim flags, axis 0 most
        significant)."""
        n = ctypes.c_size_t(0)
        self._check(load().epr_get_density_refined(self._h, t, None, 0, ctypes.byref(n)))
        out = np.zeros(n.value, np.uint8)
        self._check(load().epr_get_density_refined(self._h, t, out.ctypes.data_as(ctypes.c_void_p), n.value, ctypes.byref(n)))
        return out

    def write_density_tree(self, path: str, voxel_to_world: np.ndarray):
        """The reference's <out>.density.tree (ExteriorPoissonRecon.cpp:272-277) for this build;
        voxel_to_world is (dim+1)^2 doubles in the .tree's (column, row) order."""
        xf = np.ascontiguousarray(voxel_to_world, dtype=np.float64).ravel()
        if xf.size != (self.dim + 1) ** 2:
            raise ValueError("voxel_to_world must hold (dim+1)^2 values")
        self._check(load().epr_write_density_tree(self._h, _p(xf), os.fsencode(path)))

    def write_tree(self, path: str, voxel_to_world: np.ndarray):
        """The reference's <out>.tree (ExteriorPoissonRecon.cpp:259-270) for the last solve, with the
        context's indexer (regular grid or adaptive); voxel_to_world as for write_density_tree."""
        xf = np.ascontiguousarray(voxel_to_world, dtype=np.float64).ravel()
        if xf.size != (self.dim + 1) ** 2:
            raise ValueError("voxel_to_world must hold (dim+1)^2 values")
        self._check(load().epr_write_tree(self._h, _p(xf), os.fsencode(path)))

    def regular_coefficients(self):
        """The finest level's coefficients as the reference's regularCoefficients computes them from
        the solve's hierarchical levels (Hat.adaptive.inl:154-176)."""
        n = self.nodes(self.depth)
        x, y = np.zeros(n), np.zeros(n)
        self._check(load().epr_get_regular_coefficients(self._h, _p(x), _p(y)))
        return x, y

    def adaptive_index(self, level: int) -> dict:
        """The adaptive indexer's tables of a level: `fnodes` (grid node of every function index,
        the `active` first ones relaxed) and `enodes` (grid element of every element index)."""
        I64 = ctypes.POINTER(ctypes.c_int64)
        counts = np.zeros(3, np.int64)
        self._check(load().epr_get_adaptive_index(self._h, level, counts.ctypes.data_as(I64), None, 0, None, 0))
        fn = np.zeros(max(int(counts[0]), 1), np.int64)
        en = np.zeros(max(int(counts[2]), 1), np.int64)
        self._check(load().epr_get_adaptive_index(self._h, level, counts.ctypes.data_as(I64), fn.ctypes.data_as(I64), fn.size,
                                                  en.ctypes.data_as(I64), en.size))
        return {"fnodes": fn[:counts[0]], "active": int(counts[1]), "enodes": en[:counts[2]]}

    # ---------------------------------------------------------------- per-level operators
    def set_coefficients(self, level, x, y):
        self._check(load().epr_set_coefficients(self._h, level, _p(np.ascontiguousarray(x, np.float64)),
                                                 _p(np.ascontiguousarray(y, np.float64))))

    def coefficients(self, level):
        x = np.zeros(self.nodes(level))
        y = np.zeros(self.nodes(level))
        self._check(load().epr_get_coefficients(self._h, level, _p(x), _p(y)))
        return x, y

    def energy(self, level, x=None, y=None):
        if x is not None:
            self.set_coefficients(level, x, y)
        out = np.zeros(3)
        self._check(load().epr_energy(self._h, level, _p(out)))
        return out

    def quadfit(self, level, x=None, y=None):
        if x is not None:
            self.set_coefficients(level, x, y)
        out = np.zeros((self.nodes(level), 5))
        self._check(load().epr_quadfit(self._h, level, _p(out)))
        return out

    def gradient(self, level, x=None, y=None):
        if x is not None:
            self.set_coefficients(level, x, y)
        gx = np.zeros(self.nodes(level))
        gy = np.zeros(self.nodes(level))
        self._check(load().epr_gradient(self._h, level, _p(gx), _p(gy)))
        return gx, gy

    def gs(self, level, x=None, y=None, iters=1):
        if x is not None:
            self.set_coefficients(level, x, y)
        self._check(load().epr_gs(self._h, level, iters))
        return self.coefficients(level)

    def prolong(self, level):
        self._check(load().epr_prolong(self._h, level))

    def gn_matvec(self, level, dx, dy):
        ox = np.zeros(self.nodes(level))
        oy = np.zeros(self.nodes(level))
        self._check(load().epr_gn_matvec(self._h, level, _p(np.ascontiguousarray(dx, np.float64)),
                                         _p(np.ascontiguousarray(dy, np.float64)), _p(ox), _p(oy)))
        return ox, oy

    # ---------------------------------------------------------------- linear multigrid / alternating solve
    def linear_gs(self, level, M, b, v, iters=1):
        """iters coloured Gauss-Seidel sweeps of M v = b (GSRelaxer, MG.h:57-72); returns v."""
        v = np.array(v, dtype=np.float64)
        self._check(load().epr_linear_gs(self._h, level, _p(np.ascontiguousarray(M, np.float64)),
                                         _p(np.ascontiguousarray(b, np.float64)), _p(v), iters))
        return v

    def mg_vcycle(self, level, M, b, v, gs_iters=2, cycles=1):
        """cycles V-cycles of M v = b (MGSolver::vCycle, MG.h:150-187); returns v."""
        v = np.array(v, dtype=np.float64)
        self._check(load().epr_mg_vcycle(self._h, level, _p(np.ascontiguousarray(M, np.float64)),
                                         _p(np.ascontiguousarray(b, np.float64)), _p(v), gs_iters, cycles))
        return v

    def alternating_system(self, level, which):
        """(M, b) of one alternating half-step: which 1 solves for y, 0 for x."""
        M = np.zeros((self.nodes(level), 3 ** self.dim))
        b = np.zeros(self.nodes(level))
        self._check(load().epr_alternating_system(self._h, level, which, _p(M), _p(b)))
        return M, b

    def alternating_solve(self, level, iters=1, vcycles=1, gs_iters=2, single_level=False):
        """AlternatingSolve (ExteriorPoissonSolvers.h:86-154) on the level's coefficients."""
        self._check(load().epr_alternating_solve(self._h, level, iters, vcycles, gs_iters, int(single_level)))
        return self.coefficients(level)

    def biquadratic_fit(self, level, dx, dy, as_reference=False):
        """3 x 3 coefficients q[i, j] of s^i t^j of E(x + s dx, y + t dy)."""
        q = np.zeros((3, 3))
        self._check(load().epr_biquadratic_fit(self._h, level, _p(np.ascontiguousarray(dx, np.float64)),
                                               _p(np.ascontiguousarray(dy, np.float64)), int(as_reference), _p(q)))
        return q

    def time_kernel(self, kernel: str, level: int, reps: int = 20) -> float:
        """Mean device time (ms) of one launch of a kernel family (CUDA events on the context's stream)."""
        ms = np.zeros(1)
        self._check(load().epr_time_kernel(self._h, kernel.encode(), level, reps, _p(ms)))
        return float(ms[0])

    # ---------------------------------------------------------------- solve
    def solve(self):
        self._check(load().epr_solve(self._h, ctypes.byref(self.stats)))
        return self.stats.as_dict()

    def x(self, level):
        x = np.zeros(self.nodes(level))
        y = np.zeros(self.nodes(level))
        self._check(load().epr_get_solution(self._h, level, _p(x), _p(y)))
        return x

    def y(self, level):
        x = np.zeros(self.nodes(level))
        y = np.zeros(self.nodes(level))
        self._check(load().epr_get_solution(self._h, level, _p(x), _p(y)))
        return y

    def solution(self):
        xs, ys = [], []
        for l in range(self.depth + 1):
            x = np.zeros(self.nodes(l))
            y = np.zeros(self.nodes(l))
            self._check(load().epr_get_solution(self._h, l, _p(x), _p(y)))
            xs.append(x)
            ys.append(y)
        return xs, ys


def batch_solve(recons, build: bool = True, threads: int = 0):
    """Builds (when `build`) and solves several Reconstructors at once on one GPU
    (epr_batch_solve): host workers drive whole reconstructions on their own streams, so the
    kernels of small reconstructions overlap.  Each result is the one its Reconstructor gives
    alone.  Returns the per-reconstruction stats dicts; raises EprError naming the first failure."""
    recons = list(recons)
    n = len(recons)
    L = load()
    handles = (ctypes.c_void_p * max(n, 1))(*[r._h for r in recons])
    stats = (Stats * max(n, 1))()
    status = (ctypes.c_int * max(n, 1))()
    rc = L.epr_batch_solve(handles, n, int(bool(build)), int(threads), stats, status)
    for i, r in enumerate(recons):
        if status[i] == EPR_OK:
            ctypes.memmove(ctypes.byref(r.stats), ctypes.byref(stats[i]), ctypes.sizeof(Stats))
    if rc != EPR_OK:
        raise EprError(f"[{rc}] " + L.epr_global_error().decode())
    return [stats[i].as_dict() for i in range(n)]


class LockstepBatch:
    """Many 3D Reconstructors solved in lockstep (epr_batch_*): one launch per level colour for all
    of them, the relaxation one CUDA graph, block shapes per level from the autotuner.  Each
    result is the one its Reconstructor gives alone."""

    def __init__(self, recons, threads: int = 0):
        self.recons = list(recons)
        L = load()
        n = len(self.recons)
        self._handles = (ctypes.c_void_p * max(n, 1))(*[r._h for r in self.recons])
        self._h = L.epr_batch_create(self._handles, n, int(threads))
        if not self._h:
            raise EprError(L.epr_batch_last_error(None).decode())

    def _check(self, rc):
        if rc != EPR_OK:
            raise EprError(f"[{rc}] " + load().epr_batch_last_error(self._h).decode())

    def run(self, build: bool = False):
        """Builds (when `build`) and solves every member; returns their stats dicts."""
        n = len(self.recons)
        stats = (Stats * max(n, 1))()
        status = (ctypes.c_int * max(n, 1))()
        rc = load().epr_batch_run(self._h, int(bool(build)), ctypes.byref(stats), ctypes.byref(status))
        for i, r in enumerate(self.recons):
            if status[i] == EPR_OK:
                ctypes.memmove(ctypes.byref(r.stats), ctypes.byref(stats[i]), ctypes.sizeof(Stats))
        self._check(rc)
        return [stats[i].as_dict() for i in range(n)]

    def tune(self, reps: int = 3) -> np.ndarray:
        """Runs the autotuner; returns the (tuned levels, 3) mean sweep times per block shape."""
        out = np.zeros(3 * 32)
        self._check(load().epr_batch_tune(self._h, int(reps), out.ctypes.data_as(ctypes.c_void_p)))
        rows = out.reshape(-1, 3)
        return rows[:int(np.count_nonzero(rows.any(axis=1)))]

    def set_tile(self, level: int, tile: int):
        """Block shape index (0-2) of `level`'s colour kernel (level -1: every level)."""
        self._check(load().epr_batch_set_tile(self._h, int(level), int(tile)))

    def info(self) -> dict:
        tiles = (ctypes.c_int * 16)()
        ms = ctypes.c_double(0)
        launches = ctypes.c_longlong(0)
        self._check(load().epr_batch_info(self._h, tiles, 16, ctypes.byref(ms), ctypes.byref(launches)))
        return {"tiles": list(tiles), "relax_ms": ms.value, "graph_launches": launches.value}

    def close(self):
        if getattr(self, "_h", None):
            load().epr_batch_destroy(self._h)
            self._h = None

    def __del__(self):
        self.close()
