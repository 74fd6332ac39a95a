"""Seeded synthetic point+frame generators and the PLY sample format.

The reconstruction input is a set of points in R^Dim (Dim = 3 or 4), each carrying a
Dim x Dim skew-symmetric "frame" matrix.  The reference reads them from a PLY file whose
vertex element holds ``x y z [w]`` and ``skew_<c>_<r>`` doubles
(ExteriorPoissonRecon/ExteriorPoissonRecon.cpp:282-303, property naming
Misha/PlyVertexData.inl:228-234: entry (c, r) of the matrix is ``skew_c_r``).

Frame conventions follow the reference's sample tool:
  * curves in 3D: the Hodge dual of the unit tangent, S_ij = eps_ijk T_k
    (Include/Samples.h:73-79);
  * the Clifford torus in 4D: the tangent bivector d_u ^ d_v (Include/Samples.h:818-838).

The shapes are the ones the benchmark configurations name (torus knot, Hopf-style link of two
unit circles, Clifford torus, helices).  Noise follows the reference's sampler
(Sample/Sample.cpp:137-199): Gaussian positional noise in unit-cube units, a random rotation of
the frame by a normally distributed angle, and a fraction of uniform "spot" outliers.
"""
from __future__ import annotations

import math
import numpy as np

# ---------------------------------------------------------------------------------------------
# frames
# ---------------------------------------------------------------------------------------------

def curve_frames(tangents: np.ndarray) -> np.ndarray:
    """Hodge dual of unit tangents: M[i, j] = eps_ijk T_k (n x 3 x 3)."""
    t = tangents / np.linalg.norm(tangents, axis=1, keepdims=True)
    n = t.shape[0]
    m = np.zeros((n, 3, 3))
    m[:, 0, 1] = t[:, 2]
    m[:, 1, 0] = -t[:, 2]
    m[:, 1, 2] = t[:, 0]
    m[:, 2, 1] = -t[:, 0]
    m[:, 2, 0] = t[:, 1]
    m[:, 0, 2] = -t[:, 1]
    return m


def bivector_frames(a: np.ndarray, b: np.ndarray) -> np.ndarray:
    """Skew matrix of the bivector a ^ b, normalised: M = (a b^T - b a^T) / |.|_F."""
    m = a[:, :, None] * b[:, None, :] - b[:, :, None] * a[:, None, :]
    nrm = np.sqrt((m * m).sum(axis=(1, 2)))
    return m / nrm[:, None, None]


# ---------------------------------------------------------------------------------------------
# shapes
# ---------------------------------------------------------------------------------------------

def torus_knot(n: int, p: int = 2, q: int = 3, regular: bool = True, rng=None):
    """(p,q) torus knot ((2+cos qt) cos pt, (2+cos qt) sin pt, sin qt)."""
    if regular:
        t = np.arange(n) * (2.0 * math.pi / n)
    else:
        t = rng.uniform(0.0, 2.0 * math.pi, n)
    r = 2.0 + np.cos(q * t)
    pos = np.stack([r * np.cos(p * t), r * np.sin(p * t), np.sin(q * t)], axis=1)
    dr = -q * np.sin(q * t)
    tan = np.stack([dr * np.cos(p * t) - r * p * np.sin(p * t),
                    dr * np.sin(p * t) + r * p * np.cos(p * t),
                    q * np.cos(q * t)], axis=1)
    return pos, curve_frames(tan)


def link(n: int, rng):
    """Two interlocking unit circles: one in the xy-plane at the origin, one in the xz-plane
    centred at (1,0,0); samples uniform in arc length (both circles have the same length)."""
    t = rng.uniform(0.0, 2.0 * math.pi, n)
    which = rng.integers(0, 2, n)
    c, s = np.cos(t), np.sin(t)
    pos = np.where(which[:, None] == 0,
                   np.stack([c, s, np.zeros(n)], axis=1),
                   np.stack([1.0 + c, np.zeros(n), s], axis=1))
    tan = np.where(which[:, None] == 0,
                   np.stack([-s, c, np.zeros(n)], axis=1),
                   np.stack([-s, np.zeros(n), c], axis=1))
    return pos, curve_frames(tan)


def helix(n: int, turns: float, rng, radius: float = 0.3, height: float = 1.0):
    """Helix of the given radius along z with `turns` rotations over `height`."""
    t = rng.uniform(0.0, 1.0, n)
    a = 2.0 * math.pi * turns * t
    pos = np.stack([radius * np.cos(a), radius * np.sin(a), height * t], axis=1)
    tan = np.stack([-radius * 2 * math.pi * turns * np.sin(a),
                    radius * 2 * math.pi * turns * np.cos(a),
                    np.full(n, height)], axis=1)
    return pos, curve_frames(tan)


def clifford_torus(n: int, rng):
    """(cos u, sin u, cos v, sin v)/sqrt(2), (u,v) uniform on [0,2pi)^2; frame d_u ^ d_v."""
    u = rng.uniform(0.0, 2.0 * math.pi, n)
    v = rng.uniform(0.0, 2.0 * math.pi, n)
    k = 1.0 / math.sqrt(2.0)
    pos = k * np.stack([np.cos(u), np.sin(u), np.cos(v), np.sin(v)], axis=1)
    du = k * np.stack([-np.sin(u), np.cos(u), np.zeros(n), np.zeros(n)], axis=1)
    dv = k * np.stack([np.zeros(n), np.zeros(n), -np.sin(v), np.cos(v)], axis=1)
    return pos, bivector_frames(du, dv)


# ---------------------------------------------------------------------------------------------
# noise (Sample/Sample.cpp:137-199 semantics)
# ---------------------------------------------------------------------------------------------

def _unit_cube_scale(pos: np.ndarray, scale: float = 1.1) -> float:
    ext = pos.max(axis=0) - pos.min(axis=0)
    return float(ext.max() * scale)


def _random_rotations(n: int, dim: int, sigma_rad: float, rng) -> np.ndarray:
    """Rotations by a N(0, sigma) angle in a uniformly random 2-plane."""
    a = rng.normal(size=(n, dim))
    a /= np.linalg.norm(a, axis=1, keepdims=True)
    b = rng.normal(size=(n, dim))
    b -= (b * a).sum(axis=1, keepdims=True) * a
    b /= np.linalg.norm(b, axis=1, keepdims=True)
    th = rng.normal(0.0, sigma_rad, n)
    eye = np.broadcast_to(np.eye(dim), (n, dim, dim)).copy()
    aa = a[:, :, None] * a[:, None, :]
    bb = b[:, :, None] * b[:, None, :]
    ab = b[:, :, None] * a[:, None, :] - a[:, :, None] * b[:, None, :]
    c = np.cos(th)[:, None, None]
    s = np.sin(th)[:, None, None]
    return eye + (c - 1.0) * (aa + bb) + s * ab


def add_noise(pos, frames, rng, pos_sigma=0.0, ang_deg=0.0, spot_frac=0.0):
    """Positional noise (sigma in unit-cube units), angular frame noise and spot outliers."""
    pos = pos.copy()
    frames = frames.copy()
    n, dim = pos.shape
    if pos_sigma > 0:
        s = _unit_cube_scale(pos)
        pos = pos + rng.normal(0.0, pos_sigma * s, pos.shape)
    if ang_deg > 0:
        r = _random_rotations(n, dim, math.radians(ang_deg), rng)
        frames = np.einsum("nji,njk,nkl->nil", r, frames, r)
    if spot_frac > 0:
        m = int(round(n * spot_frac))
        lo, hi = pos.min(axis=0), pos.max(axis=0)
        sp = rng.uniform(lo, hi, (m, dim))
        sf = rng.uniform(-1.0, 1.0, (m, dim, dim))
        sf = sf - np.transpose(sf, (0, 2, 1))
        pos = np.concatenate([pos, sp])
        frames = np.concatenate([frames, sf])
    return pos, frames


# ---------------------------------------------------------------------------------------------
# named workloads
# ---------------------------------------------------------------------------------------------

def make_workload(name: str, n: int | None = None, seed: int = 0):
    """Returns (positions n x Dim, frames n x Dim x Dim) for a named synthetic workload."""
    rng = np.random.default_rng(seed)
    if name == "knot":  # torus knot (2,3), regular in t, noiseless
        return torus_knot(n or 4096)
    if name == "link":  # two unit circles, sigma .005, 5 deg, 10% spot noise
        pos, fr = link(n or 1_000_000, rng)
        return add_noise(pos, fr, rng, 0.005, 5.0, 0.10)
    if name == "clifford":  # Clifford torus, sigma .002, 2 deg
        pos, fr = clifford_torus(n or 1_000_000, rng)
        return add_noise(pos, fr, rng, 0.002, 2.0, 0.0)
    if name == "clifford_clean":
        return clifford_torus(n or 20_000, rng)
    if name == "link_clean":
        return link(n or 20_000, rng)
    raise ValueError(f"unknown workload {name!r}")


def batch_workloads(count: int = 64, seed: int = 0, n_range=(2048, 262144), depths=(5, 6, 7)):
    """The batched-reconstruction mix: the first half torus knots with seed-drawn coprime (p, q) in
    [2, 7] (t uniform), the second half helices of radius 0.3 along z over height 1 with a rotation
    count uniform in [1, 8]; sample counts log-uniform in `n_range`, depths uniform in `depths`,
    positional sigma uniform in [0, 0.01] (unit-cube units) and angular noise uniform in [0, 10]
    degrees.  Returns a list of dicts with name, depth, pos (world) and frames."""
    rng = np.random.default_rng(seed)
    out = []
    for k in range(count):
        n = int(round(math.exp(rng.uniform(math.log(n_range[0]), math.log(n_range[1])))))
        depth = int(rng.choice(depths))
        sigma = float(rng.uniform(0.0, 0.01))
        ang = float(rng.uniform(0.0, 10.0))
        if k < count // 2:
            while True:
                p, q = (int(v) for v in rng.integers(2, 8, 2))
                if math.gcd(p, q) == 1:
                    break
            pos, fr = torus_knot(n, p, q, regular=False, rng=rng)
            name = f"knot_{p}_{q}"
        else:
            turns = float(rng.uniform(1.0, 8.0))
            pos, fr = helix(n, turns, rng)
            name = f"helix_{turns:.2f}"
        pos, fr = add_noise(pos, fr, rng, sigma, ang, 0.0)
        out.append({"name": name, "depth": depth, "pos": pos, "frames": fr, "n": n,
                    "sigma": sigma, "angle_deg": ang})
    return out


# ---------------------------------------------------------------------------------------------
# PLY
# ---------------------------------------------------------------------------------------------

def write_ply(path: str, pos: np.ndarray, frames: np.ndarray) -> None:
    """Binary little-endian PLY with x y z [w] and skew_c_r (= frames[:, c, r]) doubles."""
    n, dim = pos.shape
    names = ["x", "y", "z", "w"][:dim]
    props = names + [f"skew_{c}_{r}" for c in range(dim) for r in range(dim)]
    header = "ply\nformat binary_little_endian 1.0\n"
    header += f"element vertex {n}\n"
    header += "".join(f"property double {p}\n" for p in props)
    header += "end_header\n"
    data = np.concatenate([pos.reshape(n, dim), frames.reshape(n, dim * dim)], axis=1)
    with open(path, "wb") as f:
        f.write(header.encode("ascii"))
        f.write(np.ascontiguousarray(data, dtype="<f8").tobytes())


def read_ply(path: str):
    """Reads the PLY written by write_ply (or any binary/ascii PLY with double/float x.. and
    skew_c_r vertex properties). Returns (positions, frames)."""
    with open(path, "rb") as f:
        raw = f.read()
    end = raw.index(b"end_header") + len(b"end_header")
    while raw[end:end + 1] in (b"\r", b"\n"):
        end += 1
        if raw[end - 1:end] == b"\n":
            break
    lines = raw[:end].decode("ascii").split("\n")
    fmt, nvert, props, in_vertex = None, 0, [], False
    for ln in lines:
        tok = ln.split()
        if not tok:
            continue
        if tok[0] == "format":
            fmt = tok[1]
        elif tok[0] == "element":
            in_vertex = tok[1] == "vertex"
            if in_vertex:
                nvert = int(tok[2])
        elif tok[0] == "property" and in_vertex:
            props.append((tok[-1], tok[1]))
    tmap = {"double": "f8", "float64": "f8", "float": "f4", "float32": "f4", "int": "i4",
            "uchar": "u1", "uint8": "u1", "int32": "i4", "uint": "u4"}
    if fmt == "ascii":
        body = raw[end:].decode("ascii").split()
        arr = np.array(body[: nvert * len(props)], dtype=np.float64).reshape(nvert, len(props))
        cols = {p: arr[:, i] for i, (p, _) in enumerate(props)}
    else:
        endian = "<" if fmt == "binary_little_endian" else ">"
        dt = np.dtype([(p, endian + tmap[t]) for p, t in props])
        rec = np.frombuffer(raw[end:end + nvert * dt.itemsize], dtype=dt)
        cols = {p: rec[p].astype(np.float64) for p, _ in props}
    dim = 4 if "w" in cols else 3
    pos = np.stack([cols[c] for c in ["x", "y", "z", "w"][:dim]], axis=1)
    frames = np.zeros((nvert, dim, dim))
    for c in range(dim):
        for r in range(dim):
            frames[:, c, r] = cols[f"skew_{c}_{r}"]
    return pos, frames


def pack_skew(frames: np.ndarray) -> np.ndarray:
    """Lower-triangular packing of the skew part: p[i(i-1)/2 + j] = (m(i,j) - m(j,i)) / 2 for
    i > j, with m(c, r) the PLY entry skew_c_r (Include/Hat.inl:39-45)."""
    n, dim, _ = frames.shape
    out = []
    for i in range(dim):
        for j in range(i):
            out.append(0.5 * (frames[:, i, j] - frames[:, j, i]))
    return np.stack(out, axis=1)
