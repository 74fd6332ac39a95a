"""Restatement of the reference's zero-set extraction for the regular grid (test infrastructure
only): what Extract does with a `.tree` of the regular indexer (Extract/Extract.cpp:96-262).

    * regular coefficients of the finest level: level 0, then x_d + P x_{d-1} with the multilinear
      prolongation P (regularCoefficients, Hat.adaptive.inl:154-176);
    * every finest cell that can contain a zero is split into the reference's simplices of the unit
      hypercube (HyperCubeSimplices, Misha/HyperCubeSimplices.h:51-185, oriented as
      RegularSubGridTriangulation orients them, Misha/MarchingSimplices.h:623-660; the table itself
      is dumped from the reference by oracle/ref_simplices.cpp into tests/golden/cube_simplices.npz),
      with the nodal values (x, y) at the corners (the hat basis interpolates them);
    * on each simplex the zero set of the linear interpolant of (x, y) is found face by face: on a
      codimension-two face (a triangle in 3D) the barycentric coordinates a with
      s0 + sum_i a_i (s_i - s0) = 0 are solved and the point is kept when every a_i is in [0, 1]
      (_AddLevelSet, Misha/MarchingSimplices.h:409-500); in 3D a tetrahedron's points form its
      segment of the zero curve;
    * vertices go to world coordinates by the `.tree`'s voxel-to-world transform.

Cells are pre-selected by a necessary condition (both fields change sign or vanish on the cell's
corners), which leaves the extracted set unchanged.  The comparison samples each curve's segments
at a tenth of a cell and measures exact point-to-segment distances to the other curve (symmetric
Hausdorff distance; scipy's k-d tree finds the candidate segments).
"""
from __future__ import annotations

import struct

import numpy as np


def parse_tree(raw: bytes):
    """(dim, indexer hash, voxel-to-world (dim+1)^2, x levels, y levels, max depth) of a `.tree`."""
    o = 0
    dim = struct.unpack_from("<I", raw, o)[0]; o += 4
    h = struct.unpack_from("<Q", raw, o)[0]; o += 8
    o += 8  # the XForm object's leading word
    xf = np.frombuffer(raw, "<f8", (dim + 1) ** 2, o).reshape(dim + 1, dim + 1).copy(); o += 8 * (dim + 1) ** 2
    out = []
    for _ in range(2):
        nl = struct.unpack_from("<Q", raw, o)[0]; o += 8
        lv = []
        for _ in range(nl):
            n = struct.unpack_from("<q", raw, o)[0]; o += 8
            lv.append(np.frombuffer(raw, "<f8", n, o).copy()); o += 8 * n
        out.append(lv)
    md = struct.unpack_from("<I", raw, o)[0]; o += 4
    return dim, h, xf, out[0], out[1], md


def prolong_nodes(c: np.ndarray, dim: int) -> np.ndarray:
    """Multilinear prolongation of node values from resolution r to 2r (axis 0 slowest)."""
    n = round(len(c) ** (1.0 / dim))
    a = c.reshape((n,) * dim)
    for ax in range(dim):
        shape = list(a.shape)
        shape[ax] = 2 * n - 1
        b = np.zeros(shape)
        sl_even = [slice(None)] * dim
        sl_even[ax] = slice(0, None, 2)
        b[tuple(sl_even)] = a
        sl_odd = [slice(None)] * dim
        sl_odd[ax] = slice(1, None, 2)
        lo = [slice(None)] * dim
        hi = [slice(None)] * dim
        lo[ax] = slice(0, n - 1)
        hi[ax] = slice(1, n)
        b[tuple(sl_odd)] = 0.5 * (a[tuple(lo)] + a[tuple(hi)])
        a = b
    return a.reshape(-1)


def regular_finest(levels, dim: int) -> np.ndarray:
    x = levels[0]
    for d in range(1, len(levels)):
        x = levels[d] + prolong_nodes(x, dim)
    return x


def zero_set_3d(X: np.ndarray, Y: np.ndarray, depth: int, simplices: np.ndarray) -> np.ndarray:
    """Segments (m, 2, 3) of the zero set of (X, Y) (finest-level node values, (2^depth+1)^3,
    axis 0 slowest) in grid units."""
    n = 2 ** depth + 1
    Xg, Yg = X.reshape(n, n, n), Y.reshape(n, n, n)
    # corner values of every cell: (r, r, r, 8)
    corners = [(a, b, c) for a in (0, 1) for b in (0, 1) for c in (0, 1)]

    def cell_vals(G):
        return np.stack([G[a:a + n - 1, b:b + n - 1, c:c + n - 1] for a, b, c in corners], axis=-1)

    cx, cy = cell_vals(Xg), cell_vals(Yg)
    cand = (cx.min(-1) <= 0) & (cx.max(-1) >= 0) & (cy.min(-1) <= 0) & (cy.max(-1) >= 0)
    cells = np.argwhere(cand)  # (k, 3)
    if len(cells) == 0:
        return np.zeros((0, 2, 3))
    segs = []
    tri_faces = [(1, 2, 3), (0, 2, 3), (0, 1, 3), (0, 1, 2)]
    for simp in simplices:  # (4, 3) 0/1 coordinates
        V = cells[:, None, :] + simp[None, :, :]  # (k, 4, 3) grid vertices
        vx = Xg[V[..., 0], V[..., 1], V[..., 2]]
        vy = Yg[V[..., 0], V[..., 1], V[..., 2]]
        pts, ok = [], []
        for f in tri_faces:
            i0, i1, i2 = f
            # s0 + a1 (s1 - s0) + a2 (s2 - s0) = 0
            m00, m01 = vx[:, i1] - vx[:, i0], vx[:, i2] - vx[:, i0]
            m10, m11 = vy[:, i1] - vy[:, i0], vy[:, i2] - vy[:, i0]
            det = m00 * m11 - m01 * m10
            with np.errstate(divide="ignore", invalid="ignore"):
                a1 = (-vx[:, i0] * m11 + vy[:, i0] * m01) / det
                a2 = (-vy[:, i0] * m00 + vx[:, i0] * m10) / det
            a0 = 1 - a1 - a2
            good = (det != 0) & (a0 >= 0) & (a0 <= 1) & (a1 >= 0) & (a1 <= 1) & (a2 >= 0) & (a2 <= 1)
            p = a0[:, None] * V[:, i0] + a1[:, None] * V[:, i1] + a2[:, None] * V[:, i2]
            pts.append(p)
            ok.append(good)
        pts = np.stack(pts, axis=1)  # (k, 4, 3)
        ok = np.stack(ok, axis=1)    # (k, 4)
        cnt = ok.sum(1)
        for k in np.nonzero(cnt >= 2)[0]:
            P = pts[k][ok[k]]
            for j in range(1, len(P)):
                if np.abs(P[j] - P[0]).max() > 0:
                    segs.append(np.stack([P[0], P[j]]))
    return np.array(segs).reshape(-1, 2, 3)


def to_world(points: np.ndarray, xf: np.ndarray) -> np.ndarray:
    """Apply the `.tree`'s voxel-to-world transform (stored column-major: xf[col, row])."""
    dim = points.shape[-1]
    M = xf.T  # row-major (dim+1)^2
    return points @ M[:dim, :dim].T + M[:dim, dim]


def resample_segments(segs: np.ndarray, h: float) -> np.ndarray:
    pts = [segs.reshape(-1, segs.shape[-1])]
    for a, b in segs:
        n = max(1, int(np.ceil(np.linalg.norm(b - a) / h)))
        t = np.linspace(0, 1, n + 1)[:, None]
        pts.append(a + t * (b - a))
    return np.concatenate(pts, axis=0)


def hausdorff(P: np.ndarray, Q: np.ndarray) -> float:
    """Symmetric Hausdorff distance of two point sets."""
    from scipy.spatial import cKDTree
    if len(P) == 0 or len(Q) == 0:
        return 0.0 if len(P) == len(Q) else float("inf")
    return float(max(cKDTree(Q).query(P)[0].max(), cKDTree(P).query(Q)[0].max()))


def _point_segment_distance(P, A, B):
    d = B - A
    L2 = (d * d).sum(-1)
    t = np.where(L2 > 0, ((P - A) * d).sum(-1) / np.where(L2 > 0, L2, 1), 0.0)
    t = np.clip(t, 0.0, 1.0)
    return np.linalg.norm(P - (A + t[..., None] * d), axis=-1)


def directed_distance(segs_a: np.ndarray, segs_b: np.ndarray, h: float) -> float:
    """max over points of the curve A (its segments sampled every h) of the distance to the curve B
    (exact point-to-segment distances).  Candidate segments of B are the k nearest by midpoint; a
    point is settled once its k-th nearest midpoint is farther than its best distance plus half the
    longest segment of B (no unexamined segment can then come closer), else k grows."""
    from scipy.spatial import cKDTree
    if len(segs_a) == 0:
        return 0.0
    if len(segs_b) == 0:
        return float("inf")
    P = resample_segments(segs_a, h)
    mids = 0.5 * (segs_b[:, 0] + segs_b[:, 1])
    half = 0.5 * float(np.linalg.norm(segs_b[:, 1] - segs_b[:, 0], axis=1).max())
    tree = cKDTree(mids)
    best = np.full(len(P), np.inf)
    todo = np.arange(len(P))
    k = 16
    while len(todo):
        kk = min(k, len(segs_b))
        dk, idx = tree.query(P[todo], kk)
        dk, idx = dk.reshape(len(todo), kk), idx.reshape(len(todo), kk)
        dist = _point_segment_distance(P[todo][:, None, :], segs_b[idx, 0], segs_b[idx, 1]).min(axis=1)
        best[todo] = dist
        settled = (kk == len(segs_b)) | (dk[:, -1] > dist + half)
        todo = todo[~settled]
        k *= 4
    return float(best.max())


def curve_hausdorff(segs_a: np.ndarray, segs_b: np.ndarray, h: float) -> float:
    """Symmetric Hausdorff distance of two polylines given as segment lists."""
    return max(directed_distance(segs_a, segs_b, h), directed_distance(segs_b, segs_a, h))


def tree_levels(raw: bytes):
    """(dim, voxel-to-world, x levels, y levels, max depth) of a `.tree` of either indexer, every
    level dense on its (2^l+1)^dim grid (the adaptive indexer's functions scattered to their nodes,
    zero elsewhere, as regularCoefficients's ToRegular does, Hat.adaptive.inl:159-165)."""
    h = struct.unpack_from("<Q", raw, 4)[0]
    try:
        from . import adapted_tree as AT
    except ImportError:
        import adapted_tree as AT
    if h not in AT.HASH.values():
        dim, _, xf, xs, ys, md = parse_tree(raw)
        return dim, xf, xs, ys, md
    t = AT.parse(raw)
    dim = t["dim"]
    xs, ys = [], []
    for l in range(len(t["x"])):
        r1 = 2 ** l + 1
        sel = (t["depth"] == l + 1) & (t["findex"] >= 0)
        nodes = np.ravel_multi_index(t["offset"][sel].T, (r1,) * dim)
        for src, dst in ((t["x"][l], xs), (t["y"][l], ys)):
            v = np.zeros(r1 ** dim)
            v[nodes] = src[t["findex"][sel]]
            dst.append(v)
    return dim, t["xform"].reshape(dim + 1, dim + 1), xs, ys, len(xs) - 1


def tree_zero_set(raw: bytes, simplices: np.ndarray):
    """World-space segments of the zero set of a 3D `.tree` and the world size of a finest cell."""
    dim, xf, xs, ys, md = tree_levels(raw)
    assert dim == 3
    X, Y = regular_finest(xs, dim), regular_finest(ys, dim)
    segs = zero_set_3d(X, Y, md, simplices)
    world = to_world(segs.reshape(-1, 3), xf).reshape(-1, 2, 3)
    cell = float(np.abs(np.linalg.det(xf.T[:3, :3])) ** (1 / 3))
    return world, cell
