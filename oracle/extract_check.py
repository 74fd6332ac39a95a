"""Acceptance check of `.tree` output with the reference's own zero-set extraction (test
infrastructure; needs oracle/_ref/Extract and oracle/_ref/ExteriorPoissonRecon, built by
`make -C oracle ref` where the reference checkout is present).

    python oracle/extract_check.py --ply in.ply --depth D --ours ours.tree [--ours other.tree ...]

runs the reference command line on the PLY (regular grid, same flags), extracts the zero set of its
`.tree` and of every given `.tree` with the reference's Extract (marching simplices), and prints the
symmetric Hausdorff distance between the extracted curves/surfaces in units of the finest cell
(world extent x 1.1 / 2^depth).  Each polyline edge / triangle is resampled at a tenth of a cell
so that the distance is between the sets, not just their vertices.
"""
from __future__ import annotations

import argparse
import json
import os
import subprocess
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
sys.path.insert(0, ROOT)


def read_mesh(path):
    """Vertices (n x dim) and faces (lists of vertex indices) of a binary little-endian PLY."""
    with open(path, "rb") as f:
        data = f.read()
    end = data.index(b"end_header\n") + len(b"end_header\n")
    header = data[:end].decode().splitlines()
    nv = nf = 0
    vprops = []
    cur = None
    for line in header:
        t = line.split()
        if t[:2] == ["element", "vertex"]:
            nv, cur = int(t[2]), "v"
        elif t[:2] == ["element", "face"]:
            nf, cur = int(t[2]), "f"
        elif t[0] == "property" and cur == "v":
            vprops.append((t[2], t[1]))
    sizes = {"double": 8, "float": 4}
    vt = np.dtype([(n, "<f8" if ty == "double" else "<f4") for n, ty in vprops])
    verts = np.frombuffer(data, dtype=vt, count=nv, offset=end)
    coords = [n for n, _ in vprops if n in ("x", "y", "z", "w")]
    V = np.stack([verts[c].astype(np.float64) for c in coords], axis=1)
    off = end + nv * vt.itemsize
    faces = []
    for _ in range(nf):
        k = int.from_bytes(data[off:off + 4], "little", signed=True)
        idx = np.frombuffer(data, dtype="<i4", count=k, offset=off + 4)
        faces.append(idx.copy())
        off += 4 + 4 * k
    del sizes
    return V, faces


def resample(V, faces, h):
    """Points on every edge (2-vertex faces) or triangle (3-vertex faces) at spacing ~h."""
    pts = [V]
    for f in faces:
        if len(f) == 2:
            a, b = V[f[0]], V[f[1]]
            n = max(1, int(np.ceil(np.linalg.norm(b - a) / h)))
            t = np.linspace(0, 1, n + 1)[:, None]
            pts.append(a + t * (b - a))
        elif len(f) == 3:
            a, b, c = V[f[0]], V[f[1]], V[f[2]]
            n = max(1, int(np.ceil(max(np.linalg.norm(b - a), np.linalg.norm(c - a)) / h)))
            for i in range(n + 1):
                for j in range(n + 1 - i):
                    pts.append((a + (b - a) * i / n + (c - a) * j / n)[None])
    return np.concatenate(pts, axis=0)


def hausdorff(P, Q):
    from scipy.spatial import cKDTree
    d1 = cKDTree(Q).query(P)[0].max() if len(P) else 0.0
    d2 = cKDTree(P).query(Q)[0].max() if len(Q) else 0.0
    return float(max(d1, d2))


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--ply", required=True)
    ap.add_argument("--depth", type=int, required=True)
    ap.add_argument("--ours", action="append", required=True)
    ap.add_argument("--flags", default="")
    a = ap.parse_args()
    ref_cli = os.path.join(HERE, "_ref", "ExteriorPoissonRecon")
    extract = os.path.join(HERE, "_ref", "Extract")
    from exteriorpoissonrecon_gb300 import samples
    pos, _ = samples.read_ply(a.ply)
    ext = float((pos.max(0) - pos.min(0)).max())
    cell = ext * 1.1 / 2 ** a.depth
    with tempfile.TemporaryDirectory() as td:
        ref = os.path.join(td, "ref")
        subprocess.run([ref_cli, "--in", a.ply, "--out", ref, "--depth", str(a.depth), "--aRadius", "-1"] + a.flags.split(),
                       check=True, capture_output=True)
        meshes = {}
        for name, tree in [("reference", ref + ".tree")] + [(t, t) for t in a.ours]:
            out = os.path.join(td, f"m{len(meshes)}.ply")
            subprocess.run([extract, "--in", tree, "--out", out], check=True, capture_output=True)
            V, F = read_mesh(out)
            meshes[name] = resample(V, F, cell / 10)
        res = {"cell": cell}
        for t in a.ours:
            res[os.path.basename(t)] = hausdorff(meshes["reference"], meshes[t]) / cell
        print(json.dumps(res))


if __name__ == "__main__":
    main()
