"""Writes the golden fixtures of tests/golden/*.npz from the reference implementation itself.

Run in a checkout that has the reference sources (the fixtures are committed, so the tests never
need them):

    make -C oracle ref              # builds oracle/_ref/ref_harness from the reference headers
    python tests/golden/make_golden.py

Each fixture stores the exact inputs (world positions and packed skew frames as the reference's
PLY reader returns them) and the reference's outputs for them: unit-cube positions, ordered
cells, estimator measure / noise / depth per sample, the splatted frame field S(E), leaf depths,
the system matrices of selected levels as column stencils, energies / quadratic fits / one paired
Gauss-Seidel sweep for seeded random coefficients, and the cascadic solve result.
"""
from __future__ import annotations

import os
import subprocess
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from exteriorpoissonrecon_gb300 import samples  # noqa: E402

HARNESS = os.path.join(ROOT, "oracle", "_ref", "ref_harness")
REF_CLI = os.path.join(ROOT, "oracle", "_ref", "ExteriorPoissonRecon")

# name, workload, sample count, seed, depth, levels whose full stencils are stored
CASES = [
    ("knot3_d4", "knot", 4096, 0, 4, [2, 4]),
    ("link3_d4", "link", 6000, 3, 4, [1, 4]),
    ("cliff4_d3", "clifford", 4000, 5, 3, [1, 2]),
    # the plain-method configuration exactly: (3,2) torus knot, 4096 samples regular in t, no
    # noise, depth 5 (33^3 nodes)
    # (stencils of level 3 only, and no multigrid probes: those are pinned at depth 4 already)
    ("knot3_d5", "knot", 4096, 0, 5, [3]),
]
SLIM = {"knot3_d5"}

# solver variants of the reference's CLI: name, base case, extra harness flags
VARIANTS = [
    ("knot3_d4_separate", "knot", 4096, 0, 4, ["--separate", "1"]),
    ("knot3_d4_single", "knot", 4096, 0, 4, ["--singleLevel", "1", "--gsIters", "40"]),
    ("knot3_d4_seed7_min2", "knot", 4096, 0, 4, ["--seed", "7", "--minSolveDepth", "2", "--iMult", "1.5"]),
    # --project: the reference's blade projection of S(E) (its FitBlade of every element with the
    # command line's full iteration budget) and, in 3D, the whole solve on the projected system
    ("knot3_d4_project", "knot", 4096, 0, 4, ["--project", "1"]),
    ("cliff4_d3_project", "clifford", 4000, 5, 3, ["--project", "1"]),
    # the same schedule variants with the adaptive indexer (a narrow band, so that inactive indexed
    # functions carry the random start, the prolongation and the hierarchical output)
    ("link3_d5_a1_separate", "link", 6000, 3, 5, ["--aRadius", "1", "--separate", "1"]),
    ("link3_d5_a1_single", "link", 6000, 3, 5, ["--aRadius", "1", "--singleLevel", "1", "--gsIters", "40"]),
    ("link3_d5_a1_seed7_min3", "link", 6000, 3, 5, ["--aRadius", "1", "--seed", "7", "--minSolveDepth", "3", "--iMult", "1.5"]),
]

# the adaptive indexer (--aRadius K >= 0, the reference command line's default is 3): name, workload,
# sample count, seed, depth, K, levels whose stencils are stored
ADAPTIVE = [
    ("knot3_d5_a1", "knot", 4096, 0, 5, 1, [3, 5]),
    ("link3_d5_a0", "link", 6000, 3, 5, 0, [2, 5]),
    ("link3_d5_a3", "link", 6000, 3, 5, 3, []),
    ("cliff4_d3_a1", "clifford", 4000, 5, 3, 1, [3]),
]


def make_adaptive(name, workload, n, seed, depth, K, stencil_levels):
    """The adaptive indexer's tables (function and element order, active count per level), the
    system of selected levels, energies / one sweep / prolongation for seeded coefficients on the
    indexed functions, and the cascadic solve, all written densely on each level's grid."""
    pos, frames = samples.make_workload(workload, n, seed=seed)
    with tempfile.TemporaryDirectory() as td:
        ply = os.path.join(td, "in.ply")
        samples.write_ply(ply, pos, frames)
        out = os.path.join(td, "dump")
        subprocess.run([HARNESS, ply, str(depth), out, "--aRadius", str(K)], check=True)
        L = lambda k: np.load(os.path.join(out, k + ".npy"))  # noqa: E731
        fx = {"depth": np.array(depth), "a_radius": np.array(K), "pos": L("pos"), "skew": L("skew"), "c": L("c"),
              "sol_energies": L("sol_energies"), "solX": L("solX"), "solY": L("solY"),
              "indexer_hash": L("indexer_hash"), "stencil_levels": np.array(stencil_levels)}
        for l in range(depth + 1):
            for k in ("afn", "ael", "aact", "energies", "xr", "yr", "solx", "soly"):
                fx[f"{k}_d{l}"] = L(f"{k}_d{l}")
            if l < depth:
                fx[f"prolong_d{l}"] = L(f"prolong_d{l}")
        for l in stencil_levels:
            fx[f"R_d{l}"] = L(f"R_d{l}")
            fx[f"B_d{l}"] = L(f"B_d{l}")
        for l in sorted({depth, max(depth - 2, 0)}):
            for k in ("quadfit", "gsx", "gsy"):
                fx[f"{k}_d{l}"] = L(f"{k}_d{l}")
    path = os.path.join(HERE, name + ".npz")
    np.savez_compressed(path, **fx)
    print(f"{path}: {os.path.getsize(path) / 1e6:.2f} MB")


def make_variant(name, workload, n, seed, depth, flags):
    """Solve results only (the system is the base case's)."""
    pos, frames = samples.make_workload(workload, n, seed=seed)
    with tempfile.TemporaryDirectory() as td:
        ply = os.path.join(td, "in.ply")
        samples.write_ply(ply, pos, frames)
        out = os.path.join(td, "dump")
        subprocess.run([HARNESS, ply, str(depth), out] + flags, check=True)
        L = lambda k: np.load(os.path.join(out, k + ".npy"))  # noqa: E731
        fx = {"depth": np.array(depth), "pos": L("pos"), "skew": L("skew"), "flags": np.array(flags),
              "sol_energies": L("sol_energies"), "solX": L("solX"), "solY": L("solY")}
        for l in range(depth + 1):
            fx[f"solx_d{l}"] = L(f"solx_d{l}")
            fx[f"soly_d{l}"] = L(f"soly_d{l}")
        if os.path.exists(os.path.join(out, "S_project.npy")):
            fx["S"] = L("S")
            fx["S_project"] = L("S_project")
    path = os.path.join(HERE, name + ".npz")
    np.savez_compressed(path, **fx)
    print(f"{path}: {os.path.getsize(path) / 1e6:.2f} MB")


def make(name, workload, n, seed, depth, stencil_levels):
    pos, frames = samples.make_workload(workload, n, seed=seed)
    with tempfile.TemporaryDirectory() as td:
        ply = os.path.join(td, "in.ply")
        samples.write_ply(ply, pos, frames)
        out = os.path.join(td, "dump")
        subprocess.run([HARNESS, ply, str(depth), out], check=True)
        L = lambda k: np.load(os.path.join(out, k + ".npy"))  # noqa: E731
        fx = {
            "depth": np.array(depth),
            "world_pos": L("world_pos"),
            "skew": L("skew"),
            "pos": L("pos"),
            "world_to_unit": L("world_to_unit"),
            "cells": L("cells"),
            "cell_counts": L("cell_counts"),
            "est_measure": L("est_measure"),
            "est_noise": L("est_noise"),
            "est_depth": L("est_depth"),
            "S": L("S"),
            "leaf_depth": L("leaf_depth"),
            "c": L("c"),
            "sol_energies": L("sol_energies"),
            "solX": L("solX"),
            "solY": L("solY"),
            "indexer_hash": L("indexer_hash"),
            "stencil_levels": np.array(stencil_levels),
        }
        for l in range(depth + 1):
            fx[f"energies_d{l}"] = L(f"energies_d{l}")
            fx[f"xr_d{l}"] = L(f"xr_d{l}")
            fx[f"yr_d{l}"] = L(f"yr_d{l}")
            fx[f"solx_d{l}"] = L(f"solx_d{l}")
            fx[f"soly_d{l}"] = L(f"soly_d{l}")
            if l < depth:
                fx[f"prolong_d{l}"] = L(f"prolong_d{l}")
        for l in stencil_levels:
            fx[f"R_d{l}"] = L(f"R_d{l}")
            fx[f"B_d{l}"] = L(f"B_d{l}")
        # quadratic fits and one GS sweep at the finest level and one coarse level
        for l in sorted({depth, max(depth - 2, 0)}):
            fx[f"quadfit_d{l}"] = L(f"quadfit_d{l}")
            fx[f"gsx_d{l}"] = L(f"gsx_d{l}")
            fx[f"gsy_d{l}"] = L(f"gsy_d{l}")
        for l in range(depth + 1):
            fx[f"density_l{l}"] = L(f"density_l{l}")
            fx[f"skew_l{l}"] = L(f"skew_l{l}")
        for k in ("mg_M", "mg_b", "mg_gs1", "mg_v1", "mg_v2", "qa_x", "qa_y", "qa_dx", "qa_dy", "qa_u", "qa_v",
                  "qa_gx", "qa_gy", "qa_biquad", "qa_step", "qa_newton"):
            if name not in SLIM:
                fx[k] = L(k)
    path = os.path.join(HERE, name + ".npz")
    np.savez_compressed(path, **fx)
    print(f"{path}: {os.path.getsize(path) / 1e6:.2f} MB")


REF_EXTRACT = os.path.join(ROOT, "oracle", "_ref", "Extract")
REF_SIMPLICES = os.path.join(ROOT, "oracle", "_ref", "ref_simplices")


def read_mesh(path):
    """Vertex positions and polygon index lists of the reference's binary PLY output."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    from extract_check import read_mesh as rm
    return rm(path)


def make_simplices():
    """The reference's oriented simplices of the unit cube (3D and 4D) as printed by
    oracle/ref_simplices."""
    out = subprocess.run([REF_SIMPLICES], check=True, capture_output=True, text=True).stdout.splitlines()
    fx, i = {}, 0
    while i < len(out):
        _, dim, _, num = out[i].split()
        dim, num = int(dim), int(num)
        rows = [list(map(int, out[i + 1 + k].split())) for k in range(num)]
        fx[f"simplices{dim}"] = np.array(rows, dtype=np.int64).reshape(num, dim + 1, dim)
        i += 1 + num
    path = os.path.join(HERE, "cube_simplices.npz")
    np.savez_compressed(path, **fx)
    print(f"{path}: {os.path.getsize(path) / 1e6:.3f} MB")


def make_zero_set(name, workload, n, seed, depth, ref_tree=None):
    """The reference Extract's zero set of the reference's own reconstruction of a named workload
    (positions are regenerated from the seeded generator; `ref_tree` reuses a .tree made already)."""
    with tempfile.TemporaryDirectory() as td:
        out = os.path.join(td, "out")
        tree = ref_tree
        energies = None
        if tree is None:
            pos, frames = samples.make_workload(workload, n, seed=seed)
            ply = os.path.join(td, "in.ply")
            samples.write_ply(ply, pos, frames)
            r = subprocess.run([REF_CLI, "--in", ply, "--out", out, "--depth", str(depth), "--aRadius", "-1", "--verbose"],
                               check=True, capture_output=True, text=True)
            tree = out + ".tree"
            energies = r.stdout.strip().splitlines()[-1]
        subprocess.run([REF_EXTRACT, "--in", tree, "--out", out + "_zero.ply"], check=True, capture_output=True)
        V, F = read_mesh(out + "_zero.ply")
    if energies is None and os.environ.get("EPR_REF_LOG"):
        # the verbose log of the run that wrote `ref_tree`: its final energy and time lines
        with open(os.environ["EPR_REF_LOG"]) as f:
            lines = [l.strip() for l in f if l.strip().startswith(("Error:", "Executed"))]
        energies = " | ".join(lines)
    # float32 positions (1e-7 relative, far below the 0.1-cell criterion) keep the fixture small
    fx = {"depth": np.array(depth), "workload": np.array(workload), "n": np.array(n), "seed": np.array(seed),
          "zero_vertices": V.astype(np.float32),
          "zero_simplices": np.array([list(f) for f in F], dtype=np.int32).reshape(len(F), -1)}
    if energies:
        fx["log"] = np.array(energies)
    path = os.path.join(HERE, name + ".npz")
    np.savez_compressed(path, **fx)
    print(f"{path}: {os.path.getsize(path) / 1e6:.2f} MB, {len(V)} vertices")


def make_tree(name, workload, n, seed, depth, flags):
    """The reference command line's own .tree and .density.tree outputs for a PLY input (frames
    stored in full), and the regular coefficient grids the reference's Extract writes from the
    .tree (--grid)."""
    pos, frames = samples.make_workload(workload, n, seed=seed)
    with tempfile.TemporaryDirectory() as td:
        ply = os.path.join(td, "in.ply")
        samples.write_ply(ply, pos, frames)
        out = os.path.join(td, "out")
        radius = [] if "--aRadius" in flags else ["--aRadius", "-1"]
        subprocess.run([REF_CLI, "--in", ply, "--out", out, "--depth", str(depth)] + radius + flags,
                       check=True, capture_output=True)
        with open(out + ".tree", "rb") as f:
            tree = np.frombuffer(f.read(), dtype=np.uint8)
        with open(out + ".density.tree", "rb") as f:
            density_tree = np.frombuffer(f.read(), dtype=np.uint8)
        subprocess.run([REF_EXTRACT, "--in", out + ".tree", "--grid", out, "--out", out + "_zero.ply"], check=True,
                       capture_output=True)
        grids = []
        for c in range(2):
            with open(out + f".{c}.grid", "rb") as f:
                grids.append(np.frombuffer(f.read(), dtype=np.uint8))
        V, F = read_mesh(out + "_zero.ply")
    fx = {"depth": np.array(depth), "world_pos": pos, "frames": frames, "flags": np.array(flags, dtype=str), "tree": tree,
          "grid0": grids[0], "grid1": grids[1], "density_tree": density_tree}
    if pos.shape[1] == 3:  # the zero curve (the oracle's extraction is 3D)
        fx["zero_vertices"] = V
        fx["zero_simplices"] = np.array([list(f) for f in F], dtype=np.int64).reshape(len(F), -1)
    path = os.path.join(HERE, name + ".npz")
    np.savez_compressed(path, **fx)
    print(f"{path}: {os.path.getsize(path) / 1e6:.2f} MB")


if __name__ == "__main__":
    if not os.path.exists(HARNESS):
        sys.exit("build the reference harness first: make -C oracle ref")
    only = set(sys.argv[1:])  # fixture names to (re)write; all when none are given
    TREES = [("knot3_d4_tree", "knot", 4096, 0, 4, []), ("cliff4_d3_tree", "clifford", 3000, 9, 3, ["--gsIters", "5"]),
             # the reference command line's default indexer (--aRadius 3), and a narrow one in 4D
             ("link3_d5_a3_tree", "link", 6000, 3, 5, ["--aRadius", "3"]),
             ("cliff4_d3_a1_tree", "clifford", 3000, 9, 3, ["--aRadius", "1", "--gsIters", "5"])]
    # the reference's zero set of the benchmark's input (3D link, 1.1M samples, depth 8): the
    # reference run takes ~6 minutes on 8 cores
    ZERO_SETS = [("link3_d8_zero_set", "link", 1_000_000, 0, 8)]
    if only:
        for case in CASES:
            if case[0] in only:
                make(*case)
        for v in VARIANTS:
            if v[0] in only:
                make_variant(*v)
        for case in ADAPTIVE:
            if case[0] in only:
                make_adaptive(*case)
        for case in TREES:
            if case[0] in only:
                make_tree(*case)
        if "cube_simplices" in only:
            make_simplices()
        for case in ZERO_SETS:
            if case[0] in only:
                # EPR_REF_TREE: a .tree the reference already wrote for this input (and EPR_REF_LOG
                # its verbose log), instead of running the reference here
                make_zero_set(*case, ref_tree=os.environ.get("EPR_REF_TREE"))
        sys.exit(0)
    for case in CASES:
        make(*case)
    for v in VARIANTS:
        make_variant(*v)
    for case in ADAPTIVE:
        make_adaptive(*case)
    for case in TREES:
        make_tree(*case)
    make_simplices()
    for case in ZERO_SETS:
        make_zero_set(*case)
