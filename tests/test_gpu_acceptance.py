"""Acceptance of the command line's `.tree` output by the reference's criterion: the zero set that
the reference's Extract would extract from it (restated in oracle/zero_set.py, pinned to Extract
by tests/test_zero_set.py) lies within 0.1 finest cell (symmetric Hausdorff distance) of the zero
set Extract extracted from the reference's own `.tree` of the same input (Extract/Extract.cpp:96-331).
Density trimming (Extract.cpp:217-238) is not applied: it needs the `.density.tree`, which the
command line does not write."""
import os
import subprocess
import tempfile

import numpy as np
import pytest

import exteriorpoissonrecon_gb300 as epr
from conftest import load_golden
from exteriorpoissonrecon_gb300 import samples
from exteriorpoissonrecon_gb300.build import build_cli
from oracle import zero_set as Z

pytestmark = pytest.mark.gpu

HEADLINE = ["--precision", "fp32", "--fp64From", "0", "--fp64Levels", "4", "--bandPrecision", "df"]


@pytest.fixture(scope="module")
def cli():
    epr.load()
    return build_cli()


def _zero_set_distance(cli, pos, frames, depth, flags, ref_vertices, ref_simplices):
    simp = load_golden("cube_simplices")["simplices3"]
    with tempfile.TemporaryDirectory() as td:
        ply = os.path.join(td, "in.ply")
        samples.write_ply(ply, pos, frames)
        out = os.path.join(td, "out")
        r = subprocess.run([cli, "--in", ply, "--out", out, "--depth", str(depth), "--aRadius", "-1"] + flags, capture_output=True,
                           text=True)
        assert r.returncode == 0, r.stderr
        with open(out + ".tree", "rb") as f:
            segs, cell = Z.tree_zero_set(f.read(), simp)
    ref = ref_vertices[ref_simplices]
    d = Z.curve_hausdorff(segs, ref, cell / 10)
    return d / cell, len(segs), len(ref)


@pytest.mark.parametrize("flags,bound", [([], 1e-6), (HEADLINE, 0.1)])
def test_zero_set_of_knot_matches_reference(cli, flags, bound):
    g = load_golden("knot3_d4_tree")
    d, n, nref = _zero_set_distance(cli, g["world_pos"], g["frames"], int(g["depth"]), list(g["flags"]) + flags,
                                    g["zero_vertices"], g["zero_simplices"])
    assert d <= bound, (d, n, nref)


def test_zero_set_of_benchmark_input_matches_reference(cli):
    """The benchmark's input (3D link, 1M samples + 10% outliers, depth 8) solved in the benchmark's
    precision configuration: its zero set within 0.1 cell of the reference's."""
    g = load_golden("link3_d8_zero_set")
    pos, frames = samples.make_workload(str(g["workload"]), int(g["n"]), seed=int(g["seed"]))
    d, n, nref = _zero_set_distance(cli, pos, frames, int(g["depth"]), HEADLINE, g["zero_vertices"], g["zero_simplices"])
    assert d <= 0.1, (d, n, nref)
