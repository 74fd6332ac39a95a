"""The ExteriorPoissonRecon-compatible command line (exteriorpoissonrecon_gb300/epr_recon)."""
import os
import struct
import subprocess
import tempfile

import numpy as np
import pytest

import exteriorpoissonrecon_gb300 as epr
from conftest import load_golden
from exteriorpoissonrecon_gb300 import samples
from exteriorpoissonrecon_gb300.build import build_cli


@pytest.fixture(scope="module")
def cli():
    epr.load()
    return build_cli()


def parse_tree(raw: bytes):
    """The reference's .tree layout: uint32 dim, uint64 indexer hash, raw XForm (one 8-byte word
    then (dim+1)^2 doubles), x and y as vector<VectorXd>, uint32 max depth."""
    o = 0
    dim = struct.unpack_from("<I", raw, o)[0]; o += 4
    h = struct.unpack_from("<Q", raw, o)[0]; o += 8
    o += 8
    xf = np.frombuffer(raw, "<f8", (dim + 1) ** 2, o).reshape(dim + 1, dim + 1); o += 8 * (dim + 1) ** 2
    out = []
    for _ in range(2):
        nl = struct.unpack_from("<Q", raw, o)[0]; o += 8
        lv = []
        for _ in range(nl):
            n = struct.unpack_from("<q", raw, o)[0]; o += 8
            lv.append(np.frombuffer(raw, "<f8", n, o).copy()); o += 8 * n
        out.append(lv)
    md = struct.unpack_from("<I", raw, o)[0]; o += 4
    assert o == len(raw)
    return dim, h, xf, out[0], out[1], md


def test_usage_and_argument_errors(cli):
    r = subprocess.run([cli], capture_output=True, text=True)
    assert r.returncode == 0 and "--in" in r.stdout
    r = subprocess.run([cli, "--in", "x.ply", "--aRadius", "3"], capture_output=True, text=True)
    assert r.returncode == 2 and "regular grid" in r.stderr
    r = subprocess.run([cli, "--in", "x.txt"], capture_output=True, text=True)
    assert r.returncode == 2 and "ply" in r.stderr
    r = subprocess.run([cli, "--in", "x.ply", "--bogus", "1"], capture_output=True, text=True)
    assert r.returncode == 2
    r = subprocess.run([cli, "--in", "x.ply", "--precision", "fp16"], capture_output=True, text=True)
    assert r.returncode == 2 and "precision" in r.stderr
    r = subprocess.run([cli, "--in", "x.ply", "--solver", "newton"], capture_output=True, text=True)
    assert r.returncode == 2 and "solver" in r.stderr
    r = subprocess.run([cli, "--in", "x.ply", "--bandPrecision", "half"], capture_output=True, text=True)
    assert r.returncode == 2 and "bandPrecision" in r.stderr


def test_tree_parser_reads_reference_output():
    g = load_golden("knot3_d4_tree")
    dim, h, xf, xs, ys, md = parse_tree(g["tree"].tobytes())
    assert dim == 3 and h == 0x5aa89c06ecbfe5e7 and md == 4 and len(xs) == 5


@pytest.mark.gpu
@pytest.mark.parametrize("name", ["knot3_d4_tree", "cliff4_d3_tree"])
def test_cli_tree_matches_reference_tree(cli, name):
    g = load_golden(name)
    depth = int(g["depth"])
    with tempfile.TemporaryDirectory() as td:
        ply = os.path.join(td, "in.ply")
        samples.write_ply(ply, g["world_pos"], g["frames"])
        out = os.path.join(td, "out")
        r = subprocess.run([cli, "--in", ply, "--out", out, "--grid", out, "--depth", str(depth)] + list(g["flags"]),
                           capture_output=True, text=True)
        assert r.returncode == 0, r.stderr
        with open(out + ".tree", "rb") as f:
            mine = parse_tree(f.read())
        with open(out + ".0.grid", "rb") as f:
            grid = f.read()
    ref = parse_tree(g["tree"].tobytes())
    assert mine[0] == ref[0] and mine[1] == ref[1] and mine[5] == ref[5]
    assert np.allclose(mine[2], ref[2], rtol=1e-14, atol=1e-14)
    for a, b in zip(mine[3] + mine[4], ref[3] + ref[4]):
        assert a.shape == b.shape
        assert np.abs(a - b).max() <= 1e-9 * max(np.abs(b).max(), 1e-30)
    dim = ref[0]
    assert grid.startswith(f"G{dim}\n1 DOUBLE\n".encode())
    # finest regular coefficients = sum of the prolonged hierarchical levels
    n = (2 ** depth + 1) ** dim
    assert grid[-8 * n:] and len(np.frombuffer(grid[-8 * n:], "<f8")) == n
