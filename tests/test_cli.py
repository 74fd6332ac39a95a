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
    r = subprocess.run([cli, "--in", "x.ply", "--aRadius", "6"], capture_output=True, text=True)
    assert r.returncode == 2 and "[0,5]" in r.stderr
    r = subprocess.run([cli, "--in", "x.ply", "--aRadius", "2", "--solver", "multigrid"], capture_output=True, text=True)
    assert r.returncode == 2 and "cascadic" in r.stderr
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


def _write(path, data: bytes):
    with open(path, "wb") as f:
        f.write(data)


def test_faulty_input_files_fail_cleanly(cli):
    """Host-side fault injection: truncated, garbled and incomplete PLY files and an empty sample
    set end with a non-zero exit and a message, before any device work (the reference prints and
    exits 0, Exceptions.h:102-107)."""
    pos, fr = samples.torus_knot(64)
    with tempfile.TemporaryDirectory() as td:
        good = os.path.join(td, "good.ply")
        samples.write_ply(good, pos, fr)
        raw = open(good, "rb").read()
        cases = {
            "truncated.ply": (raw[:-100], "truncated"),
            "garbled.ply": (b"plx" + raw[3:], "not a PLY"),
            "noframes.ply": (raw.replace(b"property double skew_2_2\n", b""), "skew_2_2"),
            "empty.ply": (raw[:raw.index(b"end_header\n") + 11].replace(b"element vertex 64", b"element vertex 0"),
                          "Expected some samples"),
            "missing.ply": (None, "cannot open"),
        }
        for name, (data, msg) in cases.items():
            path = os.path.join(td, name)
            if data is not None:
                _write(path, data)
            r = subprocess.run([cli, "--in", path, "--out", os.path.join(td, "o"), "--depth", "3"], capture_output=True,
                               text=True, timeout=120)
            assert r.returncode != 0 and msg in r.stderr, (name, r.returncode, r.stderr)
            assert not os.path.exists(os.path.join(td, "o.tree"))


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
        # the fixtures of the regular grid were written with --aRadius -1 (the default is 3)
        r = subprocess.run([cli, "--in", ply, "--out", out, "--grid", out, "--depth", str(depth), "--aRadius", "-1"] +
                           list(g["flags"]), capture_output=True, text=True)
        assert r.returncode == 0, r.stderr
        with open(out + ".tree", "rb") as f:
            mine = parse_tree(f.read())
        grids = []
        for c in range(2):
            with open(out + f".{c}.grid", "rb") as f:
                grids.append(f.read())
    ref = parse_tree(g["tree"].tobytes())
    assert mine[0] == ref[0] and mine[1] == ref[1] and mine[5] == ref[5]
    assert np.allclose(mine[2], ref[2], rtol=1e-14, atol=1e-14)
    for a, b in zip(mine[3] + mine[4], ref[3] + ref[4]):
        assert a.shape == b.shape
        assert np.abs(a - b).max() <= 1e-9 * max(np.abs(b).max(), 1e-30)
    # the regular coefficient grid against the one the reference's Extract writes from the
    # reference's own .tree (regularCoefficients, Hat.adaptive.inl:154-176; RegularGrid::Write,
    # RegularGrid.inl:441-472): the same text header (dimensions and transform) and the same values
    dim = ref[0]
    n = (2 ** depth + 1) ** dim
    for c, mine_grid in enumerate(grids):
        want = g[f"grid{c}"].tobytes()
        assert mine_grid[:-8 * n] == want[:-8 * n], (mine_grid[:200], want[:200])
        a = np.frombuffer(mine_grid[-8 * n:], "<f8")
        b = np.frombuffer(want[-8 * n:], "<f8")
        assert np.abs(a - b).max() <= 1e-9 * np.abs(b).max()
