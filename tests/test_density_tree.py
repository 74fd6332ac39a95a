"""The `.density.tree` output (the density estimator's tree, ExteriorPoissonRecon.cpp:272-277):
the restatement of its layout (oracle/density_tree.py) against the bytes the reference's own
command line wrote for the tree fixtures' inputs, and the command line's file against the same
bytes on the GPU.

Compared: the node sequence (depth, offset, whether the node has children) exactly, the XForm and
the trailer exactly, the node data within 1e-12 relative to the largest magnitude (the sums are
formed in another order); the pointer words and the padding word are memory addresses and
uninitialised bytes in the reference's file and are not compared."""
import os
import subprocess
import tempfile

import numpy as np
import pytest

from conftest import load_golden
from exteriorpoissonrecon_gb300 import samples
from oracle import density_tree as DT
from oracle import oracle as O

# the estimator does not depend on the indexer; the adaptive fixtures come from the default command line
TREE_CASES = ["knot3_d4_tree", "cliff4_d3_tree", "link3_d5_a3_tree", "cliff4_d3_a1_tree"]


def _reference(name):
    g = load_golden(name)
    dim = g["world_pos"].shape[1]
    return g, dim, DT.parse(g["density_tree"].tobytes(), dim)


def assert_same_tree(got: dict, ref: dict):
    assert len(got["depth"]) == len(ref["depth"])
    assert np.array_equal(got["depth"], ref["depth"])
    assert np.array_equal(got["offset"], ref["offset"])
    assert np.array_equal(got["has_children"], ref["has_children"])
    assert np.array_equal(got["xform"], ref["xform"])
    assert got["trailer"] == ref["trailer"]
    scale = np.abs(ref["data"]).max()
    assert np.abs(got["data"] - ref["data"]).max() <= 1e-12 * scale


@pytest.mark.parametrize("name", TREE_CASES)
def test_layout_restatement_reads_the_reference_file(name):
    g, dim, ref = _reference(name)
    raw = g["density_tree"].tobytes()
    node, _, _ = DT.layout(dim)
    assert node == (136 if dim == 3 else 208)
    assert ref["trailer"] == 2.0 ** (dim - 2)
    # the root, then blocks of 2^dim siblings; exterior nodes (offset beyond the vertex range of
    # their depth) and the root hold no density
    assert ref["depth"][0] == 0 and (len(ref["depth"]) - 1) % (1 << dim) == 0
    r = (1 << np.maximum(ref["depth"] - 1, 0))
    ext = (ref["offset"] > r[:, None]).any(axis=1) | (ref["depth"] == 0)
    assert ext.any() and not ref["data"][ext].any()
    # the XForm is the .tree's voxel-to-world transform
    assert np.array_equal(ref["xform"], np.frombuffer(g["tree"].tobytes(), "<f8", (dim + 1) ** 2, 20))
    # the restatement writes the file back (pointer and padding words aside)
    again = DT.parse(DT.serialize(dim, ref["xform"], ref["depth"], ref["offset"], ref["has_children"], ref["data"]), dim)
    assert_same_tree(again, ref)
    assert len(raw) == 8 + 8 * (dim + 1) ** 2 + node * len(ref["depth"]) + 8


@pytest.mark.parametrize("name", TREE_CASES)
def test_oracle_tree_matches_reference_file(name):
    """Refinement flags and regular density levels of the oracle's estimator, written in the
    reference's node order, give the reference's file."""
    g, dim, ref = _reference(name)
    depth = int(g["depth"])
    pos, _ = O.unit_cube(g["world_pos"])
    o = O.Oracle(dim, depth)
    o.set_samples(pos, samples.pack_skew(g["frames"]))
    o.build()
    refined = [o.get("density_refined", t).astype(np.uint8) for t in range(depth + 2)]
    dens = [o.get("density", l) for l in range(depth + 1)]
    d, off, has = DT.nodes(dim, refined)
    data = DT.node_data(dim, d, off, dens)
    got = DT.parse(DT.serialize(dim, ref["xform"], d, off, has, data), dim)
    assert_same_tree(got, ref)


@pytest.fixture(scope="module")
def cli():
    import exteriorpoissonrecon_gb300 as epr
    from exteriorpoissonrecon_gb300.build import build_cli
    epr.load()
    return build_cli()


@pytest.mark.gpu
@pytest.mark.parametrize("name", TREE_CASES)
def test_cli_density_tree_matches_reference_file(cli, name):
    """The command line's <out>.density.tree for the fixture's input against the reference's."""
    g, dim, ref = _reference(name)
    depth = int(g["depth"])
    with tempfile.TemporaryDirectory() as td:
        ply = os.path.join(td, "in.ply")
        samples.write_ply(ply, g["world_pos"], g["frames"])
        out = os.path.join(td, "out")
        r = subprocess.run([cli, "--in", ply, "--out", out, "--depth", str(depth), "--aRadius", "-1"] + list(g["flags"]),
                           capture_output=True, text=True, timeout=300)
        assert r.returncode == 0, r.stderr
        with open(out + ".density.tree", "rb") as f:
            raw = f.read()
    got = DT.parse(raw, dim)
    # the transform is the command line's own (the same bounding box arithmetic as the reference)
    assert np.allclose(got["xform"], ref["xform"], rtol=1e-14, atol=1e-14)
    got["xform"] = ref["xform"]
    assert_same_tree(got, ref)
    # pointer words: zero parents, children words 1 exactly where children follow
    node, ptr, _ = DT.layout(dim)
    rec = np.frombuffer(raw, np.uint8, node * len(got["depth"]), 8 + 8 * (dim + 1) ** 2).reshape(-1, node)
    assert not rec[:, ptr:ptr + 8].any()
    assert np.array_equal(rec[:, ptr + 8:ptr + 16].copy().view("<u8")[:, 0], got["has_children"].astype(np.uint64))


@pytest.mark.gpu
@pytest.mark.parametrize("name", TREE_CASES)
def test_api_refinement_and_writer_match_oracle(tmp_path, name):
    """epr_get_density_refined against the oracle's tree structure at every depth, and
    Reconstructor.write_density_tree against the restatement of the file from those flags and the
    oracle's density levels."""
    import exteriorpoissonrecon_gb300 as epr
    g, dim, ref = _reference(name)
    depth = int(g["depth"])
    pos, _ = O.unit_cube(g["world_pos"])
    sk = samples.pack_skew(g["frames"])
    o = O.Oracle(dim, depth)
    o.set_samples(pos, sk)
    o.build()
    r = epr.Reconstructor(dim, depth, pos, sk)
    try:
        for t in range(depth + 2):
            assert np.array_equal(r.density_refined(t), o.get("density_refined", t).astype(np.uint8)), t
        path = str(tmp_path / "t.density.tree")
        r.write_density_tree(path, ref["xform"])
        with open(path, "rb") as f:
            got = DT.parse(f.read(), dim)
    finally:
        r.close()
    assert_same_tree(got, ref)
    with pytest.raises(epr.EprError):
        epr.Reconstructor(dim, depth, pos, sk).write_density_tree(str(tmp_path / "no" / "such" / "dir" / "x"), ref["xform"])
