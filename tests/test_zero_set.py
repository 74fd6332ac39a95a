"""The oracle's restatement of the reference's zero-set extraction (oracle/zero_set.py) against the
reference's own Extract on the reference's own `.tree` (fixture written by
tests/golden/make_golden.py): the same segments to rounding."""
import numpy as np

from conftest import load_golden
from oracle import zero_set as Z


def test_extraction_matches_reference_extract():
    g = load_golden("knot3_d4_tree")
    simp = load_golden("cube_simplices")["simplices3"]
    segs, cell = Z.tree_zero_set(g["tree"].tobytes(), simp)
    ref = g["zero_vertices"][g["zero_simplices"]]
    assert len(segs) == len(ref)
    d = Z.curve_hausdorff(segs, ref, cell / 10)
    assert d <= 1e-9 * cell, d / cell


def test_extraction_of_adaptive_tree_matches_reference_extract():
    """The reference's Extract on its own adaptive .tree (the command line's default indexer): the
    indexer's functions scattered to their grid nodes, then regular coefficients and marching
    simplices as for the regular grid."""
    g = load_golden("link3_d5_a3_tree")
    simp = load_golden("cube_simplices")["simplices3"]
    segs, cell = Z.tree_zero_set(g["tree"].tobytes(), simp)
    ref = g["zero_vertices"][g["zero_simplices"]]
    assert len(segs) == len(ref)
    d = Z.curve_hausdorff(segs, ref, cell / 10)
    assert d <= 1e-9 * cell, d / cell


def test_simplex_table_tiles_the_cube():
    """The reference's 6 (3D) / 24 (4D) simplices each have volume 1/Dim! and positive orientation."""
    import math
    s = load_golden("cube_simplices")
    for dim in (3, 4):
        S = s[f"simplices{dim}"].astype(np.float64)
        assert S.shape == (math.factorial(dim), dim + 1, dim)
        vol = [np.linalg.det(T[1:] - T[0]) for T in S]
        assert np.allclose(vol, 1.0)  # oriented, unit determinant = dim! x volume 1/dim!
