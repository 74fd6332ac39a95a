import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")


GOLDEN = os.path.join(ROOT, "tests", "golden")
# fixtures with every probe the harness writes (including the multigrid and bi-quadratic probes)
GOLDEN_CASES = ["knot3_d4", "link3_d4", "cliff4_d3"]
# every fixture of a full build + solve: the cases above plus the plain-method configuration
# exactly as specified (torus knot, 4096 regular samples, depth 5), which stores the build, the
# energies, fits, sweeps and the solve but not the probes pinned at depth 4 already
SOLVE_CASES = GOLDEN_CASES + ["knot3_d5"]


def load_golden(name):
    import numpy as np
    return dict(np.load(os.path.join(GOLDEN, name + ".npz")))


VARIANT_CASES = ["knot3_d4_separate", "knot3_d4_single", "knot3_d4_seed7_min2", "link3_d5_a1_separate",
                 "link3_d5_a1_single", "link3_d5_a1_seed7_min3"]
# the adaptive indexer (--aRadius K): fixtures of its tables, system, probes and solve; and the
# reference command line's own adaptive .tree files
ADAPTIVE_CASES = ["knot3_d5_a1", "link3_d5_a0", "link3_d5_a3", "cliff4_d3_a1"]
ADAPTIVE_TREES = {"link3_d5_a3_tree": 3, "cliff4_d3_a1_tree": 1}


def variant_params(flags):
    """Harness flags of a variant fixture -> parameter keywords (the reference's flag names)."""
    conv = {"--separate": ("separate", int), "--singleLevel": ("singleLevel", int), "--gsIters": ("gsIters", int),
            "--seed": ("seed", int), "--minSolveDepth": ("minSolveDepth", int), "--iMult": ("iMult", float),
            "--aRadius": ("aRadius", int)}
    flags = [str(f) for f in flags]
    out = {}
    for k, v in zip(flags[0::2], flags[1::2]):
        name, cast = conv[k]
        out[name] = cast(v)
    return out


def stencil_apply(G, v, dim, level):
    """out_j = sum_i G(j, i) v_i for a column stencil G[i, o] = G(i + off(o), i) (numpy, tests only)."""
    import numpy as np
    r = 1 << level
    N = (r + 1) ** dim
    idx = np.array(np.unravel_index(np.arange(N), (r + 1,) * dim)).T
    out = np.zeros(N)
    for o in range(3 ** dim):
        off = np.array(np.unravel_index(o, (3,) * dim)) - 1
        J = idx + off
        ok = np.all((J >= 0) & (J <= r), axis=1)
        j = np.ravel_multi_index(J[ok].T, (r + 1,) * dim)
        np.add.at(out, j, G[ok, o] * v[ok])
    return out
