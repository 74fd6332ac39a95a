"""Kernel variants that must not change any bit, through whole solves (direct launches and the graph
replay) in double-float and double: the two-block cluster kernel of level 1 against the one-block
kernel (EPR_TINY_LEVELS=1 / 3), the optional level-2 cluster on 16 blocks against 8
(EPR_CLUSTER_LEVELS=16 / 8: the node sums run in one order whatever the cluster size), and, with
the adaptive indexer, the
per-colour lists of active nodes against whole colours with the inactive nodes skipped
(EPR_ADAPTIVE_LISTS=1 / 0).  The
variant is chosen when the library creates its first context, so each run is its own process.
The cluster kernel of double-float level 2 against the default launch per colour
(EPR_CLUSTER_LEVELS=1 / unset) sums each node's element integrals in another order, so it is
compared within rounding instead."""
import json
import os
import subprocess
import sys

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

SCRIPT = r"""
import json, sys
import numpy as np
sys.path.insert(0, sys.argv[1])
import exteriorpoissonrecon_gb300 as epr
pos, fr = epr.samples.make_workload("link", 30000, seed=4)
pu, _ = epr.unit_cube(pos)
sk = epr.pack_skew(fr)
out = {}
for name, kw in (("df", dict(precision="fp32", fp64_from=0, fp64_levels=4, band_precision="df")),
                 ("fp64", dict()),
                 ("df_adaptive", dict(precision="fp32", fp64_from=0, fp64_levels=4, band_precision="df", aRadius=1)),
                 ("fp64_adaptive", dict(aRadius=1))):
    r = epr.Reconstructor(3, 5, pu, sk, **kw)
    r.solve()
    r.solve()  # the graph replay
    xs, ys = r.solution()
    out[name] = [np.concatenate(xs).tolist(), np.concatenate(ys).tolist()]
    r.close()
print(json.dumps(out))
"""


def _run(env):
    e = dict(os.environ)
    e.update(env)
    r = subprocess.run([sys.executable, "-c", SCRIPT, ROOT], capture_output=True, text=True, env=e, timeout=600)
    assert r.returncode == 0, r.stderr
    return json.loads(r.stdout.strip().splitlines()[-1])


@pytest.mark.parametrize("base_env,env", [({}, {"EPR_TINY_LEVELS": "3"}), ({}, {"EPR_ADAPTIVE_LISTS": "0"}),
                                           ({"EPR_CLUSTER_LEVELS": "16"}, {"EPR_CLUSTER_LEVELS": "8"})])
def test_launch_variants_give_the_same_bits(base_env, env):
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    base = _run(base_env)
    other = _run(env)
    for name in ("df", "fp64", "df_adaptive", "fp64_adaptive"):
        for a, b in zip(base[name], other[name]):
            assert np.array_equal(np.array(a), np.array(b)), (env, name)


def test_cluster_level_agrees_within_rounding():
    """Double-float level 2 on one cluster launch against a launch per colour: the same solve up to
    the order of the element sums (double-float rounding, 2^-48 relative per operation)."""
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    base = _run({"EPR_CLUSTER_LEVELS": "1"})
    other = _run({})
    for name in ("fp64", "fp64_adaptive"):  # no double-float level: the same kernels
        for a, b in zip(base[name], other[name]):
            assert np.array_equal(np.array(a), np.array(b)), name
    for name in ("df", "df_adaptive"):
        for a, b in zip(base[name], other[name]):
            a, b = np.array(a), np.array(b)
            assert np.linalg.norm(a - b) <= 1e-7 * np.linalg.norm(b), name
