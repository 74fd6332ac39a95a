"""Host-side logic that needs no GPU: the batched workload mix, the sampler parameter defaults and
the benchmark's schedule arithmetic."""
import math
import os
import sys

import numpy as np

import exteriorpoissonrecon_gb300 as epr

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_batch_workload_mix():
    w = epr.samples.batch_workloads(16, seed=2, n_range=(2048, 8192))
    assert len(w) == 16
    for k, item in enumerate(w):
        assert item["depth"] in (5, 6, 7)
        assert 2048 <= item["n"] <= 8192
        assert 0.0 <= item["sigma"] <= 0.01 and 0.0 <= item["angle_deg"] <= 10.0
        assert item["pos"].shape == (item["n"], 3) and item["frames"].shape == (item["n"], 3, 3)
        if k < 8:
            p, q = (int(v) for v in item["name"].split("_")[1:])
            assert 2 <= p <= 7 and 2 <= q <= 7 and math.gcd(p, q) == 1
        else:
            assert item["name"].startswith("helix_") and 1.0 <= float(item["name"].split("_")[1]) <= 8.0
    again = epr.samples.batch_workloads(16, seed=2, n_range=(2048, 8192))
    assert all(np.array_equal(a["pos"], b["pos"]) for a, b in zip(w, again))


def test_sampler_defaults():
    k = epr.sampler("knot")
    assert (k.shape, k.a, k.b) == (0, 2.0, 3.0)
    h = epr.sampler("helix", 4.0)
    assert (h.shape, h.a, h.b, h.c) == (2, 4.0, 0.3, 1.0)
    assert epr.sampler("clifford", seed=5).seed == 5


def test_schedule_node_updates():
    sys.path.insert(0, ROOT)
    import bench
    # sum over levels of ceil(2^(8-l) 10) sweeps of (2^l + 1)^3 nodes
    assert bench.schedule_node_updates(3, 8) == 227694070
    assert bench.schedule_node_updates(3, 5) == sum(math.ceil(2 ** (5 - l) * 10) * (2 ** l + 1) ** 3 for l in range(6))
