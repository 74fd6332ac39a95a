"""Launches one kernel family of the solve path a few times on a built problem, for profilers.

    python -m exteriorpoissonrecon_gb300.profile_kernels --dim 3 --depth 7 --kernel gs --reps 3
    python -m exteriorpoissonrecon_gb300.profile_kernels --depth 8 --level 3 --band df --kernel gs

Builds the named synthetic workload on the GPU, sets seeded random coefficients on the finest
level and times `reps` launches of the kernel (plus one warm-up launch) with CUDA events through
epr_time_kernel.  Kernel families: gs, energy, quadfit, prolong, gn, and the multigrid families
lgs, residual, assemble, biquad.
"""
from __future__ import annotations

import argparse
import json

import numpy as np

import exteriorpoissonrecon_gb300 as epr


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--dim", type=int, default=3)
    ap.add_argument("--depth", type=int, default=7)
    ap.add_argument("--samples", type=int, default=200_000)
    ap.add_argument("--workload", default=None)
    ap.add_argument("--kernel", default="gs")
    ap.add_argument("--reps", type=int, default=3)
    ap.add_argument("--precision", default="fp32")
    ap.add_argument("--level", type=int, default=None)
    ap.add_argument("--band", default=None, help="with --precision fp32: df or fp64 arithmetic for levels 2-3")
    a = ap.parse_args()
    wl = a.workload or ("link" if a.dim == 3 else "clifford")
    pos, frames = epr.samples.make_workload(wl, a.samples, seed=0)
    pu, _ = epr.unit_cube(pos)
    band = dict(fp64_from=2, fp64_levels=4, band_precision=a.band) if a.band else {}
    r = epr.Reconstructor(a.dim, a.depth, pu, epr.pack_skew(frames), precision=a.precision, **band)
    level = a.depth if a.level is None else a.level
    n = r.nodes(level)
    rng = np.random.default_rng(0)
    r.set_coefficients(level, rng.uniform(-0.1, 0.1, n), rng.uniform(-0.1, 0.1, n))
    ms = r.time_kernel(a.kernel, level, a.reps)
    print(json.dumps({"kernel": a.kernel, "dim": a.dim, "depth": a.depth, "level": level, "nodes": n,
                      "precision": a.precision, "ms_per_launch": ms}))


if __name__ == "__main__":
    main()
