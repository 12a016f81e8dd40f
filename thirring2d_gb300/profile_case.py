"""A fixed, small piece of the hot path for profilers (ncu) and quick timing.

    python -m thirring2d_gb300.profile_case --size 1024 --iters 100 --applies 20

On one lattice of the benchmark's couplings (m 0.05, g 0.6, A ~ N(0, 0.3^2),
t antiperiodic, x periodic) it runs `applies` M and `applies` M^dag FP64
operator applies, then one CG solve capped at `iters` iterations (no
tolerance, so it runs exactly that many), in the chosen precision, and prints
the CUDA-event timings.  Numbers printed under a profiler are not benchmark
values.
"""
from __future__ import annotations

import argparse
import json

import numpy as np

from . import native as N
from .lattice import Lattice, cg_params


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--size", type=int, default=1024)
    ap.add_argument("--iters", type=int, default=100)
    ap.add_argument("--applies", type=int, default=20)
    ap.add_argument("--precision", choices=["fp64", "mixed"], default="fp64")
    ap.add_argument("--graph", type=int, default=1)
    a = ap.parse_args()
    n = a.size
    rng = np.random.default_rng(n)
    L = Lattice(n, n, 0.05, 0.6, 0.0, N.BC_ANTIPERIODIC, N.BC_PERIODIC)
    L.set_gauge(rng.normal(0, 0.3, (n, n, 2)))
    out = {"size": n}
    if a.applies:
        out["ms_M"] = L.time_apply(a.applies, False, N.PREC_FP64)
        out["ms_Mdag"] = L.time_apply(a.applies, True, N.PREC_FP64)
        out["ms_M32"] = L.time_apply(a.applies, False, N.PREC_MIXED)
    if a.iters:
        import os
        os.environ["TG_GRAPH"] = "1" if a.graph else "0"
        b = rng.normal(size=(n, n)) + 1j * rng.normal(size=(n, n))
        prec = N.PREC_MIXED if a.precision == "mixed" else N.PREC_FP64
        x, res = L.fmdm_invert_cg(b, cg_params(rel_tol=0.0, abs_tol2=0.0, maxiter=a.iters, precision=prec))
        out["cg_iterations"] = res.iterations
        out["cg_status"] = N.STATUS_NAMES[res.status]
    L.close()
    print(json.dumps(out))


if __name__ == "__main__":
    main()
