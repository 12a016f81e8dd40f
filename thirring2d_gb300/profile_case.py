"""A fixed, small piece of the hot path for profilers (ncu) and quick timing.

    python -m thirring2d_gb300.profile_case --size 1024 --iters 100 --applies 20

On one lattice of the benchmark's couplings (m 0.05, g 0.6, A ~ N(0, 0.3^2),
t antiperiodic, x periodic) it runs `applies` M and `applies` M^dag FP64
operator applies, then one CG solve capped at `iters` iterations (no
tolerance, so it runs exactly that many), in the chosen precision, and prints
the CUDA-event timings.  Numbers printed under a profiler are not benchmark
values.

Report modes:
    --all-kernels                every kernel once, for a per-kernel ncu table
    --batch N [--sequential K]   N chains of mixed sizes in one batched launch
    --mixed-report --size 2048   FP64 vs mixed-precision solve and trajectories at m 0.02
    --scaling-report             dH against the leapfrog step at 64^2, two pseudofermions
"""
from __future__ import annotations

import argparse
import json

import numpy as np

from . import native as N
from .lattice import Lattice, cg_params
from .workloads import mixed_size_chains


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--size", type=int, default=1024, help="lattice side (the mixed-precision report uses 2048)")
    ap.add_argument("--iters", type=int, default=100)
    ap.add_argument("--applies", type=int, default=20)
    ap.add_argument("--precision", choices=["fp64", "mixed"], default="fp64")
    ap.add_argument("--graph", type=int, default=1)
    ap.add_argument("--solver", choices=["default", "launches", "persistent"], default="default",
                    help="CG scheduling: two launches per iteration, or one cooperative launch per solve")
    ap.add_argument("--batch", type=int, default=0, help="run the batched-chain case with this many chains")
    ap.add_argument("--trajectories", type=int, default=2)
    ap.add_argument("--sequential", type=int, default=0, help="chains to also run one at a time (FP64 path)")
    ap.add_argument("--ru-interval", type=int, default=50, help="mixed precision: iterations between reliable updates")
    ap.add_argument("--side", type=int, default=0, help="batched case: give every chain this side")
    ap.add_argument("--instance", type=int, default=0, help="batched case: this kernel instance, no autotuning")
    ap.add_argument("--scaling-report", action="store_true", help="the 64^2 two-pseudofermion dH-scaling report")
    ap.add_argument("--mixed-report", action="store_true", help="the ill-conditioned (m 0.02) mixed-precision report")
    ap.add_argument("--mixed-tau", type=float, nargs="+", default=[1.0, 0.05],
                    help="trajectory lengths of the mixed-precision report")
    ap.add_argument("--all-kernels", action="store_true",
                    help="every kernel of the library once or a few times, for a per-kernel ncu table")
    a = ap.parse_args()
    if a.all_kernels:
        return all_kernels_case(a)
    if a.batch:
        return batch_case(a)
    if a.scaling_report:
        return scaling_report(a)
    if a.mixed_report:
        return mixed_report(a)
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
        solver = {"default": N.SOLVER_DEFAULT, "launches": N.SOLVER_LAUNCHES, "persistent": N.SOLVER_PERSISTENT}
        x, res = L.fmdm_invert_cg(b, cg_params(rel_tol=0.0, abs_tol2=0.0, maxiter=a.iters, precision=prec,
                                               solver=solver[a.solver]))
        out["cg_iterations"] = res.iterations
        out["cg_status"] = N.STATUS_NAMES[res.status]
    L.close()
    print(json.dumps(out))


def all_kernels_case(a):
    """Each kernel of the library at a size where its traffic leaves L2 where
    that is possible: on 2048^2 (m 0.02, g 0.8, A ~ N(0, 0.5^2)) the operator
    in both precisions, a short trajectory in each precision and scheduling
    (CG to 1e-2 relative, 2 leapfrog steps, launched eagerly), the
    measurements and the pure-gauge sweep; the fermion-bag operator, CG and
    propagator, the dense matrix and the log-determinant on small lattices; one
    trajectory of a 16-chain batch."""
    import os

    from .lattice import Batch, batch_params, hmc_params
    os.environ["TG_GRAPH"] = "0"
    out = {}
    n = 2048
    rng = np.random.default_rng(n)
    L = Lattice(n, n, 0.02, 0.8, 0.0, N.BC_ANTIPERIODIC, N.BC_PERIODIC)
    L.set_gauge(rng.normal(0, 0.5, (n, n, 2)))
    out["ms_M64"] = L.time_apply(2, False, N.PREC_FP64)
    out["ms_M32"] = L.time_apply(2, False, N.PREC_MIXED)
    for prec in (N.PREC_FP64, N.PREC_MIXED):
        for solver in (N.SOLVER_LAUNCHES, N.SOLVER_PERSISTENT):
            hp = hmc_params(nsteps=2, tau=0.1, rng=N.RNG_PHILOX, seed=5, use_graph=False,
                            cg=cg_params(rel_tol=1e-2, abs_tol2=0.0, precision=prec, ru_interval=50, solver=solver))
            r = L.update_gauge(hp)
            out[f"traj_p{prec}_s{solver}_its"] = r.cg_iterations
    out["magnetisation"] = L.magnetisation()
    out["pbp"] = L.chiral_condensate(2, seed=1, cp=cg_params(rel_tol=1e-4, abs_tol2=0.0))[0]
    L.update_puregauge_hb(1)
    L.close()
    s = 64
    L = Lattice(s, s, 0.3, 0.5, 0.0, N.BC_ANTIPERIODIC, N.BC_ANTIPERIODIC)
    mask = (rng.random((s, s)) < 0.1).astype(np.int32)
    v = rng.normal(size=(s, s))
    L.fM(mask, v)
    L.fM(mask, v, transpose=True)
    out["cg_MdM_its"] = L.cg_MdM(mask, v)[1].iterations
    L.close()
    L = Lattice(8, 8, 0.3, 0.5, 0.0, N.BC_ANTIPERIODIC, N.BC_ANTIPERIODIC)
    L.fm_propagator()
    L.set_gauge(rng.normal(0, 0.3, (8, 8, 2)))
    L.fermion_matrix()
    out["log_det"] = L.log_det(rng.normal(0, 0.3, (64, 8, 8, 2)))[0][0]
    L.close()
    chains, fields = mixed_size_chains(16)
    B = Batch(chains)
    for i, A in enumerate(fields):
        B.set_gauge(i, A)
    B.trajectory(batch_params(nsteps=2, use_graph=False, block=451241,
                              cg=cg_params(rel_tol=1e-6, abs_tol2=0.0, precision=N.PREC_MIXED)))
    B.close()
    print(json.dumps(out))


def batch_case(a):
    import time

    from .lattice import Batch, batch_params, hmc_params
    chains, fields = mixed_size_chains(a.batch, side=a.side)
    B = Batch(chains)
    for i, A in enumerate(fields):
        B.set_gauge(i, A)
    prec = N.PREC_MIXED if a.precision == "mixed" else N.PREC_FP64
    bp = batch_params(nsteps=10, use_graph=bool(a.graph), block=a.instance,
                      cg=cg_params(rel_tol=1e-10, abs_tol2=0.0, precision=prec, ru_interval=a.ru_interval))
    block, tune_ms = (a.instance, None) if a.instance else B.autotune(bp)
    out = {"chains": a.batch, "sites": B.total_sites(), "precision": a.precision, "block": block,
           "tune_ms": tune_ms, "traj_ms": []}
    for _ in range(a.trajectories):
        res = B.trajectory(bp)
        out["traj_ms"].append(res[0].cg_ms)
        out["status"] = max(r.status for r in res)
        out["acceptance"] = float(np.mean([r.accepted for r in res]))
        out["cg_iterations_mean"] = float(np.mean([r.cg_iterations for r in res]))
        out["cg_iterations_max"] = int(max(r.cg_iterations for r in res))
        out["reliable_updates_mean"] = float(np.mean([r.reliable_updates for r in res]))
        out["dH"] = [r.dH for r in res[:8]]
    B.close()
    if a.sequential:
        cg64 = cg_params(rel_tol=1e-10, abs_tol2=0.0, precision=N.PREC_FP64)
        t0 = time.perf_counter()
        for c, A in list(zip(chains, fields))[: a.sequential]:
            L = Lattice(c["nt"], c["nx"], c["m"], c["g"], c["mu"], c["bc_t"], c["bc_x"])
            L.set_gauge(A)
            L.update_gauge(hmc_params(nsteps=10, rng=N.RNG_PHILOX, seed=c["seed"], cg=cg64))
            L.close()
        out["sequential_fp64_s"] = time.perf_counter() - t0
        out["sequential_chains"] = a.sequential
    print(json.dumps(out))


def scaling_report(a):
    """64^2, m 0.1, g 0.5, A ~ N(0, 0.3^2), two pseudofermions: dH statistics over
    a.trajectories trajectories at leapfrog step sizes 0.2, 0.1, 0.05 (and 0.025,
    0.0125 over fewer), FP64 and mixed precision on the same Philox stream."""
    from .lattice import hmc_params
    n = 64
    A0 = np.random.default_rng(64).normal(0, 0.3, (n, n, 2))
    out = {"lattice": f"{n}x{n}", "m": 0.1, "g": 0.5, "npf": 2, "rows": []}
    for nsteps, ntraj in ((5, a.trajectories), (10, a.trajectories), (20, a.trajectories),
                          (40, max(1, a.trajectories // 5)), (80, max(1, a.trajectories // 5))):
        row = {"eps": 1.0 / nsteps, "trajectories": ntraj}
        dhs = {}
        for prec, name in ((N.PREC_FP64, "fp64"), (N.PREC_MIXED, "mixed")):
            L = Lattice(n, n, 0.1, 0.5, 0.0, N.BC_ANTIPERIODIC, N.BC_PERIODIC)
            L.set_gauge(A0)
            hp = hmc_params(nsteps=nsteps, tau=1.0, npf=2, stochastic_term=False, rng=N.RNG_PHILOX, seed=55,
                            cg=cg_params(rel_tol=1e-12, abs_tol2=0.0, precision=prec, ru_interval=50))
            res = [L.update_gauge(hp) for _ in range(ntraj)]
            L.close()
            dh = np.array([r.dH for r in res])
            dhs[name] = (dh, [r.accepted for r in res])
            row[name] = {"mean_dH": float(dh.mean()), "mean_abs_dH": float(np.abs(dh).mean()),
                         "rms_dH": float(np.sqrt((dh ** 2).mean())), "median_abs_dH": float(np.median(np.abs(dh))),
                         "acceptance": float(np.mean([r.accepted for r in res])),
                         "mean_exp_minus_dH": float(np.mean(np.exp(-np.clip(dh, -50, 50)))),
                         "status": max(r.status for r in res)}
        d64, dmx = dhs["fp64"][0], dhs["mixed"][0]
        row["max_abs_dH_diff_mixed_vs_fp64"] = float(np.abs(d64 - dmx).max())
        row["max_rel_dH_diff_mixed_vs_fp64"] = float((np.abs(d64 - dmx) / np.maximum(1.0, np.abs(d64))).max())
        row["accept_mismatch"] = int(sum(x != y for x, y in zip(dhs["fp64"][1], dhs["mixed"][1])))
        out["rows"].append(row)
        print(json.dumps(row), flush=True)
    print(json.dumps(out))


def mixed_report(a):
    """2048^2 (a.size), m 0.02, g 0.8, A ~ N(0, 0.5^2): one CG solve of M^dag M x = b
    to relative residual 1e-10 in FP64 and in FP32 with FP64 reliable updates
    every 50 iterations (iterations, wall time, true residual, distance between
    the two solutions), then a.trajectories trajectories of 30 leapfrog steps in
    each precision on the same Philox stream (dH per trajectory and their
    difference)."""
    import time

    from .lattice import hmc_params
    n, m, g = a.size, 0.02, 0.8
    rng = np.random.default_rng(2048)
    A0 = rng.normal(0, 0.5, (n, n, 2))
    b = rng.normal(size=(n, n)) + 1j * rng.normal(size=(n, n))
    out = {"lattice": f"{n}x{n}", "m": m, "g": g, "solve": {}, "trajectories": []}
    L = Lattice(n, n, m, g, 0.0, N.BC_ANTIPERIODIC, N.BC_PERIODIC)
    L.set_gauge(A0)
    xs = {}
    for prec, name in ((N.PREC_FP64, "fp64"), (N.PREC_MIXED, "mixed")):
        cp = cg_params(rel_tol=1e-10, abs_tol2=0.0, maxiter=200000, precision=prec, ru_interval=50)
        L.fmdm_invert_cg(b, cp)  # warm-up (graph instantiation)
        t0 = time.perf_counter()
        x, res = L.fmdm_invert_cg(b, cp)
        ms = 1e3 * (time.perf_counter() - t0)
        true_res = float(np.linalg.norm(b - L.fm_conjugate_mul(L.fm_mul(x))) / np.linalg.norm(b))
        xs[name] = x
        out["solve"][name] = {"iterations": res.iterations, "reliable_updates": res.reliable_updates,
                              "status": N.STATUS_NAMES[res.status], "ms": ms, "true_rel_residual": true_res}
    out["solve"]["rel_diff_mixed_vs_fp64"] = float(np.linalg.norm(xs["mixed"] - xs["fp64"]) / np.linalg.norm(xs["fp64"]))
    print(json.dumps(out["solve"]), flush=True)
    L.close()
    # tau 1 is the configuration as specified (30 steps of 1/30: the MD is
    # unstable there, |dH| ~ 1e12); tau 0.05 (30 steps of 1/600) is a step
    # size at which it is stable, so the dH difference measures the solver
    for tau in a.mixed_tau:
        runs = {}
        for prec, name in ((N.PREC_FP64, "fp64"), (N.PREC_MIXED, "mixed")):
            L = Lattice(n, n, m, g, 0.0, N.BC_ANTIPERIODIC, N.BC_PERIODIC)
            L.set_gauge(A0)
            hp = hmc_params(nsteps=30, tau=tau, rng=N.RNG_PHILOX, seed=3,
                            cg=cg_params(rel_tol=1e-10, abs_tol2=0.0, maxiter=200000, precision=prec, ru_interval=50))
            rs = []
            for _ in range(a.trajectories):
                t0 = time.perf_counter()
                r = L.update_gauge(hp)
                rs.append((r.dH, r.accepted, r.status, r.cg_iterations, r.cg_solves, time.perf_counter() - t0))
            runs[name] = rs
            L.close()
        for k in range(a.trajectories):
            f, x = runs["fp64"][k], runs["mixed"][k]
            row = {"tau": tau, "traj": k, "dH_fp64": f[0], "dH_mixed": x[0], "abs_diff": abs(f[0] - x[0]),
                   "rel_diff": abs(f[0] - x[0]) / max(1.0, abs(f[0])), "accepted": [f[1], x[1]],
                   "status": [N.STATUS_NAMES[f[2]], N.STATUS_NAMES[x[2]]], "cg_iterations": [f[3], x[3]],
                   "cg_solves": [f[4], x[4]], "s": [f[5], x[5]]}
            out["trajectories"].append(row)
            print(json.dumps(row), flush=True)
    print(json.dumps(out))


if __name__ == "__main__":
    main()
