"""Whole trajectories through the column-march stencil, against the reference.

The large-lattice workloads (1024^2, 2048^2) run the warp column march
(nx a multiple of 32, nt of 4) and, in the persistent solver, one 512-thread
block per SM.  The fixtures march_* (tests/golden/make_golden.py) are
trajectory sequences of the reference's own hmc.c at such shapes -- its seed,
543210 warm-up draws, pure-gauge start, then update_gauge (hmc.c:671-746) --
at step sizes where the MD is stable (|dH| < 1), so dH is pinned absolutely.

Each run replays them through update_gauge on the reference's MT stream:
  * dH within 1e-9 absolute of the reference's, the same accept/reject
    decisions, and A within 1e-9 after the three trajectories;
  * FP64 with the reference's own CG stop (|r|^2 < 1e-30), and FP32 CG with
    FP64 reliable updates solved to 1e-13 relative (the oracle shows that a
    1e-12 solve already moves dH by up to 1.8e-9 at these volumes);
  * the two-launches-per-iteration solver, the persistent solver at its
    size-chosen shape, and the persistent solver on the launch shape of a
    lattice that fills the GPU (TG_PCG_BLOCK=512: 512-thread blocks, one per SM).
"""
import numpy as np
import pytest

from helpers import MARCH_CONFIGS, golden, lat_args

pytestmark = pytest.mark.gpu

DH_TOL = 1e-9
A_TOL = 1e-9


@pytest.fixture(scope="module")
def tg():
    import thirring2d_gb300 as tg
    tg.native.load()
    return tg


def _cg(tg, precision, solver):
    if precision == "fp64":
        return tg.cg_params(solver=solver)  # hmc.c's stop: |r|^2 < 1e-30
    return tg.cg_params(rel_tol=1e-13, abs_tol2=0, precision=tg.native.PREC_MIXED, ru_interval=50, solver=solver)


SCHEDULES = {
    "launches": dict(solver=1, block=None),
    "persistent": dict(solver=2, block=None),
    "persistent_512x1": dict(solver=2, block="512"),
}


@pytest.mark.parametrize("name", MARCH_CONFIGS)
@pytest.mark.parametrize("precision", ["fp64", "mixed"])
@pytest.mark.parametrize("schedule", list(SCHEDULES))
def test_march_trajectories_match_reference(tg, monkeypatch, name, precision, schedule):
    d = golden(name)
    nt, nx = int(d["nt"]), int(d["nx"])
    assert nx % 32 == 0 and nt % 4 == 0  # the column-march path
    sch = SCHEDULES[schedule]
    if sch["block"] is None:
        monkeypatch.delenv("TG_PCG_BLOCK", raising=False)
    else:
        monkeypatch.setenv("TG_PCG_BLOCK", sch["block"])
    monkeypatch.delenv("TG_MARCH", raising=False)
    hp = tg.hmc_params(nsteps=int(d["traj_nsteps"]), tau=1.0, npf=1, stochastic_term=True, rng=tg.native.RNG_MT,
                       cg=_cg(tg, precision, sch["solver"]))
    L = tg.Lattice(*lat_args(d))
    L.seed_mersenne(int(d["traj_seed"]), 543210)
    L.update_puregauge_hb(int(d["traj_sweeps"]))
    assert np.array_equal(L.get_gauge(), d["traj_A_start"])
    for k, want in enumerate(d["traj_stats"]):
        r = L.update_gauge(hp)
        assert r.status == 0, (k, r.status)
        assert abs(r.dH - want[0]) <= DH_TOL, (k, r.dH, want[0])
        assert r.accepted == int(want[9]), (k, r.accepted, want[9])
        if precision == "mixed":
            assert r.reliable_updates > 0
    assert np.abs(L.get_gauge() - d["traj_A"][-1]).max() <= A_TOL
    L.close()
