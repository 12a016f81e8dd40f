"""Observables of a GPU HMC chain against an oracle chain (hmc.c's algorithm,
bitwise-pinned to the reference) on independent random streams: acceptance,
auxiliary-field action per site and chiral condensate Re tr M^-1 / V must agree
within their binned statistical errors.  Also checks <exp(-dH)> = 1 on the GPU
chain.  8x8, m 0.3, g 0.5, t antiperiodic, x periodic, 20 leapfrog steps."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

N_SIDE, MASS, G, NSTEPS = 8, 0.3, 0.5, 20
NTRAJ, BURN, BIN = 400, 50, 25
Z_MAX = 5.0   # 14 bins per chain: a loose bound on the estimated error


def binned(x):
    x = np.asarray(x[BURN:], dtype=float)
    nb = len(x) // BIN
    bm = x[: nb * BIN].reshape(nb, BIN).mean(1)
    return float(x.mean()), float(bm.std(ddof=1) / np.sqrt(nb))


def condensate(Md):
    return float(np.trace(np.linalg.inv(Md)).real) / Md.shape[0]


@pytest.fixture(scope="module")
def chains(oracle_lib):
    import thirring2d_gb300 as tg
    V = N_SIDE * N_SIDE
    # oracle chain: reference MT stream, seed 7 with the reference's warm-up
    o = oracle_lib.Oracle(N_SIDE, N_SIDE, MASS, G, 0.0, -1, 1)
    mt = oracle_lib.MT(7, 543210)
    A = np.zeros((N_SIDE, N_SIDE, 2))
    ref = {"acc": [], "sg": [], "pbp": []}
    for _ in range(NTRAJ):
        s, st, _ = o.trajectory(A, mt, NSTEPS, 1.0, 1, True)
        assert st == 0
        ref["acc"].append(s[9])
        ref["sg"].append(o.gauge_action(A) / V)
        ref["pbp"].append(condensate(o.dense_M(A)))
    # GPU chain: Philox stream, seed 11
    L = tg.Lattice(N_SIDE, N_SIDE, MASS, G, 0.0, tg.native.BC_ANTIPERIODIC, tg.native.BC_PERIODIC)
    L.set_gauge(np.zeros((N_SIDE, N_SIDE, 2)))
    hp = tg.hmc_params(nsteps=NSTEPS, rng=tg.native.RNG_PHILOX, seed=11)
    gpu = {"acc": [], "sg": [], "pbp": [], "edh": []}
    for _ in range(NTRAJ):
        r = L.update_gauge(hp)
        assert r.status == 0
        gpu["acc"].append(r.accepted)
        gpu["edh"].append(np.exp(-r.dH))
        gpu["sg"].append(L.calc_gauge_action() / V)
        gpu["pbp"].append(condensate(L.fermion_matrix()))
    L.close()
    return ref, gpu


@pytest.mark.parametrize("obs", ["acc", "sg", "pbp"])
def test_observable_consistent_with_oracle_chain(chains, obs):
    ref, gpu = chains
    (ma, ea), (mb, eb) = binned(ref[obs]), binned(gpu[obs])
    z = abs(ma - mb) / np.hypot(ea, eb)
    assert z < Z_MAX, (obs, ma, ea, mb, eb, z)


def test_exp_minus_dH_is_one(chains):
    _, gpu = chains
    m, e = binned(gpu["edh"])
    assert abs(m - 1.0) < Z_MAX * e + 1e-3, (m, e)
