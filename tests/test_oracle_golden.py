"""Pins the CPU oracle (oracle/thirring_oracle.c) to the reference's own
outputs (tests/golden/, generated from hmc.c by tests/golden/make_golden.py).
No GPU needed."""
import numpy as np
import pytest

from helpers import STABLE, TRAJ_CONFIGS, dH_ok, golden, lat_args, maxrel, rel

CFGS = TRAJ_CONFIGS


def test_mt_stream(oracle_lib):
    d = golden("mt_stream")
    for s in (12345, 4354365264, -7):
        mt = oracle_lib.MT(s, 543210)
        assert np.array_equal(mt.uniforms(3000), d[f"seed_{s}"])
    mt = oracle_lib.MT(12345, 0)
    assert np.array_equal(mt.uniforms(1300), d["seed_12345_nowarmup"])


@pytest.mark.parametrize("name", CFGS)
def test_operator(oracle_lib, name):
    d = golden(name)
    o = oracle_lib.Oracle(*lat_args(d))
    assert rel(o.M(d["A"], d["psi"]), d["M_psi"]) < 1e-14
    assert rel(o.Mdag(d["A"], d["psi"]), d["Mdag_psi"]) < 1e-14


@pytest.mark.parametrize("name", CFGS)
def test_cg_and_actions(oracle_lib, name):
    d = golden(name)
    o = oracle_lib.Oracle(*lat_args(d))
    x, st, it = o.cg(d["A"], d["psi"])
    assert st == 0
    assert rel(x, d["cg_x"]) < 1e-12
    assert abs(o.gauge_action(d["A"]) - d["S_gauge"]) <= 1e-12 * abs(d["S_gauge"])
    assert abs(o.md_action(d["A"], d["noise"]) - d["S_md"]) <= 1e-12 * abs(d["S_md"])
    S_pf = float(np.vdot(d["psi"], x).real)
    assert abs(S_pf - d["S_pf"]) <= 1e-12 * abs(d["S_pf"])


@pytest.mark.parametrize("name", CFGS)
def test_momentum_step(oracle_lib, name):
    d = golden(name)
    o = oracle_lib.Oracle(*lat_args(d))
    p, st, it = o.momentum_step(d["A"], d["mom0"], d["psi"], d["noise"], 0.1)
    assert st == 0
    assert maxrel(p - d["mom0"], d["mom_step"] - d["mom0"]) < 1e-11


@pytest.mark.parametrize("name", CFGS)
def test_trajectories(oracle_lib, name):
    d = golden(name)
    nt, nx = int(d["nt"]), int(d["nx"])
    o = oracle_lib.Oracle(*lat_args(d))
    mt = oracle_lib.MT(int(d["traj_seed"]), 543210)
    A = np.zeros((nt, nx, 2))
    for _ in range(int(d["traj_sweeps"])):
        o.puregauge_sweep(A, mt)
    assert np.array_equal(A, d["traj_A_start"])
    for k, want in enumerate(d["traj_stats"]):
        s, st, it = o.trajectory(A, mt, int(d["traj_nsteps"]), 1.0, 1, True)
        assert st == 0
        assert dH_ok(s[0], want[0], name in STABLE), (k, s[0], want[0])
        assert s[9] == want[9]
        assert np.abs(A - d["traj_A"][k]).max() < 1e-9


@pytest.mark.parametrize("name", ["det_4x4_apx", "det_4x4_px", "det_6x4_apx"])
def test_dense_matrix(oracle_lib, name):
    d = golden(name)
    o = oracle_lib.Oracle(int(d["nt"]), int(d["nx"]), float(d["m"]), 0.5, float(d["mu"]), -1, int(d["bc_x"]))
    Md = o.dense_M(d["A"])
    assert np.abs(Md - d["M"]).max() < 1e-15
    sign, logdet = np.linalg.slogdet(Md)
    assert abs(logdet - d["logabsdet"]) < 1e-12
    assert abs(sign - d["phase"]) < 1e-12


def test_adjoint_identity(oracle_lib):
    rng = np.random.default_rng(5)
    for (nt, nx, bcx, mu) in [(8, 6, 1, 0.0), (6, 10, -1, 0.4), (4, 4, 0, 0.2)]:
        o = oracle_lib.Oracle(nt, nx, 0.3, 0.5, mu, -1, bcx)
        A = rng.normal(0, 0.7, (nt, nx, 2))
        u = rng.normal(size=(nt, nx)) + 1j * rng.normal(size=(nt, nx))
        v = rng.normal(size=(nt, nx)) + 1j * rng.normal(size=(nt, nx))
        assert abs(np.vdot(u, o.M(A, v)) - np.vdot(o.Mdag(A, u), v)) < 1e-12
        Md = o.dense_M(A)
        assert np.abs(Md.conj().T @ u.ravel() - o.Mdag(A, u).ravel()).max() < 1e-13


def test_force_finite_difference(oracle_lib):
    """dS/dA of the oracle against central differences of S_g + S_pf + S_md."""
    rng = np.random.default_rng(11)
    nt, nx = 6, 8
    o = oracle_lib.Oracle(nt, nx, 0.4, 0.7, 0.25, -1, 1)
    A = rng.normal(0, 0.5, (nt, nx, 2))
    phi = rng.normal(size=(nt, nx)) + 1j * rng.normal(size=(nt, nx))
    noise = rng.normal(size=(nt, nx)) + 1j * rng.normal(size=(nt, nx))

    def S(A):
        x, st, _ = o.cg(A, phi, rel_tol=1e-14, abs_tol2=0)
        return o.gauge_action(A) + float(np.vdot(phi, x).real) + o.md_action(A, noise)

    x, _, _ = o.cg(A, phi, rel_tol=1e-14, abs_tol2=0)
    F = o.force(A, x, noise)
    h = 1e-6
    for k in range(24):
        t, xx, dr = rng.integers(nt), rng.integers(nx), rng.integers(2)
        Ap, Am = A.copy(), A.copy()
        Ap[t, xx, dr] += h
        Am[t, xx, dr] -= h
        fd = (S(Ap) - S(Am)) / (2 * h)
        assert abs(fd - F[t, xx, dr]) < 1e-6 * max(1.0, abs(fd))


@pytest.mark.parametrize("name", ["vecops_8x8", "vecops_6x4", "vecops_16x16"])
def test_masked_operator_oracle(oracle_lib, name):
    """The fermion-bag operator of vec_ops.c:96-174 and its CG (261-307)."""
    d = golden(name)
    o = oracle_lib.Oracle(int(d["nt"]), int(d["nx"]), float(d["m"]), 0.5, float(d["mu"]), -1, -1)
    assert np.abs(o.fM(d["mask"], d["v"]) - d["fM_v"]).max() < 1e-14
    assert np.abs(o.fM(d["mask"], d["v"], True) - d["fMt_v"]).max() < 1e-14
    x, st, it = o.cg_MdM(d["mask"], d["b"], maxiter=10000)
    assert st == 0 and rel(x, d["cg_x"]) < 1e-12


@pytest.mark.parametrize("name", ["free_det_8x8", "free_det_6x4"])
def test_free_matrix_equals_fermion_bag_matrix(oracle_lib, name):
    """At A = 0 hmc.c's M (antiperiodic t and x) is the fermion-bag matrix of
    vec_ops.c / fermion_matrix.c:28-64 with no monomers; the fixture holds the
    latter, built from the reference's own fM."""
    d = golden(name)
    nt, nx = int(d["nt"]), int(d["nx"])
    o = oracle_lib.Oracle(nt, nx, float(d["m"]), 0.5, float(d["mu"]), -1, -1)
    Md = o.dense_M(np.zeros((nt, nx, 2)))
    assert np.abs(Md - d["M"]).max() < 1e-15
    sign, logabs = np.linalg.slogdet(Md)
    assert abs(logabs - float(d["logabsdet"])) < 1e-12 and abs(sign - float(d["sign"])) < 1e-12


@pytest.mark.parametrize("name", ["prop_8x8", "prop_6x4_mask"])
def test_propagator_oracle(oracle_lib, name):
    """calc_Dinv (fermion_matrix.c:189-351): the oracle's restatement against the
    reference's propagator matrix."""
    d = golden(name)
    o = oracle_lib.Oracle(int(d["nt"]), int(d["nx"]), float(d["m"]), 0.5, float(d["mu"]), -1, -1)
    D = o.fm_propagator(d["mask"])
    assert np.abs(D - d["Dinv"]).max() < 1e-12 * np.abs(d["Dinv"]).max()
