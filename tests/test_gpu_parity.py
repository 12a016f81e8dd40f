"""Parity of the CUDA library (through its C ABI) with the reference's outputs
(tests/golden/) and with the CPU oracle.  Tolerances are the ones the
reference's hot path is held to: M v within 1e-13 relative, CG solutions
within the stated residual, forces within 1e-11 (max-abs relative), dH
within 1e-9."""
import os

import numpy as np
import pytest

from helpers import STABLE, TRAJ_CONFIGS, dH_ok, golden, lat_args, maxrel, rel

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def tg():
    import thirring2d_gb300 as tg
    tg.native.load()
    return tg


def make(tg, d):
    nt, nx, m, g, mu, bct, bcx = lat_args(d)
    L = tg.Lattice(nt, nx, m, g, mu, bct, bcx)
    return L


def cplx(rng, shape):
    return rng.normal(size=shape) + 1j * rng.normal(size=shape)


# --------------------------------------------------------------------------
# operator
# --------------------------------------------------------------------------
@pytest.mark.parametrize("name", TRAJ_CONFIGS)
def test_operator_golden(tg, name):
    d = golden(name)
    L = make(tg, d)
    L.set_gauge(d["A"])
    assert rel(L.fm_mul(d["psi"]), d["M_psi"]) < 1e-13
    assert rel(L.fm_conjugate_mul(d["psi"]), d["Mdag_psi"]) < 1e-13


@pytest.mark.parametrize("nt,nx,bcx,mu", [(1024, 1024, 1, 0.0), (2048, 2048, 1, 0.0), (48, 24, -1, 0.3),
                                          (2, 2, 1, 0.0), (3, 5, 0, 0.1), (96, 16, -1, 0.0)])
def test_operator_oracle_sizes(tg, oracle_lib, nt, nx, bcx, mu):
    """M and M^dag vs the oracle from 2x2 to the 2048^2 workload."""
    rng = np.random.default_rng(nt * 7 + nx)
    A = rng.normal(0, 0.5, (nt, nx, 2))
    psi = cplx(rng, (nt, nx))
    o = oracle_lib.Oracle(nt, nx, 0.05, 0.6, mu, -1, bcx)
    L = tg.Lattice(nt, nx, 0.05, 0.6, mu, -1, bcx)
    L.set_gauge(A)
    assert rel(L.fm_mul(psi), o.M(A, psi)) < 1e-13
    assert rel(L.fm_conjugate_mul(psi), o.Mdag(A, psi)) < 1e-13


def test_adjoint_identity(tg):
    rng = np.random.default_rng(2)
    L = tg.Lattice(32, 48, 0.2, 0.5, 0.35, -1, 1)
    L.set_gauge(rng.normal(0, 1.0, (32, 48, 2)))
    u, v = cplx(rng, (32, 48)), cplx(rng, (32, 48))
    lhs = np.vdot(u, L.fm_mul(v))
    rhs = np.vdot(L.fm_conjugate_mul(u), v)
    assert abs(lhs - rhs) < 1e-12 * abs(lhs)


def test_fp32_operator(tg):
    """The FP32 operator of the mixed-precision solver agrees with FP64 to FP32 rounding."""
    torch = pytest.importorskip("torch")
    rng = np.random.default_rng(3)
    nt, nx = 64, 96
    A = rng.normal(0, 0.5, (nt, nx, 2))
    psi = cplx(rng, (nt, nx))
    L = tg.Lattice(nt, nx, 0.1, 0.5, 0.2, -1, 1)
    L.set_gauge(A)
    ref = L.fm_mul(psi)
    x = torch.from_numpy(np.stack([psi.real, psi.imag], -1).astype(np.float32)).cuda()
    y = torch.empty_like(x)
    torch.cuda.synchronize()
    L.apply_dev(x.data_ptr(), y.data_ptr(), False, tg.native.PREC_MIXED)
    L.synchronize()
    got = y.cpu().numpy().astype(np.float64)
    assert rel(got[..., 0] + 1j * got[..., 1], ref) < 3e-7


# --------------------------------------------------------------------------
# CG
# --------------------------------------------------------------------------
@pytest.mark.parametrize("name", TRAJ_CONFIGS)
def test_cg_golden(tg, name):
    d = golden(name)
    L = make(tg, d)
    L.set_gauge(d["A"])
    x, res = L.fmdm_invert_cg(d["psi"], tg.cg_params())  # hmc.c's stop |r|^2 < 1e-30
    assert res.status == 0
    assert rel(x, d["cg_x"]) < 1e-12
    S, _ = L.pseudofermion_action(d["psi"])
    assert abs(S - d["S_pf"]) <= 1e-12 * abs(d["S_pf"])
    assert abs(L.calc_gauge_action() - d["S_gauge"]) <= 1e-12 * abs(d["S_gauge"])
    assert abs(L.stochastic_md_action(d["noise"]) - d["S_md"]) <= 1e-12 * abs(d["S_md"])


def test_cg_iterations_match_oracle(tg, oracle_lib):
    d = golden("c1_16x16_px")
    L = make(tg, d)
    L.set_gauge(d["A"])
    o = oracle_lib.Oracle(*lat_args(d))
    for tol in (1e-6, 1e-10, 1e-12):
        x, res = L.fmdm_invert_cg(d["psi"], tg.cg_params(rel_tol=tol, abs_tol2=0))
        xo, st, it = o.cg(d["A"], d["psi"], rel_tol=tol, abs_tol2=0)
        assert abs(res.iterations - it) <= 2
        assert rel(x, xo) < 50 * tol


@pytest.mark.parametrize("m,mu", [(0.0, 0.0), (0.3, 0.0), (0.3, 0.25)])
def test_cg_mass_forms(tg, oracle_lib, m, mu):
    """For m != 0 the FP64 CG iterates on (M/m)^dag (M/m) with links W/m
    (same residuals and stopping test as hmc.c:341-404); m = 0 keeps the plain
    form.  Both against the oracle's CG; the lattice is created at another mass
    so the W/m links must follow tg_set_couplings."""
    rng = np.random.default_rng(21)
    nt, nx = 16, 32   # column-march stencil path
    A = rng.normal(0, 0.5, (nt, nx, 2))
    b = cplx(rng, (nt, nx))
    L = tg.Lattice(nt, nx, 0.7, 0.5, 0.0, -1, 1)
    L.set_gauge(A)
    L.set_couplings(m, 0.5, mu)
    o = oracle_lib.Oracle(nt, nx, m, 0.5, mu, -1, 1)
    x, res = L.fmdm_invert_cg(b, tg.cg_params(rel_tol=1e-12, abs_tol2=0))
    xo, st, it = o.cg(A, b, rel_tol=1e-12, abs_tol2=0)
    assert res.status == 0 and st == 0
    assert abs(res.iterations - it) <= 2
    assert rel(x, xo) < 1e-10
    assert rel(L.fm_mul(b), o.M(A, b)) < 1e-13


@pytest.mark.parametrize("precision", [0, 1])
def test_cg_true_residual_1024(tg, oracle_lib, precision):
    """The 1024^2 workload (m=0.05, g=0.6, A ~ N(0, 0.3^2)): CG to 1e-10 relative,
    checked on the true residual |b - M^dag M x| / |b| computed by the oracle."""
    nt = nx = 1024
    rng = np.random.default_rng(1024)
    A = rng.normal(0, 0.3, (nt, nx, 2))
    b = cplx(rng, (nt, nx))
    L = tg.Lattice(nt, nx, 0.05, 0.6, 0.0, -1, 1)
    L.set_gauge(A)
    x, res = L.fmdm_invert_cg(b, tg.cg_params(rel_tol=1e-10, abs_tol2=0, precision=precision, ru_interval=50))
    assert res.status == 0
    o = oracle_lib.Oracle(nt, nx, 0.05, 0.6, 0.0, -1, 1)
    r = b - o.Mdag(A, o.M(A, x))
    assert np.linalg.norm(r) / np.linalg.norm(b) < 1.5e-10
    if precision == 1:
        assert res.reliable_updates >= 1


def test_cg_graph_equals_eager(tg, monkeypatch):
    """The CUDA-graph solve (conditional WHILE node) and the eagerly launched
    solve run the same kernels with deterministic reductions: bitwise equal."""
    d = golden("mu_8x8_px")
    out = []
    for flag in ("1", "0"):
        monkeypatch.setenv("TG_GRAPH", flag)
        L = make(tg, d)
        L.set_gauge(d["A"])
        for prec in (0, 1):
            x, res = L.fmdm_invert_cg(d["psi"], tg.cg_params(rel_tol=1e-11, abs_tol2=0, precision=prec,
                                                             ru_interval=20))
            out.append((x, res.iterations))
    for k in range(2):
        assert np.array_equal(out[k][0], out[k + 2][0])
        assert out[k][1] == out[k + 2][1]


def test_cg_edge_cases(tg):
    rng = np.random.default_rng(9)
    L = tg.Lattice(8, 8, 0.3, 0.5, 0.0, -1, 1)
    L.set_gauge(rng.normal(0, 0.5, (8, 8, 2)))
    x, res = L.fmdm_invert_cg(np.zeros((8, 8), complex))       # b = 0: hmc.c:359-361 returns x = 0
    assert res.status == 0 and res.iterations == 0 and not x.any()
    x, res = L.fmdm_invert_cg(cplx(rng, (8, 8)), tg.cg_params(maxiter=3))
    assert res.status == tg.native.TG_E_NOCONV and res.iterations == 3
    bad = cplx(rng, (8, 8))
    bad[2, 3] = np.nan
    x, res = L.fmdm_invert_cg(bad)
    assert res.status == tg.native.TG_E_NAN
    with pytest.raises(tg.native.TGError):
        L.fmdm_invert_cg(bad, tg.cg_params(maxiter=0))


@pytest.mark.parametrize("precision", [0, 1])
def test_cg_singular_operator_is_reported(tg, precision):
    """m = 0 with t and x periodic and A = 0: the free staggered operator has
    exact zero modes, so M^dag M x = b has no solution for a generic b.  The
    solve must end with a failure status (hmc.c:383-386 stops with "Cannot
    invert fermion matrix"; NaN and the iteration cap are reported too), and
    the lattice stays usable."""
    rng = np.random.default_rng(2)
    L = tg.Lattice(8, 8, 0.0, 0.5, 0.0, 1, 1)
    b = cplx(rng, (8, 8))
    x, res = L.fmdm_invert_cg(b, tg.cg_params(rel_tol=1e-12, abs_tol2=0, maxiter=5000, precision=precision))
    assert res.status in (tg.native.TG_E_DIVERGED, tg.native.TG_E_NAN, tg.native.TG_E_NOCONV)
    L.set_couplings(0.3, 0.5, 0.0)
    x, res = L.fmdm_invert_cg(b, tg.cg_params(rel_tol=1e-10, abs_tol2=0, precision=precision))
    assert res.status == 0


def test_cg_mixed_vs_fp64(tg):
    d = golden("c1_16x16_px")
    L = make(tg, d)
    L.set_gauge(d["A"])
    x64, r64 = L.fmdm_invert_cg(d["psi"], tg.cg_params(rel_tol=1e-12, abs_tol2=0))
    xmx, rmx = L.fmdm_invert_cg(d["psi"], tg.cg_params(rel_tol=1e-12, abs_tol2=0, precision=1, ru_interval=50))
    assert rmx.status == 0 and rmx.reliable_updates >= 2
    assert rel(xmx, x64) < 1e-9
    assert rmx.rr <= 1e-24 * rmx.rr0


# --------------------------------------------------------------------------
# forces and the leapfrog pieces
# --------------------------------------------------------------------------
@pytest.mark.parametrize("name", TRAJ_CONFIGS)
def test_force_vs_oracle(tg, oracle_lib, name):
    d = golden(name)
    o = oracle_lib.Oracle(*lat_args(d))
    x, st, _ = o.cg(d["A"], d["psi"])
    F_o = o.force(d["A"], x, d["noise"])
    L = make(tg, d)
    L.set_gauge(d["A"])
    F = L.force(x, d["noise"])
    assert maxrel(F, F_o) < 1e-11


@pytest.mark.parametrize("name", TRAJ_CONFIGS)
def test_momentum_step_golden(tg, name):
    d = golden(name)
    L = make(tg, d)
    L.set_gauge(d["A"])
    p, res = L.momentum_step(d["mom0"], d["psi"], d["noise"], 0.1)
    assert res.status == 0
    assert maxrel(p - d["mom0"], d["mom_step"] - d["mom0"]) < 1e-11


def test_gauge_step(tg):
    rng = np.random.default_rng(4)
    A = rng.normal(0, 1, (6, 10, 2))
    p = rng.normal(0, 1, (6, 10, 2))
    L = tg.Lattice(6, 10, 0.2)
    L.set_gauge(A)
    L.gauge_step(p, 0.05)
    assert np.array_equal(L.get_gauge(), A + 2.0 * 0.05 * p)


# --------------------------------------------------------------------------
# trajectories on the reference's random stream
# --------------------------------------------------------------------------
def _replay(tg, d, hp):
    L = make(tg, d)
    L.seed_mersenne(int(d["traj_seed"]), 543210)
    L.update_puregauge_hb(int(d["traj_sweeps"]))
    assert np.array_equal(L.get_gauge(), d["traj_A_start"])
    return L, [L.update_gauge(hp) for _ in range(len(d["traj_stats"]))]


@pytest.mark.parametrize("name", TRAJ_CONFIGS)
def test_trajectories_golden(tg, name):
    d = golden(name)
    hp = tg.hmc_params(nsteps=int(d["traj_nsteps"]), tau=1.0, npf=1, stochastic_term=True,
                       rng=tg.native.RNG_MT, cg=tg.cg_params())
    L, res = _replay(tg, d, hp)
    for k, (r, want) in enumerate(zip(res, d["traj_stats"])):
        assert r.status == 0
        assert dH_ok(r.dH, want[0], name in STABLE), (k, r.dH, want[0])
        assert r.accepted == int(want[9])
        assert abs(r.Spf0 - want[2]) <= 1e-12 * abs(want[2])
    assert np.abs(L.get_gauge() - d["traj_A"][-1]).max() < 1e-9


def test_trajectory_graph_equals_eager(tg):
    d = golden("c1s_16x16_px")
    runs = []
    for use_graph in (True, False):
        hp = tg.hmc_params(nsteps=40, rng=tg.native.RNG_MT, use_graph=use_graph)
        _, res = _replay(tg, d, hp)
        runs.append([r.dH for r in res])
    assert runs[0] == runs[1]


def test_trajectory_mixed_precision(tg):
    """FP32 CG + FP64 reliable updates inside the trajectory: same dH to 1e-9
    and the same accept/reject decisions as the FP64 run."""
    d = golden("c1s_16x16_px")
    hp64 = tg.hmc_params(nsteps=40, rng=tg.native.RNG_MT, cg=tg.cg_params(rel_tol=1e-12, abs_tol2=0))
    hpmx = tg.hmc_params(nsteps=40, rng=tg.native.RNG_MT,
                         cg=tg.cg_params(rel_tol=1e-12, abs_tol2=0, precision=1, ru_interval=50))
    _, r64 = _replay(tg, d, hp64)
    _, rmx = _replay(tg, d, hpmx)
    for a, b, want in zip(r64, rmx, d["traj_stats"]):
        assert abs(a.dH - want[0]) < 1e-9
        assert abs(b.dH - want[0]) < 1e-9
        assert a.accepted == b.accepted == int(want[9])
        assert b.reliable_updates > 0


def test_trajectory_ext_matches_mt(tg, oracle_lib):
    """Caller-supplied fields reproduce the internal reference-stream trajectory."""
    d = golden("odd_6x4_apx")
    nt, nx = int(d["nt"]), int(d["nx"])
    hp = tg.hmc_params(nsteps=8, rng=tg.native.RNG_MT)
    L1, res = _replay(tg, d, hp)
    mt = oracle_lib.MT(int(d["traj_seed"]), 543210)
    mt.uniforms(2 * 2 * nt * nx * int(d["traj_sweeps"]))
    L2 = make(tg, d)
    L2.set_gauge(d["traj_A_start"])
    for r in res:
        eta, _ = mt.gaussian_field(nt, nx)
        mom, _ = mt.momentum(nt, nx)
        noise, _ = mt.gaussian_field(nt, nx)
        u = mt.next()
        r2 = L2.trajectory_ext(hp, eta, mom, noise, u)
        assert r2.dH == r.dH and r2.accepted == r.accepted
    assert np.array_equal(L1.get_gauge(), L2.get_gauge())


def test_philox_trajectories(tg):
    """Device RNG: reproducible for a seed, Gaussian moments as expected."""
    nt = nx = 32
    hp = tg.hmc_params(nsteps=40, rng=tg.native.RNG_PHILOX, seed=1234,
                       cg=tg.cg_params(rel_tol=1e-10, abs_tol2=0), stochastic_term=False)
    runs = []
    for _ in range(2):
        L = tg.Lattice(nt, nx, 0.5, 0.5, 0.0, -1, 1)
        runs.append([L.update_gauge(hp) for _ in range(3)])
    for a, b in zip(*runs):
        assert a.dH == b.dH and a.Spf0 == b.Spf0
    V = nt * nx
    for r in runs[0]:
        assert abs(r.Spf0 - 2 * V) < 6 * np.sqrt(4 * V)    # sum |eta|^2, E = 2V, Var = 4V
        assert abs(r.Smom0 - 2 * V) < 6 * np.sqrt(4 * V)
        assert r.status == 0 and np.isfinite(r.dH) and abs(r.dH) < 100
    assert runs[0][0].Spf0 != runs[0][1].Spf0             # new fields every trajectory


def test_errors_are_reported(tg):
    with pytest.raises(tg.native.TGError):
        tg.Lattice(1, 4, 0.1)
    with pytest.raises(tg.native.TGError):
        tg.Lattice(4, 4, 0.1, bc_x=3)
    L = tg.Lattice(4, 4, 0.1)
    with pytest.raises(tg.native.TGError):
        L.update_gauge(tg.hmc_params(npf=9))
    with pytest.raises(tg.native.TGError):
        L.update_gauge(tg.hmc_params(nsteps=0))


@pytest.mark.parametrize("nt,nx,mu", [(32, 32, 0.0), (64, 96, 0.3), (8, 64, 0.1)])
def test_column_march_equals_site_path(tg, monkeypatch, nt, nx, mu):
    """The warp column march (nx % 32 == 0) computes the same operator values,
    bit for bit, as the one-site-per-thread path, and the same CG solution."""
    rng = np.random.default_rng(nt + nx)
    A = rng.normal(0, 0.6, (nt, nx, 2))
    psi = cplx(rng, (nt, nx))
    out = []
    for flag in ("1", "0"):
        monkeypatch.setenv("TG_MARCH", flag)
        L = tg.Lattice(nt, nx, 0.2, 0.5, mu, -1, 1)
        L.set_gauge(A)
        x, res = L.fmdm_invert_cg(psi, tg.cg_params(rel_tol=1e-12, abs_tol2=0))
        xm, resm = L.fmdm_invert_cg(psi, tg.cg_params(rel_tol=1e-12, abs_tol2=0, precision=1))
        out.append((L.fm_mul(psi), L.fm_conjugate_mul(psi), x, xm, res.iterations))
    assert np.array_equal(out[0][0], out[1][0]) and np.array_equal(out[0][1], out[1][1])
    assert rel(out[0][2], out[1][2]) < 1e-10 and rel(out[0][3], out[1][3]) < 1e-9
    assert abs(out[0][4] - out[1][4]) <= 2
