"""The persistent CG solver (TG_SOLVER_PERSISTENT: one cooperative launch per
solve, grid barriers inside) against the reference's outputs, the oracle and
the launch-per-iteration solver: same stopping rules (hmc.c:341-404), same
solutions to rounding, same trajectories."""
import numpy as np
import pytest

from helpers import STABLE, TRAJ_CONFIGS, dH_ok, golden, lat_args, rel

pytestmark = pytest.mark.gpu

PERSISTENT = 2
LAUNCHES = 1


@pytest.fixture(scope="module")
def tg():
    import thirring2d_gb300 as tg
    tg.native.load()
    return tg


def make(tg, d):
    return tg.Lattice(*lat_args(d))


def cplx(rng, shape):
    return rng.normal(size=shape) + 1j * rng.normal(size=shape)


@pytest.mark.parametrize("name", TRAJ_CONFIGS)
def test_persistent_cg_golden(tg, name):
    d = golden(name)
    L = make(tg, d)
    L.set_gauge(d["A"])
    x, res = L.fmdm_invert_cg(d["psi"], tg.cg_params(solver=PERSISTENT))  # hmc.c's stop |r|^2 < 1e-30
    assert res.status == 0
    assert rel(x, d["cg_x"]) < 1e-12


@pytest.mark.parametrize("nt,nx,mu", [(64, 64, 0.0), (96, 128, 0.3), (12, 10, 0.0), (2, 64, 0.0)])
def test_persistent_equals_launches(tg, oracle_lib, nt, nx, mu):
    rng = np.random.default_rng(nt * 1000 + nx)
    A = rng.normal(0, 0.5, (nt, nx, 2))
    b = cplx(rng, (nt, nx))
    L = tg.Lattice(nt, nx, 0.2, 0.5, mu, -1, 1)
    L.set_gauge(A)
    out = {}
    for solver in (LAUNCHES, PERSISTENT):
        out[solver] = L.fmdm_invert_cg(b, tg.cg_params(rel_tol=1e-12, abs_tol2=0, solver=solver))
    (x1, r1), (x2, r2) = out[LAUNCHES], out[PERSISTENT]
    assert r1.status == r2.status == 0
    assert abs(r1.iterations - r2.iterations) <= 2
    assert rel(x2, x1) < 1e-11
    # the stop tests the recursive residual (1e-12); the true one drifts above it
    # by the same amount in both solvers
    o = oracle_lib.Oracle(nt, nx, 0.2, 0.5, mu, -1, 1)
    true = [np.linalg.norm(b - o.Mdag(A, o.M(A, x))) / np.linalg.norm(b) for x in (x1, x2)]
    assert true[1] < 5e-11 and true[1] < 3 * true[0] + 1e-12, true


@pytest.mark.parametrize("precision", [0, 1])
def test_persistent_1024(tg, oracle_lib, precision):
    """The 1024^2 workload: true residual below the target, iteration counts
    as the launch-per-iteration solver's."""
    n = 1024
    rng = np.random.default_rng(1024)
    A = rng.normal(0, 0.3, (n, n, 2))
    b = cplx(rng, (n, n))
    L = tg.Lattice(n, n, 0.05, 0.6, 0.0, -1, 1)
    L.set_gauge(A)
    cp = dict(rel_tol=1e-10, abs_tol2=0, precision=precision, ru_interval=50)
    x, res = L.fmdm_invert_cg(b, tg.cg_params(solver=PERSISTENT, **cp))
    _, ref = L.fmdm_invert_cg(b, tg.cg_params(solver=LAUNCHES, **cp))
    assert res.status == 0
    assert abs(res.iterations - ref.iterations) <= max(3, ref.iterations // 50)
    o = oracle_lib.Oracle(n, n, 0.05, 0.6, 0.0, -1, 1)
    r = b - o.Mdag(A, o.M(A, x))
    assert np.linalg.norm(r) / np.linalg.norm(b) < 1.5e-10
    if precision == 1:
        assert res.reliable_updates >= 1


@pytest.mark.parametrize("form", ["fp64", "twosum", "onesum"])
def test_grid_of_more_than_256_blocks(tg, oracle_lib, monkeypatch, form):
    """256-thread blocks, two per SM, on a lattice whose work fills them all:
    the grid has more blocks than warp 0 reads in one round of partial loads
    (256), so every grid sum takes two.  The solution against the oracle and
    against the default 512-thread shape."""
    nt, nx = 1024, 512
    rng = np.random.default_rng(77)
    A = rng.normal(0, 0.3, (nt, nx, 2))
    b = cplx(rng, (nt, nx))
    L = tg.Lattice(nt, nx, 0.05, 0.6, 0.0, -1, 1)
    L.set_gauge(A)
    prec = 0 if form == "fp64" else 1
    monkeypatch.setenv("TG_MIXED_CG", "twosum" if form == "fp64" else form)
    cp = tg.cg_params(rel_tol=1e-10, abs_tol2=0, precision=prec, ru_interval=50, solver=PERSISTENT)
    out = {}
    for block in ("256", "512"):
        monkeypatch.setenv("TG_PCG_BLOCK", block)
        out[block] = L.fmdm_invert_cg(b, cp)
    (x2, r2), (x5, r5) = out["256"], out["512"]
    assert r2.status == r5.status == 0
    assert abs(r2.iterations - r5.iterations) <= max(3, r5.iterations // 50)
    o = oracle_lib.Oracle(nt, nx, 0.05, 0.6, 0.0, -1, 1)
    true = np.linalg.norm(b - o.Mdag(A, o.M(A, x2))) / np.linalg.norm(b)
    assert true < 1.5e-10, true
    assert rel(x2, x5) < 1e-6   # both at 1e-10 residual; M^dag M at m 0.05 has a condition number of ~2000


@pytest.mark.parametrize("case", ["heavy", "tiny", "large"])
def test_mixed_fixed_point_sums_leave_their_scale(tg, oracle_lib, case):
    """The mixed solver adds its iteration sums as integers at a power-of-two
    scale that follows the last total of the same kind.  Systems whose sums
    leave that scale: a heavy mass (the first |Mp|^2 is ~2500 |b|^2, past a
    block's 256-fold headroom, so every block takes the exact path), and
    right-hand sides of norm 1e-6 and 1e+12 per site (scales of 2^70 and
    2^-51).  Each solve against the FP64 solve and the oracle's residual.  (The
    FP32 iterations themselves need |b| within FP32's range: at 1e-15 per site
    the converged residual's squares, ~1e-50, underflow FP32.)"""
    nt, nx = 128, 128   # a multi-block grid (fixed-point sums)
    m = 50.0 if case == "heavy" else 0.2
    amp = {"heavy": 1.0, "tiny": 1e-6, "large": 1e12}[case]
    rng = np.random.default_rng(31)
    A = rng.normal(0, 0.4, (nt, nx, 2))
    b = amp * cplx(rng, (nt, nx))
    L = tg.Lattice(nt, nx, m, 0.5, 0.0, -1, 1)
    L.set_gauge(A)
    out = {}
    for prec in (0, 1):
        out[prec] = L.fmdm_invert_cg(b, tg.cg_params(rel_tol=1e-10, abs_tol2=0, precision=prec, ru_interval=50,
                                                    solver=PERSISTENT))
    (x64, r64), (xmx, rmx) = out[0], out[1]
    assert r64.status == rmx.status == 0
    assert abs(rmx.iterations - r64.iterations) <= max(3, r64.iterations // 10)
    assert rel(xmx, x64) < 1e-7
    o = oracle_lib.Oracle(nt, nx, m, 0.5, 0.0, -1, 1)
    assert np.linalg.norm(b - o.Mdag(A, o.M(A, xmx))) / np.linalg.norm(b) < 1.5e-10


@pytest.mark.parametrize("precision", [0, 1])
def test_persistent_edge_cases(tg, precision):
    rng = np.random.default_rng(9)
    L = tg.Lattice(32, 32, 0.3, 0.5, 0.0, -1, 1)
    L.set_gauge(rng.normal(0, 0.5, (32, 32, 2)))
    cp = dict(solver=PERSISTENT, precision=precision, ru_interval=50)
    x, res = L.fmdm_invert_cg(np.zeros((32, 32), complex), tg.cg_params(**cp))  # hmc.c:359-361
    assert res.status == 0 and res.iterations == 0 and not x.any()
    x, res = L.fmdm_invert_cg(cplx(rng, (32, 32)), tg.cg_params(maxiter=3, **cp))
    assert res.status == tg.native.TG_E_NOCONV and res.iterations == 3
    bad = cplx(rng, (32, 32))
    bad[2, 3] = np.nan
    x, res = L.fmdm_invert_cg(bad, tg.cg_params(**cp))
    assert res.status == tg.native.TG_E_NAN
    # the lattice is still usable afterwards
    x, res = L.fmdm_invert_cg(cplx(rng, (32, 32)), tg.cg_params(rel_tol=1e-10, abs_tol2=0, **cp))
    assert res.status == 0


def test_single_reduction_edge_cases(tg, monkeypatch):
    """The single-reduction mixed CG (TG_MIXED_CG=onesum) on a column-march
    lattice: b = 0 returns x = 0 at once (hmc.c:359-361), the iteration cap
    reports TG_E_NOCONV with exactly that many iterations, a NaN in b reports
    TG_E_NAN, a singular operator ends with a failure status, and the lattice
    solves normally afterwards."""
    monkeypatch.setenv("TG_MIXED_CG", "onesum")
    rng = np.random.default_rng(19)
    L = tg.Lattice(32, 32, 0.3, 0.5, 0.0, -1, 1)
    L.set_gauge(rng.normal(0, 0.5, (32, 32, 2)))
    cp = dict(solver=PERSISTENT, precision=tg.native.PREC_MIXED, ru_interval=50)
    x, res = L.fmdm_invert_cg(np.zeros((32, 32), complex), tg.cg_params(**cp))
    assert res.status == 0 and res.iterations == 0 and not x.any()
    x, res = L.fmdm_invert_cg(cplx(rng, (32, 32)), tg.cg_params(maxiter=3, **cp))
    assert res.status == tg.native.TG_E_NOCONV and res.iterations == 3
    bad = cplx(rng, (32, 32))
    bad[2, 3] = np.nan
    x, res = L.fmdm_invert_cg(bad, tg.cg_params(**cp))
    assert res.status == tg.native.TG_E_NAN
    x, res = L.fmdm_invert_cg(cplx(rng, (32, 32)), tg.cg_params(rel_tol=1e-10, abs_tol2=0, **cp))
    assert res.status == 0
    S = tg.Lattice(32, 32, 0.0, 0.5, 0.0, 1, 1)   # m = 0, periodic, A = 0: exact zero modes
    x, res = S.fmdm_invert_cg(cplx(rng, (32, 32)), tg.cg_params(rel_tol=1e-12, abs_tol2=0, maxiter=5000, **cp))
    assert res.status in (tg.native.TG_E_DIVERGED, tg.native.TG_E_NAN, tg.native.TG_E_NOCONV)
    S.set_couplings(0.3, 0.5, 0.0)
    x, res = S.fmdm_invert_cg(cplx(rng, (32, 32)), tg.cg_params(rel_tol=1e-10, abs_tol2=0, **cp))
    assert res.status == 0


def _replay(tg, d, hp):
    L = make(tg, d)
    L.seed_mersenne(int(d["traj_seed"]), 543210)
    L.update_puregauge_hb(int(d["traj_sweeps"]))
    return L, [L.update_gauge(hp) for _ in range(len(d["traj_stats"]))]


@pytest.mark.parametrize("name", TRAJ_CONFIGS)
@pytest.mark.parametrize("use_graph", [True, False])
def test_persistent_trajectories_golden(tg, name, use_graph):
    d = golden(name)
    hp = tg.hmc_params(nsteps=int(d["traj_nsteps"]), tau=1.0, npf=1, stochastic_term=True,
                       rng=tg.native.RNG_MT, use_graph=use_graph, cg=tg.cg_params(solver=PERSISTENT))
    L, res = _replay(tg, d, hp)
    for k, (r, want) in enumerate(zip(res, d["traj_stats"])):
        assert r.status == 0
        assert dH_ok(r.dH, want[0], name in STABLE), (k, r.dH, want[0])
        assert r.accepted == int(want[9])
    assert np.abs(L.get_gauge() - d["traj_A"][-1]).max() < 1e-9


def test_persistent_mixed_trajectory(tg):
    d = golden("c1s_16x16_px")
    hp = tg.hmc_params(nsteps=40, rng=tg.native.RNG_MT,
                       cg=tg.cg_params(rel_tol=1e-12, abs_tol2=0, precision=1, ru_interval=50, solver=PERSISTENT))
    _, res = _replay(tg, d, hp)
    for r, want in zip(res, d["traj_stats"]):
        assert abs(r.dH - want[0]) < 1e-9
        assert r.accepted == int(want[9])
        assert r.reliable_updates > 0


def test_grid_barrier_gives_up_and_device_stays_usable(tg):
    """The grid barrier's bounded wait: a barrier that also waits for blocks
    that never arrive returns TG_E_TIMEOUT after its poll limit instead of
    hanging, and the device keeps working (a solve right after converges)."""
    import ctypes as C
    lib = tg.native.load()
    st = C.c_int(-99)
    tg.native.check(lib.tg_grid_barrier_check(0, 0, C.byref(st)))
    assert st.value == 0
    tg.native.check(lib.tg_grid_barrier_check(0, 1, C.byref(st)))
    assert st.value == tg.native.TG_E_TIMEOUT
    L = tg.Lattice(32, 32, 0.2, 0.5, 0.0, -1, 1)
    L.set_gauge(np.random.default_rng(4).normal(0, 0.3, (32, 32, 2)))
    b = np.random.default_rng(5).normal(size=(32, 32)) + 0j
    x, res = L.fmdm_invert_cg(b, tg.cg_params(rel_tol=1e-10, abs_tol2=0, solver=tg.native.SOLVER_PERSISTENT))
    assert res.status == 0
    r = b - L.fm_conjugate_mul(L.fm_mul(x))
    assert np.linalg.norm(r) < 2e-10 * np.linalg.norm(b)


@pytest.mark.parametrize("nt,nx,mu,m,tol", [(64, 64, 0.0, 0.1, 1e-10), (32, 96, 0.3, 0.2, 1e-12), (256, 256, 0.0, 0.05, 1e-10),
                                            (4, 32, 0.0, 0.3, 1e-10), (1024, 1024, 0.0, 0.05, 1e-10),
                                            (2048, 2048, 0.0, 0.02, 1e-10)])
def test_single_reduction_mixed_cg(tg, oracle_lib, monkeypatch, nt, nx, mu, m, tol):
    """The single-reduction mixed CG on column-march lattices (one grid sum and
    one fused M^dag M pass per iteration, after an elementwise update;
    TG_MIXED_CG=onesum; the default above 1.5 times the L2) against the two-sum
    form on the same system: the same status, iteration counts within 2%,
    solutions within the tolerance's reach, and the true residual
    |b - M^dag M x| / |b| (oracle, FP64) below the target."""
    form = "onesum"
    rng = np.random.default_rng(nt + 7 * nx)
    A = rng.normal(0, 0.3, (nt, nx, 2))
    b = cplx(rng, (nt, nx))
    cp = tg.cg_params(rel_tol=tol, abs_tol2=0, precision=tg.native.PREC_MIXED, ru_interval=50, solver=PERSISTENT)
    out = {}
    for f in ("twosum", form):
        monkeypatch.setenv("TG_MIXED_CG", f)
        L = tg.Lattice(nt, nx, m, 0.5, mu, -1, 1)
        L.set_gauge(A)
        out[f] = L.fmdm_invert_cg(b, cp)
        L.close()
    (x2, r2), (x1, r1) = out["twosum"], out[form]
    assert r1.status == r2.status == 0
    assert abs(r1.iterations - r2.iterations) <= max(2, r2.iterations // 50), (r1.iterations, r2.iterations)
    assert r1.reliable_updates >= 1
    assert rel(x1, x2) < 100 * tol
    o = oracle_lib.Oracle(nt, nx, m, 0.5, mu, -1, 1)
    true = np.linalg.norm(b - o.Mdag(A, o.M(A, x1))) / np.linalg.norm(b)
    assert true < 1.5 * tol, true


def test_single_reduction_trajectories_match_reference(tg, monkeypatch):
    """Whole trajectories with the single-reduction mixed CG on a column-march
    reference fixture: dH within 1e-9 of the reference's, same decisions."""
    monkeypatch.setenv("TG_MIXED_CG", "onesum")
    d = golden("march_32x64_mu_px")
    hp = tg.hmc_params(nsteps=int(d["traj_nsteps"]), tau=1.0, npf=1, stochastic_term=True, rng=tg.native.RNG_MT,
                       cg=tg.cg_params(rel_tol=1e-13, abs_tol2=0, precision=tg.native.PREC_MIXED, ru_interval=50,
                                       solver=PERSISTENT))
    L, res = _replay(tg, d, hp)
    for k, (r, want) in enumerate(zip(res, d["traj_stats"])):
        assert r.status == 0
        assert abs(r.dH - want[0]) <= 1e-9, (k, r.dH, want[0])
        assert r.accepted == int(want[9])
    assert np.abs(L.get_gauge() - d["traj_A"][-1]).max() <= 1e-9


def test_single_reduction_graph_equals_eager(tg, monkeypatch):
    """The single-reduction mixed solve inside a trajectory captured as a CUDA
    graph and launched eagerly: the same kernels on the same data, so bitwise
    the same dH, decisions and field."""
    monkeypatch.setenv("TG_MIXED_CG", "onesum")
    d = golden("march_32x96_apx")
    runs = []
    for use_graph in (True, False):
        hp = tg.hmc_params(nsteps=int(d["traj_nsteps"]), rng=tg.native.RNG_MT, use_graph=use_graph,
                           cg=tg.cg_params(rel_tol=1e-12, abs_tol2=0, precision=tg.native.PREC_MIXED, ru_interval=50,
                                           solver=PERSISTENT))
        L, res = _replay(tg, d, hp)
        runs.append(([r.dH for r in res], [r.accepted for r in res], L.get_gauge()))
    assert runs[0][0] == runs[1][0] and runs[0][1] == runs[1][1]
    assert np.array_equal(runs[0][2], runs[1][2])
