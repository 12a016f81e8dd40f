"""Beside the HMC path: the fermion-bag operator of vec_ops.c and its CG
(against the reference's own outputs), and the measurements of hmc.c's
measure() plus a stochastic chiral condensate (against the oracle / exact
inverse)."""
import numpy as np
import pytest

from helpers import golden, rel

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def tg():
    import thirring2d_gb300 as tg
    tg.native.load()
    return tg


@pytest.mark.parametrize("name", ["vecops_8x8", "vecops_6x4", "vecops_16x16"])
def test_masked_operator_golden(tg, name):
    d = golden(name)
    L = tg.Lattice(int(d["nt"]), int(d["nx"]), float(d["m"]), 0.5, float(d["mu"]), -1, -1)
    assert np.abs(L.fM(d["mask"], d["v"]) - d["fM_v"]).max() < 1e-14
    assert np.abs(L.fM(d["mask"], d["v"], True) - d["fMt_v"]).max() < 1e-14
    x, res = L.cg_MdM(d["mask"], d["b"], tg.cg_params(maxiter=10000))   # vec_ops.c's stop, |r|^2 < 1e-30
    assert res.status == 0
    assert rel(x, d["cg_x"]) < 1e-12


def test_masked_operator_all_occupied_is_identity(tg):
    L = tg.Lattice(8, 8, 0.3, 0.5, 0.0, -1, -1)
    v = np.random.default_rng(1).normal(size=(8, 8))
    assert np.array_equal(L.fM(np.ones((8, 8), np.int32), v), v)


def test_magnetisation(tg):
    A = np.random.default_rng(2).normal(0, 0.7, (12, 20, 2))
    L = tg.Lattice(12, 20, 0.2)
    L.set_gauge(A)
    assert abs(L.magnetisation() - A.sum() / (12 * 20)) < 1e-13


def test_fermion_phase_reference_stream(tg, oracle_lib):
    """fermion_phase (hmc.c:794-815) with sources from the reference MT stream."""
    nt, nx, mu = 8, 8, 0.4
    A = np.random.default_rng(3).normal(0, 0.5, (nt, nx, 2))
    L = tg.Lattice(nt, nx, 0.3, 0.5, mu, -1, -1)
    L.set_gauge(A)
    L.seed_mersenne(99, 1000)
    got = L.fermion_phase(20)
    o = oracle_lib.Oracle(nt, nx, 0.3, 0.5, mu, -1, -1)
    mt = oracle_lib.MT(99, 1000)
    im = 0.0
    for _ in range(20):
        c, _ = mt.gaussian_field(nt, nx)
        mdc = o.Mdag(A, c)
        im += float((c.real * mdc.imag - c.imag * mdc.real).sum())
    assert abs(got - im / 20) < 1e-11 * max(1.0, abs(im / 20))
    assert abs(got) > 1e-6   # nonzero at mu != 0


def test_chiral_condensate_against_exact_trace(tg, oracle_lib):
    nt, nx, m = 8, 8, 0.3
    A = np.random.default_rng(4).normal(0, 0.5, (nt, nx, 2))
    L = tg.Lattice(nt, nx, m, 0.5, 0.0, -1, 1)
    L.set_gauge(A)
    pbp, err = L.chiral_condensate(400, seed=5, cp=tg.cg_params(rel_tol=1e-12, abs_tol2=0.0))
    o = oracle_lib.Oracle(nt, nx, m, 0.5, 0.0, -1, 1)
    exact = float(np.trace(np.linalg.inv(o.dense_M(A))).real) / (nt * nx)
    assert err > 0 and abs(pbp - exact) < 5 * err, (pbp, exact, err)


@pytest.mark.parametrize("name", ["det_4x4_apx", "det_4x4_px", "det_6x4_apx"])
def test_dense_matrix_and_determinant_golden(tg, name):
    """fermion_matrix / determinant (hmc.c:269-336) against the reference's
    dense matrix and numpy's log-determinant of it."""
    d = golden(name)
    L = tg.Lattice(int(d["nt"]), int(d["nx"]), float(d["m"]), 0.5, float(d["mu"]), -1, int(d["bc_x"]))
    L.set_gauge(d["A"])
    assert np.abs(L.fermion_matrix() - d["M"]).max() < 1e-15
    la, ph = L.log_det()
    assert abs(la - float(d["logabsdet"])) < 1e-12
    assert abs(np.exp(1j * ph) - complex(d["phase"])) < 1e-12


def test_batched_determinant_vs_numpy(tg, oracle_lib):
    nt, nx, m, mu = 8, 8, 0.2, 0.3
    rng = np.random.default_rng(6)
    As = rng.normal(0, 0.6, (12, nt, nx, 2))
    As[0] = 0.0   # A = 0: the free operator (fermion_matrix.c / full_determinant.c at an empty field)
    L = tg.Lattice(nt, nx, m, 0.5, mu, -1, -1)
    la, ph = L.log_det(As)
    o = oracle_lib.Oracle(nt, nx, m, 0.5, mu, -1, -1)
    for k, A in enumerate(As):
        sign, logabs = np.linalg.slogdet(o.dense_M(A))
        assert abs(la[k] - logabs) < 1e-10 * max(1.0, abs(logabs))
        assert abs(np.exp(1j * ph[k]) - sign) < 1e-10


@pytest.mark.parametrize("name", ["free_det_8x8", "free_det_6x4"])
def test_free_determinant_golden(tg, name):
    """log det M at A = 0 against the fermion-bag matrix of the reference's vec_ops.c."""
    d = golden(name)
    nt, nx = int(d["nt"]), int(d["nx"])
    L = tg.Lattice(nt, nx, float(d["m"]), 0.5, float(d["mu"]), -1, -1)
    la, ph = L.log_det(np.zeros((1, nt, nx, 2)))
    assert abs(la[0] - float(d["logabsdet"])) < 1e-12
    assert abs(np.exp(1j * ph[0]) - float(d["sign"])) < 1e-12


@pytest.mark.parametrize("name", ["prop_8x8", "prop_6x4_mask"])
def test_fm_propagator_golden(tg, name):
    """calc_Dinv (fermion_matrix.c:189-351): one CG per source on the GPU against
    the reference's propagator matrix."""
    d = golden(name)
    L = tg.Lattice(int(d["nt"]), int(d["nx"]), float(d["m"]), 0.5, float(d["mu"]), -1, -1)
    D, res = L.fm_propagator(d["mask"])
    assert res.status == 0 and res.iterations > 0
    assert np.abs(D - d["Dinv"]).max() < 1e-10 * np.abs(d["Dinv"]).max()


def test_fm_propagator_vs_dense_inverse(tg, oracle_lib):
    """32x32, m 0.1, mu 0.1, 15% monomers: every block of the propagator matrix
    against numpy's inverse of the oracle's dense masked operator."""
    nt = nx = 32
    V = nt * nx
    rng = np.random.default_rng(32)
    mask = (rng.random((nt, nx)) < 0.15).astype(np.int32)
    o = oracle_lib.Oracle(nt, nx, 0.1, 0.5, 0.1, -1, -1)
    Mf = np.stack([o.fM(mask, np.eye(V)[j].reshape(nt, nx)).ravel() for j in range(V)], 1)
    Minv = np.linalg.inv(Mf)
    L = tg.Lattice(nt, nx, 0.1, 0.5, 0.1, -1, -1)
    D, res = L.fm_propagator(mask)
    assert res.status == 0
    t, x = np.divmod(np.arange(V), nx)
    par = (t + x) & 1
    idx = np.arange(V) // 2
    for p_src, blk in ((1, 0), (0, 1)):   # odd sources -> block 0, even sources -> block 1
        src = np.where(par == p_src)[0]
        dst = np.where(par != p_src)[0]
        want = np.zeros_like(D[blk])
        want[np.ix_(idx[dst], idx[src])] = Minv[np.ix_(dst, src)]
        assert np.abs(D[blk] - want).max() < 1e-9 * np.abs(Minv).max()
