"""Size-independent properties at the benchmark sizes and above, where the CPU
oracle is too slow to replay a solve or a trajectory:
  * the pseudofermion force at 1024^2 (the bench workload's couplings) equals
    the central difference of the pseudofermion action along a random
    direction of all 2 * 1024^2 links;
  * on the largest lattice the library takes (4092 x 4096, just under its
    2^24-site limit) the operator is linear, M^dag is its adjoint, and the
    FP32 operator agrees with FP64 to FP32 rounding; 4096 x 4096 is refused;
  * the CG at 2048^2 (m 0.02, A ~ N(0, 0.5^2)) reaches its target on the true
    residual in both precisions."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def tg():
    import thirring2d_gb300 as tg
    tg.native.load()
    return tg


def cplx(rng, shape):
    return rng.normal(size=shape) + 1j * rng.normal(size=shape)


def test_force_is_the_derivative_of_the_action_1024(tg):
    n = 1024
    rng = np.random.default_rng(101)
    A = rng.normal(0, 0.3, (n, n, 2))
    L = tg.Lattice(n, n, 0.05, 0.6, 0.0, -1, 1)
    L.set_gauge(A)
    phi = L.fm_conjugate_mul(cplx(rng, (n, n)))           # phi = M^dag eta, as the heatbath draws it
    cp = tg.cg_params(rel_tol=1e-12, abs_tol2=0)
    F, res = L.pf_force(phi, cp)
    assert res.status == 0
    D = rng.normal(size=(n, n, 2))
    h = 1e-4

    def S(At):
        L.set_gauge(At)
        s, r = L.pseudofermion_action(phi, cp)
        assert r.status == 0
        return s

    fd = (S(A + h * D) - S(A - h * D)) / (2 * h)
    want = float((F * D).sum())
    assert abs(fd - want) < 1e-5 * abs(want), (fd, want)


def test_operator_properties_largest_lattice(tg):
    with pytest.raises(tg.native.TGError):
        tg.Lattice(4096, 4096, 0.02)                            # 2^24 sites: over the limit
    nt, nx = 4092, 4096
    rng = np.random.default_rng(4096)
    L = tg.Lattice(nt, nx, 0.02, 0.8, 0.0, -1, 1)
    L.set_gauge(rng.normal(0, 0.5, (nt, nx, 2)))
    u, v = cplx(rng, (nt, nx)), cplx(rng, (nt, nx))
    Mv, Mdu = L.fm_mul(v), L.fm_conjugate_mul(u)
    lhs, rhs = np.vdot(u, Mv), np.vdot(Mdu, v)                  # <u, M v> = <M^dag u, v>
    assert abs(lhs - rhs) < 1e-12 * abs(lhs)
    a, b = 0.3 - 1.1j, 2.0 + 0.5j                               # linearity
    Mw = L.fm_mul(a * u + b * v)
    assert np.linalg.norm(Mw - (a * L.fm_mul(u) + b * Mv)) < 1e-13 * np.linalg.norm(Mw)
    torch = pytest.importorskip("torch")
    x = torch.from_numpy(np.stack([v.real, v.imag], -1).astype(np.float32)).cuda()
    y = torch.empty_like(x)
    torch.cuda.synchronize()
    L.apply_dev(x.data_ptr(), y.data_ptr(), False, tg.native.PREC_MIXED)
    L.synchronize()
    got = y.cpu().numpy().astype(np.float64)
    got = got[..., 0] + 1j * got[..., 1]
    assert np.linalg.norm(got - Mv) < 3e-7 * np.linalg.norm(Mv)


@pytest.mark.parametrize("precision", [0, 1])
def test_cg_true_residual_2048(tg, precision):
    n = 2048
    rng = np.random.default_rng(2048)
    L = tg.Lattice(n, n, 0.02, 0.8, 0.0, -1, 1)
    L.set_gauge(rng.normal(0, 0.5, (n, n, 2)))
    b = cplx(rng, (n, n))
    x, res = L.fmdm_invert_cg(b, tg.cg_params(rel_tol=1e-10, abs_tol2=0, precision=precision, ru_interval=50))
    assert res.status == 0
    r = b - L.fm_conjugate_mul(L.fm_mul(x))
    assert np.linalg.norm(r) / np.linalg.norm(b) < 1.5e-10
