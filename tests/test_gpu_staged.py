"""The FP32 stencil kernels with their rows staged through shared memory by
TMA bulk copies (TG_STAGED=1, on lattices with nx a multiple of 32) against
the same kernels loading from global memory (the default): the arithmetic is
the same, so operator applies are bitwise equal and solves agree to the rounding
of their grid sums; and no staged wait ever ran out."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")


@pytest.fixture(scope="module")
def tg():
    import thirring2d_gb300 as tg
    tg.native.load()
    return tg


def cplx(rng, shape):
    return rng.normal(size=shape) + 1j * rng.normal(size=shape)


def fp32_apply(tg, L, psi, dagger):
    x = torch.from_numpy(np.stack([psi.real, psi.imag], -1).astype(np.float32)).cuda()
    y = torch.empty_like(x)
    torch.cuda.synchronize()
    L.apply_dev(x.data_ptr(), y.data_ptr(), dagger, tg.native.PREC_MIXED)
    L.synchronize()
    return y.cpu().numpy()


# sizes: chunks only, a tail row per segment (nt = 4k+1, +2), a lattice
# smaller than one warp range, and the 1024^2 workload
@pytest.mark.parametrize("nt,nx,mu", [(64, 64, 0.0), (96, 128, 0.3), (36, 32, 0.0), (8, 64, 0.2), (1024, 1024, 0.0)])
def test_staged_apply_bitwise(tg, monkeypatch, nt, nx, mu):
    rng = np.random.default_rng(nt + nx)
    A = rng.normal(0, 0.5, (nt, nx, 2))
    psi = cplx(rng, (nt, nx))
    L = tg.Lattice(nt, nx, 0.1, 0.5, mu, -1, 1)
    L.set_gauge(A)
    out = {}
    for staged in ("1", "0"):
        monkeypatch.setenv("TG_STAGED", staged)
        out[staged] = [fp32_apply(tg, L, psi, d) for d in (False, True)]
    for a, b in zip(out["1"], out["0"]):
        assert np.array_equal(a, b)
    assert tg.native.stage_faults() == 0


@pytest.mark.parametrize("nt,nx", [(64, 64), (1024, 1024)])
def test_staged_mixed_cg_agrees(tg, monkeypatch, nt, nx):
    rng = np.random.default_rng(7 * nt)
    A = rng.normal(0, 0.3, (nt, nx, 2))
    b = cplx(rng, (nt, nx))
    res = {}
    for staged in ("1", "0"):
        monkeypatch.setenv("TG_STAGED", staged)
        L = tg.Lattice(nt, nx, 0.05, 0.6, 0.0, -1, 1)     # new lattice: no cached graph
        L.set_gauge(A)
        res[staged] = L.fmdm_invert_cg(b, tg.cg_params(rel_tol=1e-10, abs_tol2=0, precision=1, ru_interval=50))
        L.close()
    (x1, r1), (x0, r0) = res["1"], res["0"]
    assert r1.status == r0.status == 0
    # same arithmetic per site; the two kernels may run on different grids
    # (the staged one is limited by shared memory), so the per-block partial
    # sums of the dot products, and with them the last bits, can differ
    assert abs(r1.iterations - r0.iterations) <= 2
    assert np.linalg.norm(x1 - x0) / np.linalg.norm(x0) < 1e-7
    assert tg.native.stage_faults() == 0

