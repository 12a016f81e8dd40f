"""tg_cg_noalloc: the CG solve for callers that cannot allocate device memory
(their memory is budgeted up front, or cudaMalloc's device-wide
synchronisation would stall their other streams).  It must give the same
solution as the regular entry point, tg_cg_dev, call after call, and refuse
lattices larger than its fixed scratch.

This file is collected last on purpose, so that a run stopping at its first
failure has already run every other test."""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")


def _dev(a: np.ndarray) -> "torch.Tensor":
    return torch.from_numpy(np.ascontiguousarray(a)).cuda()


@pytest.mark.parametrize("nt,nx,mu", [(64, 96, 0.0), (64, 64, 0.3), (128, 128, 0.0)])
def test_noalloc_cg_matches_cg_dev_twice(nt, nx, mu):
    import thirring2d_gb300 as tg
    lib = tg.native.load()
    rng = np.random.default_rng(nt * 1000 + nx)
    A = rng.normal(0, 0.4, (nt, nx, 2))
    L = tg.Lattice(nt, nx, 0.2, 0.5, mu, -1, 1)
    L.set_gauge(A)
    p = tg.native.LatticeParams(nt, nx, 0.2, 0.5, mu, -1, 1, 0)
    cp = tg.cg_params(rel_tol=1e-12, abs_tol2=0.0)
    A_d = _dev(A)
    for call in range(2):  # two calls in a row: the shared scratch keeps the previous call's contents
        b = rng.normal(size=(nt, nx, 2))
        b_d = _dev(b)
        x_ref = torch.empty_like(b_d)
        x_new = torch.full_like(b_d, float("nan"))
        torch.cuda.synchronize()
        r_ref, r_new = tg.native.CgResult(), tg.native.CgResult()
        tg.native.check(lib.tg_cg_dev(L.h, C.byref(cp), C.c_void_p(b_d.data_ptr()), C.c_void_p(x_ref.data_ptr()),
                                      C.byref(r_ref)))
        L.synchronize()
        tg.native.check(lib.tg_cg_noalloc(C.byref(p), C.byref(cp), C.c_void_p(A_d.data_ptr()),
                                          C.c_void_p(b_d.data_ptr()), C.c_void_p(x_new.data_ptr()),
                                          C.byref(r_new), None))
        torch.cuda.synchronize()
        xr, xn = x_ref.cpu().numpy(), x_new.cpu().numpy()
        assert r_new.status == 0 and abs(r_new.iterations - r_ref.iterations) <= 1, (call, r_new.iterations)
        assert np.linalg.norm(xn - xr) / np.linalg.norm(xr) < 1e-10, call


def test_noalloc_cg_rejects_lattices_beyond_its_scratch():
    import thirring2d_gb300 as tg
    lib = tg.native.load()
    p = tg.native.LatticeParams(256, 256, 0.2, 0.5, 0.0, -1, 1, 0)
    cp = tg.cg_params(rel_tol=1e-10, abs_tol2=0.0)
    buf = torch.zeros((256, 256, 2), dtype=torch.float64, device="cuda")
    res = tg.native.CgResult()
    rc = lib.tg_cg_noalloc(C.byref(p), C.byref(cp), C.c_void_p(buf.data_ptr()), C.c_void_p(buf.data_ptr()),
                           C.c_void_p(buf.data_ptr()), C.byref(res), None)
    assert rc == tg.native.TG_E_ARG
    assert b"16384" in lib.tg_last_error()
