"""tg_cg_noalloc: the CG solve for callers that cannot allocate device memory
(their memory is budgeted up front, or cudaMalloc's device-wide
synchronisation would stall their other streams).  It must give the same
solution as the regular entry point, tg_cg_dev, and as the CPU oracle, call
after call, on the column-march and the one-site-per-thread stencil paths and
every boundary condition; it must allocate nothing, refuse lattices larger
than its fixed scratch, and refuse a stream under capture.

This file is collected last on purpose, so that a run stopping at its first
failure has already run every other test."""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")


def _dev(a: np.ndarray) -> "torch.Tensor":
    return torch.from_numpy(np.ascontiguousarray(a)).cuda()


def _noalloc(lib, p, cp, A_d, b_d, x_d, res, stream=None):
    return lib.tg_cg_noalloc(C.byref(p), C.byref(cp), C.c_void_p(A_d.data_ptr()), C.c_void_p(b_d.data_ptr()),
                             C.c_void_p(x_d.data_ptr()), C.byref(res), stream)


# (nt, nx, mu, bc_t, bc_x): march shapes (nx % 32 == 0, nt % 4 == 0) and
# site-path shapes, with antiperiodic, periodic and open boundaries, odd sides
SHAPES = [(64, 96, 0.0, -1, 1), (64, 64, 0.3, -1, 1), (128, 128, 0.0, -1, 1), (6, 4, 0.2, 0, 1),
          (24, 20, 0.0, -1, -1), (15, 9, 0.1, -1, 1), (16, 16, 0.0, 1, 0)]


@pytest.mark.parametrize("nt,nx,mu,bc_t,bc_x", SHAPES)
def test_noalloc_cg_matches_cg_dev_and_oracle_twice(oracle_lib, nt, nx, mu, bc_t, bc_x):
    import thirring2d_gb300 as tg
    lib = tg.native.load()
    rng = np.random.default_rng(nt * 1000 + nx)
    A = rng.normal(0, 0.4, (nt, nx, 2))
    L = tg.Lattice(nt, nx, 0.2, 0.5, mu, bc_t, bc_x)
    L.set_gauge(A)
    o = oracle_lib.Oracle(nt, nx, 0.2, 0.5, mu, bc_t, bc_x)
    p = tg.native.LatticeParams(nt, nx, 0.2, 0.5, mu, bc_t, bc_x, 0)
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
        tg.native.check(_noalloc(lib, p, cp, A_d, b_d, x_new, r_new))
        torch.cuda.synchronize()
        xr, xn = x_ref.cpu().numpy(), x_new.cpu().numpy()
        assert r_new.status == 0 and abs(r_new.iterations - r_ref.iterations) <= 1, (call, r_new.iterations)
        assert np.linalg.norm(xn - xr) / np.linalg.norm(xr) < 1e-10, call
        xo, st, it = o.cg(A, b[..., 0] + 1j * b[..., 1], rel_tol=1e-12, abs_tol2=0)
        got = xn[..., 0] + 1j * xn[..., 1]
        assert st == 0 and abs(r_new.iterations - it) <= 2, (call, r_new.iterations, it)
        assert np.linalg.norm(got - xo) / np.linalg.norm(xo) < 1e-10, call
    L.close()


def test_noalloc_cg_allocates_nothing():
    """After a first call (which loads the kernels), a second call changes
    neither the device's free memory nor torch's allocator."""
    import thirring2d_gb300 as tg
    lib = tg.native.load()
    nt, nx = 64, 64
    rng = np.random.default_rng(11)
    A_d = _dev(rng.normal(0, 0.4, (nt, nx, 2)))
    b_d = _dev(rng.normal(size=(nt, nx, 2)))
    x_d = torch.empty_like(b_d)
    p = tg.native.LatticeParams(nt, nx, 0.2, 0.5, 0.0, -1, 1, 0)
    cp = tg.cg_params(rel_tol=1e-10, abs_tol2=0.0)
    res = tg.native.CgResult()
    torch.cuda.synchronize()
    tg.native.check(_noalloc(lib, p, cp, A_d, b_d, x_d, res))
    torch.cuda.synchronize()
    free0, torch0 = torch.cuda.mem_get_info()[0], torch.cuda.memory_allocated()
    tg.native.check(_noalloc(lib, p, cp, A_d, b_d, x_d, res))
    torch.cuda.synchronize()
    assert res.status == 0
    assert torch.cuda.mem_get_info()[0] == free0
    assert torch.cuda.memory_allocated() == torch0


def test_noalloc_cg_rejects_lattices_beyond_its_scratch():
    import thirring2d_gb300 as tg
    lib = tg.native.load()
    p = tg.native.LatticeParams(256, 256, 0.2, 0.5, 0.0, -1, 1, 0)
    cp = tg.cg_params(rel_tol=1e-10, abs_tol2=0.0)
    buf = torch.zeros((256, 256, 2), dtype=torch.float64, device="cuda")
    res = tg.native.CgResult()
    rc = _noalloc(lib, p, cp, buf, buf, buf, res)
    assert rc == tg.native.TG_E_ARG
    assert b"16384" in lib.tg_last_error()


def test_noalloc_cg_refuses_a_capturing_stream():
    """A call on a stream under capture returns TG_E_ARG before it enqueues
    anything; the capture then ends cleanly and the stream works again."""
    import thirring2d_gb300 as tg
    lib = tg.native.load()
    nt, nx = 16, 16
    rng = np.random.default_rng(12)
    A_d = _dev(rng.normal(0, 0.4, (nt, nx, 2)))
    b_d = _dev(rng.normal(size=(nt, nx, 2)))
    x_d = torch.zeros_like(b_d)
    p = tg.native.LatticeParams(nt, nx, 0.2, 0.5, 0.0, -1, 1, 0)
    cp = tg.cg_params(rel_tol=1e-10, abs_tol2=0.0)
    res = tg.native.CgResult()
    s = torch.cuda.Stream()
    torch.cuda.synchronize()
    graph = torch.cuda.CUDAGraph()
    with torch.cuda.graph(graph, stream=s):
        y = x_d * 2.0  # the capture holds one node of torch's own
        rc = _noalloc(lib, p, cp, A_d, b_d, x_d, res, C.c_void_p(s.cuda_stream))
    assert rc == tg.native.TG_E_ARG
    assert b"capture" in lib.tg_last_error()
    graph.replay()
    torch.cuda.synchronize()
    assert y.shape == x_d.shape
    tg.native.check(_noalloc(lib, p, cp, A_d, b_d, x_d, res, C.c_void_p(s.cuda_stream)))
    s.synchronize()
    assert res.status == 0
