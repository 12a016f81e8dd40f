"""numpy front end over the C ABI: one `Lattice` per tg_lattice.

Method names follow the reference hmc.c functions they replace (fm_mul,
fm_conjugate_mul, fmdm_invert_cg, calc_gauge_action, ...).  Arrays:
A / momenta / forces float64[nt, nx, 2]; fermion vectors complex128[nt, nx].
Every call runs on the GPU through libthirring_gpu.so; errors raise TGError.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import native as N

_dp = C.POINTER(C.c_double)


def _f64(a) -> np.ndarray:
    return np.ascontiguousarray(a, dtype=np.float64)


def _c128(a) -> np.ndarray:
    return np.ascontiguousarray(a, dtype=np.complex128)


def _p(a: np.ndarray):
    return a.ctypes.data_as(_dp)


def cg_params(rel_tol=0.0, abs_tol2=1e-30, maxiter=100000, precision=N.PREC_FP64, ru_interval=50,
              solver=N.SOLVER_DEFAULT) -> N.CgParams:
    """CG settings; the defaults are hmc.c's (CG_ACCURACY 1e-30 absolute, hmc.c:34-35)."""
    return N.CgParams(rel_tol, abs_tol2, maxiter, precision, ru_interval, solver)


def hmc_params(nsteps=10, tau=1.0, npf=1, stochastic_term=True, rng=N.RNG_MT, use_graph=True, seed=0,
               cg=None) -> N.HmcParams:
    """Trajectory settings; the defaults are hmc.c's update_gauge (hmc.c:708-709)."""
    return N.HmcParams(nsteps, tau, npf, int(stochastic_term), rng, int(use_graph), seed, cg or cg_params())


class Lattice:
    def __init__(self, nt: int, nx: int, m: float, g: float = 0.5, mu: float = 0.0,
                 bc_t: int = N.BC_ANTIPERIODIC, bc_x: int = N.BC_ANTIPERIODIC, device: int = 0):
        self.lib = N.load()
        self.nt, self.nx, self.V = nt, nx, nt * nx
        p = N.LatticeParams(nt, nx, m, g, mu, bc_t, bc_x, device)
        h = C.c_void_p()
        N.check(self.lib.tg_create(C.byref(p), C.byref(h)))
        self.h = h

    def close(self):
        if getattr(self, "h", None):
            self.lib.tg_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    # -- state -------------------------------------------------------------
    @property
    def params(self) -> N.LatticeParams:
        p = N.LatticeParams()
        N.check(self.lib.tg_get_params(self.h, C.byref(p)))
        return p

    def set_couplings(self, m, g, mu):
        N.check(self.lib.tg_set_couplings(self.h, m, g, mu))

    def set_gauge(self, A):
        A = _f64(A).reshape(self.nt, self.nx, 2)
        N.check(self.lib.tg_set_gauge(self.h, _p(A)))

    def get_gauge(self, out: np.ndarray | None = None) -> np.ndarray:
        """A as double[nt][nx][2]; into `out` (C-contiguous float64, for example a
        pinned host buffer) when given."""
        if out is None:
            out = np.empty((self.nt, self.nx, 2))
        elif out.dtype != np.float64 or not out.flags.c_contiguous or out.size != 2 * self.nt * self.nx:
            raise ValueError("out must be a C-contiguous float64 array of nt * nx * 2 values")
        N.check(self.lib.tg_get_gauge(self.h, _p(out)))
        return out

    # -- checkpoint and resume ------------------------------------------------
    def checkpoint(self) -> bytes:
        """The lattice's state (couplings, MT stream, Philox counter, A) as bytes."""
        n = self.lib.tg_checkpoint_size(self.h)
        buf = (C.c_ubyte * n)()
        N.check(self.lib.tg_checkpoint_save(self.h, buf, n))
        return bytes(buf)

    def restore(self, data: bytes):
        buf = (C.c_ubyte * len(data)).from_buffer_copy(data)
        N.check(self.lib.tg_checkpoint_load(self.h, buf, len(data)))

    def save(self, path: str):
        with open(path, "wb") as f:
            f.write(self.checkpoint())

    def load(self, path: str):
        with open(path, "rb") as f:
            self.restore(f.read())

    def synchronize(self):
        N.check(self.lib.tg_synchronize(self.h))

    # -- operator (hmc.c:123-249) -------------------------------------------
    def fm_mul(self, v):
        v = _c128(v).reshape(self.nt, self.nx)
        out = np.empty_like(v)
        N.check(self.lib.tg_apply(self.h, _p(v), _p(out), 0))
        return out

    def fm_conjugate_mul(self, v):
        v = _c128(v).reshape(self.nt, self.nx)
        out = np.empty_like(v)
        N.check(self.lib.tg_apply(self.h, _p(v), _p(out), 1))
        return out

    def apply_dev(self, in_ptr: int, out_ptr: int, dagger=False, precision=N.PREC_FP64):
        N.check(self.lib.tg_apply_dev(self.h, C.c_void_p(in_ptr), C.c_void_p(out_ptr), int(dagger), precision))

    def time_apply(self, n: int, dagger=False, precision=N.PREC_FP64) -> float:
        ms = C.c_double()
        N.check(self.lib.tg_time_apply(self.h, n, int(dagger), precision, C.byref(ms)))
        return ms.value

    # -- CG (hmc.c:341-404) -------------------------------------------------
    def fmdm_invert_cg(self, b, cp: N.CgParams | None = None):
        """x = (M^dag M)^-1 b; returns (x, CgResult)."""
        b = _c128(b).reshape(self.nt, self.nx)
        x = np.empty_like(b)
        res = N.CgResult()
        N.check(self.lib.tg_cg(self.h, C.byref(cp or cg_params()), _p(b), _p(x), C.byref(res)), True)
        return x, res

    # -- actions and forces --------------------------------------------------
    def calc_gauge_action(self) -> float:
        s = C.c_double()
        N.check(self.lib.tg_gauge_action(self.h, C.byref(s)))
        return s.value

    def pseudofermion_action(self, phi, cp: N.CgParams | None = None):
        phi = _c128(phi).reshape(self.nt, self.nx)
        s = C.c_double()
        res = N.CgResult()
        N.check(self.lib.tg_pseudofermion_action(self.h, C.byref(cp or cg_params()), _p(phi), C.byref(s),
                                                 C.byref(res)), True)
        return s.value, res

    def stochastic_md_action(self, n) -> float:
        n = _c128(n).reshape(self.nt, self.nx)
        s = C.c_double()
        N.check(self.lib.tg_md_action(self.h, _p(n), C.byref(s)))
        return s.value

    def force(self, chis, noise=None) -> np.ndarray:
        """dS/dA from solved chi_k = (M^dag M)^-1 phi_k (array [npf, nt, nx] or [nt, nx])."""
        chis = _c128(np.asarray(chis).reshape(-1, self.nt, self.nx))
        F = np.empty((self.nt, self.nx, 2))
        nz = _c128(noise) if noise is not None else None
        N.check(self.lib.tg_force(self.h, len(chis), _p(chis), _p(nz) if nz is not None else None, _p(F)))
        return F

    def pf_force(self, phis, cp: N.CgParams | None = None):
        """dS_pf/dA for pseudofermions phis ([npf, nt, nx]); solves afresh.  Returns (F, CgResult)."""
        phis = _c128(np.asarray(phis).reshape(-1, self.nt, self.nx))
        F = np.empty((self.nt, self.nx, 2))
        res = N.CgResult()
        N.check(self.lib.tg_pf_force(self.h, C.byref(cp or cg_params()), len(phis), _p(phis), _p(F), C.byref(res)),
                True)
        return F, res

    def momentum_step(self, mom, phis, noise, eps, cp: N.CgParams | None = None):
        mom = _f64(mom).copy()
        phis = _c128(np.asarray(phis).reshape(-1, self.nt, self.nx))
        nz = _c128(noise) if noise is not None else None
        res = N.CgResult()
        N.check(self.lib.tg_momentum_step(self.h, C.byref(cp or cg_params()), _p(mom), len(phis), _p(phis),
                                          _p(nz) if nz is not None else None, eps, C.byref(res)), True)
        return mom, res

    def gauge_step(self, mom, eps):
        N.check(self.lib.tg_gauge_step(self.h, _p(_f64(mom)), eps))

    # -- measurements (hmc.c:794-842) ----------------------------------------
    def magnetisation(self) -> float:
        v = C.c_double()
        N.check(self.lib.tg_magnetisation(self.h, C.byref(v)))
        return v.value

    def fermion_phase(self, sources: int = 20, noise=None) -> float:
        """hmc.c:794-815; noise [sources, nt, nx] or None (the reference MT stream)."""
        nz = _c128(np.asarray(noise).reshape(sources, self.nt, self.nx)) if noise is not None else None
        v = C.c_double()
        N.check(self.lib.tg_fermion_phase(self.h, sources, _p(nz) if nz is not None else None, C.byref(v)))
        return v.value

    def chiral_condensate(self, sources: int = 16, seed: int = 0, cp: N.CgParams | None = None):
        v, e = C.c_double(), C.c_double()
        N.check(self.lib.tg_chiral_condensate(self.h, C.byref(cp or cg_params(rel_tol=1e-10, abs_tol2=0.0)), sources,
                                              seed, C.byref(v), C.byref(e)))
        return v.value, e.value

    def fm_propagator(self, mask=None, cp: N.CgParams | None = None):
        """calc_Dinv (fermion_matrix.c:189-351): Dinv as double[2, V/2, V/2] in the
        reference's layout, and the CgResult (largest iteration count, worst status)."""
        n = self.V // 2
        out = np.empty((2, n, n))
        res = N.CgResult()
        mp = None
        if mask is not None:
            mask = np.ascontiguousarray(mask, dtype=np.int32).reshape(self.nt, self.nx)
            mp = mask.ctypes.data_as(C.POINTER(C.c_int))
        N.check(self.lib.tg_fm_propagator(self.h, C.byref(cp or cg_params(maxiter=9999)), mp, _p(out),
                                          C.byref(res)), True)
        return out, res

    # -- dense matrix and determinant (hmc.c:269-336) -------------------------
    def fermion_matrix(self) -> np.ndarray:
        out = np.empty((self.V, self.V), np.complex128)
        N.check(self.lib.tg_dense_M(self.h, _p(out)))
        return out

    def log_det(self, A_batch=None):
        """(log|det M|, arg det M) per gauge field of A_batch [n, nt, nx, 2] (None: the current field)."""
        if A_batch is None:
            la, ph = C.c_double(), C.c_double()
            N.check(self.lib.tg_log_det(self.h, 1, None, C.byref(la), C.byref(ph)))
            return la.value, ph.value
        A_batch = _f64(A_batch).reshape(-1, self.nt, self.nx, 2)
        n = len(A_batch)
        la, ph = np.empty(n), np.empty(n)
        N.check(self.lib.tg_log_det(self.h, n, _p(A_batch), _p(la), _p(ph)))
        return la, ph

    # -- fermion-bag operator (vec_ops.c:96-307) ------------------------------
    def fM(self, mask, v, transpose=False) -> np.ndarray:
        mask = np.ascontiguousarray(mask, dtype=np.int32).reshape(self.nt, self.nx)
        v = _f64(v).reshape(self.nt, self.nx)
        out = np.empty_like(v)
        N.check(self.lib.tg_fm_apply(self.h, mask.ctypes.data_as(C.POINTER(C.c_int)), _p(v), _p(out), int(transpose)))
        return out

    def cg_MdM(self, mask, b, cp: N.CgParams | None = None):
        mask = np.ascontiguousarray(mask, dtype=np.int32).reshape(self.nt, self.nx)
        b = _f64(b).reshape(self.nt, self.nx)
        x = np.empty_like(b)
        res = N.CgResult()
        N.check(self.lib.tg_cg_mdm_masked(self.h, C.byref(cp or cg_params(maxiter=10000)),
                                          mask.ctypes.data_as(C.POINTER(C.c_int)), _p(b), _p(x), C.byref(res)), True)
        return x, res

    # -- random numbers and trajectories --------------------------------------
    def seed_mersenne(self, seed: int, warmup: int = 543210):
        N.check(self.lib.tg_mt_seed(self.h, seed, warmup))

    def mersenne(self, n: int) -> np.ndarray:
        out = np.empty(n)
        N.check(self.lib.tg_mt_uniforms(self.h, _p(out), n))
        return out

    def update_puregauge_hb(self, sweeps: int = 1):
        N.check(self.lib.tg_puregauge_sweeps(self.h, sweeps))

    def update_gauge(self, hp: N.HmcParams | None = None) -> N.TrajResult:
        r = N.TrajResult()
        N.check(self.lib.tg_trajectory(self.h, C.byref(hp or hmc_params()), C.byref(r)), True)
        return r

    def trajectory_ext(self, hp: N.HmcParams, eta, mom, noise, u_accept: float) -> N.TrajResult:
        eta = _c128(np.asarray(eta).reshape(-1, self.nt, self.nx))
        mom = _f64(mom)
        nz = _c128(noise) if noise is not None else None
        r = N.TrajResult()
        N.check(self.lib.tg_trajectory_ext(self.h, C.byref(hp), _p(eta), _p(mom), _p(nz) if nz is not None else None,
                                           u_accept, C.byref(r)), True)
        return r


def batch_params(nsteps=10, tau=1.0, stochastic_term=True, use_graph=True, block=0, cg=None) -> N.BatchParams:
    """Settings of a batched trajectory (block = 0: the tuned default)."""
    return N.BatchParams(nsteps, tau, int(stochastic_term), int(use_graph), block, cg or cg_params(rel_tol=1e-10,
                                                                                                  abs_tol2=0.0))


class Batch:
    """Many independent chains advanced together (tg_batch_*).  `chains` is a
    list of dicts with keys nt, nx, m, g, mu, bc_t, bc_x, seed."""

    def __init__(self, chains, device: int = 0):
        self.lib = N.load()
        self.shapes = [(c["nt"], c["nx"]) for c in chains]
        arr = (N.ChainParams * len(chains))(*[
            N.ChainParams(c["nt"], c["nx"], c["m"], c.get("g", 0.5), c.get("mu", 0.0), c.get("bc_t", -1),
                          c.get("bc_x", -1), c.get("seed", 0)) for c in chains])
        h = C.c_void_p()
        N.check(self.lib.tg_batch_create(arr, len(chains), device, C.byref(h)))
        self.h = h
        self.n = len(chains)

    def close(self):
        if getattr(self, "h", None):
            self.lib.tg_batch_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def total_sites(self) -> int:
        n, t = C.c_int(), C.c_longlong()
        N.check(self.lib.tg_batch_size(self.h, C.byref(n), C.byref(t)))
        return t.value

    def set_gauge(self, i: int, A):
        nt, nx = self.shapes[i]
        A = _f64(A).reshape(nt, nx, 2)
        N.check(self.lib.tg_batch_set_gauge(self.h, i, _p(A)))

    def get_gauge(self, i: int) -> np.ndarray:
        nt, nx = self.shapes[i]
        A = np.empty((nt, nx, 2))
        N.check(self.lib.tg_batch_get_gauge(self.h, i, _p(A)))
        return A

    # -- checkpoint and resume ------------------------------------------------
    def checkpoint(self) -> bytes:
        """Every chain's parameters, Philox trajectory counter and field, as bytes."""
        n = self.lib.tg_batch_checkpoint_size(self.h)
        buf = (C.c_ubyte * n)()
        N.check(self.lib.tg_batch_checkpoint_save(self.h, buf, n))
        return bytes(buf)

    def restore(self, data: bytes):
        buf = (C.c_ubyte * len(data)).from_buffer_copy(data)
        N.check(self.lib.tg_batch_checkpoint_load(self.h, buf, len(data)))

    def save(self, path: str):
        with open(path, "wb") as f:
            f.write(self.checkpoint())

    def load(self, path: str):
        with open(path, "rb") as f:
            self.restore(f.read())

    def trajectory(self, bp: N.BatchParams | None = None):
        res = (N.TrajResult * self.n)()
        N.check(self.lib.tg_batch_trajectory(self.h, C.byref(bp or batch_params()), res), True)
        return list(res)

    def autotune(self, bp: N.BatchParams | None = None):
        b, ms = C.c_int(), C.c_double()
        N.check(self.lib.tg_batch_autotune(self.h, C.byref(bp or batch_params()), C.byref(b), C.byref(ms)))
        return b.value, ms.value
