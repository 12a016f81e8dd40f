"""numpy/ctypes front end of the CPU oracle.

TEST INFRASTRUCTURE ONLY: imported by tests/, __graft_entry__.smoke() and the
CPU-baseline leg of bench.py to check the CUDA library; never by the product.

Two back ends:
  * ``Oracle``  -- oracle/liboracle.so, the C restatement in thirring_oracle.c
                   (run-time lattice size, boundary conditions and mu);
  * ``RefHMC``  -- oracle/_ref/libhmcref_T<nt>X<nx>_<variant>.so, the
                   reference hmc.c itself (adjoint corrected), built by
                   oracle/make_ref.py.  Compile-time size, one mu per loaded
                   instance (hmc.c caches exp(+-mu) in statics), so each
                   RefHMC loads a private copy of the library.

Field conventions: A, momenta float64[nt, nx, 2]; fermion vectors
complex128[nt, nx]; t-major like hmc.c.
"""
from __future__ import annotations

import ctypes as C
import os
import shutil
import subprocess
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB = os.path.join(HERE, "liboracle.so")
SRC = os.path.join(HERE, "thirring_oracle.c")

_dp = C.POINTER(C.c_double)
_ip = C.POINTER(C.c_int)


def build() -> str:
    """Compile the C restatement (seconds)."""
    if os.path.exists(LIB) and os.path.getmtime(LIB) >= os.path.getmtime(SRC):
        return LIB
    subprocess.run(["gcc", "-O2", "-std=gnu99", "-fPIC", "-shared", "-o", LIB, SRC, "-lm"], check=True)
    return LIB


class _Lat(C.Structure):
    _fields_ = [("nt", C.c_int), ("nx", C.c_int), ("m", C.c_double), ("g", C.c_double), ("mu", C.c_double),
                ("bc_t", C.c_int), ("bc_x", C.c_int)]


def _ptr(a: np.ndarray, typ=_dp):
    return a.ctypes.data_as(typ)


def _c128(a) -> np.ndarray:
    return np.ascontiguousarray(a, dtype=np.complex128)


def _f64(a) -> np.ndarray:
    return np.ascontiguousarray(a, dtype=np.float64)


_lib = None


def lib():
    global _lib
    if _lib is None:
        build()
        _lib = C.CDLL(LIB)
        _lib.orc_mt_sizeof.restype = C.c_size_t
        _lib.orc_mt_next.restype = C.c_double
        for name in ("orc_gaussian_field", "orc_random_momentum", "orc_gauge_action", "orc_md_action"):
            getattr(_lib, name).restype = C.c_double
    return _lib


class MT:
    """The reference's MT19937 stream (mersenne_inline.c / mersenne.h)."""

    def __init__(self, seed: int, warmup: int = 0):
        self.buf = C.create_string_buffer(int(lib().orc_mt_sizeof()))
        lib().orc_mt_seed(self.buf, C.c_long(seed))
        if warmup:
            self.uniforms(warmup)

    def next(self) -> float:
        return lib().orc_mt_next(self.buf)

    def uniforms(self, n: int) -> np.ndarray:
        out = np.empty(n, np.float64)
        lib().orc_mt_fill(self.buf, _ptr(out), C.c_long(n))
        return out

    def gaussian_field(self, nt: int, nx: int):
        v = np.empty((nt, nx), np.complex128)
        s = lib().orc_gaussian_field(self.buf, nt * nx, _ptr(v))
        return v, s

    def momentum(self, nt: int, nx: int):
        p = np.empty((nt, nx, 2), np.float64)
        s = lib().orc_random_momentum(self.buf, nt * nx, _ptr(p))
        return p, s


class Oracle:
    """C restatement of the hmc.c hot path on one lattice."""

    def __init__(self, nt: int, nx: int, m: float, g: float = 0.5, mu: float = 0.0, bc_t: int = -1, bc_x: int = -1):
        self.nt, self.nx = nt, nx
        self.lat = _Lat(nt, nx, m, g, mu, bc_t, bc_x)
        self.V = nt * nx
        self.L = lib()

    def apply(self, A, psi, dagger: bool = False) -> np.ndarray:
        A, psi = _f64(A), _c128(psi)
        out = np.empty_like(psi)
        self.L.orc_apply(C.byref(self.lat), _ptr(A), _ptr(psi), _ptr(out), int(dagger))
        return out

    def M(self, A, psi):
        return self.apply(A, psi, False)

    def Mdag(self, A, psi):
        return self.apply(A, psi, True)

    def dense_M(self, A) -> np.ndarray:
        out = np.empty((self.V, self.V), np.complex128)
        self.L.orc_dense_M(C.byref(self.lat), _ptr(_f64(A)), _ptr(out))
        return out

    def cg(self, A, b, rel_tol: float = 0.0, abs_tol2: float = 1e-30, maxiter: int = 100000):
        A, b = _f64(A), _c128(b)
        x = np.empty_like(b)
        it = C.c_int(0)
        rr = C.c_double(0)
        st = self.L.orc_cg(C.byref(self.lat), _ptr(A), _ptr(b), _ptr(x), C.c_double(abs_tol2), C.c_double(rel_tol),
                           maxiter, C.byref(it), C.byref(rr))
        return x, st, it.value

    def gauge_action(self, A) -> float:
        return self.L.orc_gauge_action(C.byref(self.lat), _ptr(_f64(A)))

    def md_action(self, A, n) -> float:
        return self.L.orc_md_action(C.byref(self.lat), _ptr(_f64(A)), _ptr(_c128(n)))

    def force(self, A, chis, noise=None) -> np.ndarray:
        """dS/dA (gauge + pseudofermion + stochastic term) for solved chi_k = (M^dag M)^-1 phi_k."""
        A = _f64(A)
        chis = _c128(np.asarray(chis).reshape(-1, self.nt, self.nx))
        Mchis = _c128(np.stack([self.M(A, c) for c in chis]))
        F = np.empty((self.nt, self.nx, 2), np.float64)
        nz = _c128(noise) if noise is not None else None
        self.L.orc_total_force(C.byref(self.lat), _ptr(A), len(chis), _ptr(chis), _ptr(Mchis),
                               _ptr(nz) if nz is not None else None, _ptr(F))
        return F

    def pf_force(self, A, chis) -> np.ndarray:
        """dS_pf/dA alone for solved chi_k (hmc.c:517-576)."""
        A = _f64(A)
        chis = _c128(np.asarray(chis).reshape(-1, self.nt, self.nx))
        F = np.zeros((self.nt, self.nx, 2), np.float64)
        for c in chis:
            Mc = self.M(A, c)
            self.L.orc_pf_force(C.byref(self.lat), _ptr(A), _ptr(_c128(c)), _ptr(Mc), _ptr(F))
        return F

    def momentum_step(self, A, p, phis, noise, eps, rel_tol=0.0, abs_tol2=1e-30, maxiter=100000):
        A = _f64(A)
        p = _f64(p).copy()
        phis = _c128(np.asarray(phis).reshape(-1, self.nt, self.nx))
        nz = _c128(noise) if noise is not None else None
        it = C.c_int(0)
        st = self.L.orc_momentum_step(C.byref(self.lat), _ptr(A), _ptr(p), len(phis), _ptr(phis),
                                      _ptr(nz) if nz is not None else None, C.c_double(eps), C.c_double(abs_tol2),
                                      C.c_double(rel_tol), maxiter, C.byref(it))
        return p, st, it.value

    def trajectory(self, A, mt: MT, nsteps=10, tau=1.0, npf=1, use_noise=True, rel_tol=0.0, abs_tol2=1e-30,
                   maxiter=100000):
        """One HMC trajectory (hmc.c:671-746); A is updated in place on acceptance."""
        assert A.dtype == np.float64 and A.flags.c_contiguous
        stats = np.empty(10, np.float64)
        it = C.c_int(0)
        st = self.L.orc_trajectory(C.byref(self.lat), _ptr(A), mt.buf, nsteps, C.c_double(tau), npf, int(use_noise),
                                   C.c_double(abs_tol2), C.c_double(rel_tol), maxiter, _ptr(stats), C.byref(it))
        return stats, st, it.value

    def puregauge_sweep(self, A, mt: MT):
        assert A.dtype == np.float64 and A.flags.c_contiguous
        self.L.orc_puregauge_sweep(C.byref(self.lat), _ptr(A), mt.buf)

    def fM(self, mask, v, transpose=False):
        mask = np.ascontiguousarray(mask, dtype=np.int32)
        v = _f64(v)
        out = np.empty_like(v)
        self.L.orc_fM(C.byref(self.lat), _ptr(mask, _ip), _ptr(v), _ptr(out), int(transpose))
        return out

    def fm_propagator(self, mask=None, abs_tol2=1e-30, maxiter=9999):
        """calc_Dinv (fermion_matrix.c:189-351) restated: for every source the column
        fM^-1 e_src by cg_propagator (vec_ops.c:311-321), the entries on the other
        parity in the reference's layout double[2, V/2, V/2] (i = (nx*t + x)/2):
        [0] odd sources / even sites, [1] even sources / odd sites."""
        nt, nx, V = self.nt, self.nx, self.nt * self.nx
        mask = np.zeros((nt, nx), np.int32) if mask is None else mask
        n = V // 2
        out = np.zeros((2, n, n))
        for src in range(V):
            e = np.zeros(V)
            e[src] = 1.0
            b = self.fM(mask, e.reshape(nt, nx), True)
            x, st, _ = self.cg_MdM(mask, b, abs_tol2=abs_tol2, maxiter=maxiter)
            if st == 2:
                x = np.full_like(x, 1e50)
            ts, xs = divmod(src, nx)
            par = (ts + xs) & 1
            blk = out[0 if par else 1]
            for s in range(V):
                t, xx = divmod(s, nx)
                if ((t + xx) & 1) != par:
                    blk[s // 2, src // 2] = x.ravel()[s]
        return out

    def cg_MdM(self, mask, b, rel_tol=0.0, abs_tol2=1e-30, maxiter=100000):
        mask = np.ascontiguousarray(mask, dtype=np.int32)
        b = _f64(b)
        x = np.empty_like(b)
        it = C.c_int(0)
        st = self.L.orc_cg_MdM(C.byref(self.lat), _ptr(mask, _ip), _ptr(b), _ptr(x), C.c_double(abs_tol2),
                               C.c_double(rel_tol), maxiter, C.byref(it))
        return x, st, it.value


# ---------------------------------------------------------------------------
# The reference hmc.c itself (oracle/_ref), when it has been built.
# ---------------------------------------------------------------------------
REF_DIR = os.path.join(HERE, "_ref")


def ref_lib_path(nt: int, nx: int, variant: str = "fixed_apx") -> str:
    return os.path.join(REF_DIR, f"libhmcref_T{nt}X{nx}_{variant}.so")


def ref_available(nt: int, nx: int, variant: str = "fixed_apx") -> bool:
    return os.path.exists(ref_lib_path(nt, nx, variant))


class RefHMC:
    """A private instance of the reference hmc.c (adjoint-corrected build)."""

    def __init__(self, nt, nx, m, g, mu=0.0, seed=12345, warmup=543210, variant="fixed_apx"):
        src = ref_lib_path(nt, nx, variant)
        if not os.path.exists(src):
            raise FileNotFoundError(f"{src} not built (python oracle/make_ref.py {nt}x{nx})")
        self._tmp = tempfile.mkdtemp(prefix="hmcref_")
        path = os.path.join(self._tmp, os.path.basename(src))
        shutil.copy(src, path)
        self.L = C.CDLL(path)
        for name in ("ref_mersenne", "ref_gauge_action", "ref_pseudofermion_action", "ref_md_action",
                     "ref_random_pseudofermion", "ref_random_momentum"):
            getattr(self.L, name).restype = C.c_double
        self.nt, self.nx = nt, nx
        self.L.ref_setup(C.c_double(m), C.c_double(g), C.c_double(mu), C.c_long(seed), warmup)

    def __del__(self):
        shutil.rmtree(getattr(self, "_tmp", ""), ignore_errors=True)

    def set_A(self, A):
        self.L.ref_set_A(_ptr(_f64(A)))

    def get_A(self):
        A = np.empty((self.nt, self.nx, 2))
        self.L.ref_get_A(_ptr(A))
        return A

    def uniforms(self, n):
        out = np.empty(n)
        self.L.ref_mersenne_fill(_ptr(out), C.c_long(n))
        return out

    def puregauge(self, sweeps):
        self.L.ref_puregauge(sweeps)

    def M(self, psi):
        psi = _c128(psi)
        out = np.empty_like(psi)
        self.L.ref_fm_mul(_ptr(psi), _ptr(out))
        return out

    def Mdag(self, psi):
        psi = _c128(psi)
        out = np.empty_like(psi)
        self.L.ref_fm_conjugate_mul(_ptr(psi), _ptr(out))
        return out

    def cg(self, b):
        b = _c128(b)
        x = np.empty_like(b)
        self.L.ref_cg(_ptr(b), _ptr(x))
        return x

    def gauge_action(self):
        return self.L.ref_gauge_action()

    def pseudofermion_action(self, phi):
        return self.L.ref_pseudofermion_action(_ptr(_c128(phi)))

    def md_action(self, n):
        return self.L.ref_md_action(_ptr(_c128(n)))

    def momentum_step(self, p, psi, st, eps):
        p = _f64(p).copy()
        self.L.ref_momentum_step(_ptr(p), _ptr(_c128(psi)), _ptr(_c128(st)), C.c_double(eps))
        return p

    def trajectory(self, nsteps=10, tau=1.0):
        stats = np.empty(10)
        self.L.ref_trajectory(nsteps, C.c_double(tau), _ptr(stats))
        return stats

    def update_gauge(self):
        """The reference's own update_gauge(A) (hmc.c:671-746; prints to stdout)."""
        self.L.ref_update_gauge()


def _ref_dense(self):
    """hmc.c fermion_matrix as a row-major complex [V, V] array (M psi = Md @ psi)."""
    V = self.nt * self.nx
    out = np.empty(V * V, np.complex128)
    self.L.ref_fermion_matrix(_ptr(out))
    return out.reshape(V, V).T.copy()  # the reference stores element (i, j) at i + j*V


RefHMC.dense_M = _ref_dense


def vec_ref_lib_path(nt: int, nx: int, prop: bool = False) -> str:
    return os.path.join(REF_DIR, f"libpropref_T{nt}X{nx}.so" if prop else f"libvecopsref_T{nt}X{nx}.so")


class RefVecOps:
    """A private instance of the reference's vec_ops.c (fM, fM_transpose,
    cg_MdM of the fermion-bag programs; ANTISYMMETRIC build).  prop=True loads
    the build with fermion_matrix.c's calc_Dinv (PROPAGATOR_MATRIX,
    WITH_MASS_MONOMERS)."""

    def __init__(self, nt, nx, m, mu=0.0, prop=False):
        src = vec_ref_lib_path(nt, nx, prop)
        if not os.path.exists(src):
            raise FileNotFoundError(f"{src} not built (python oracle/make_ref.py)")
        self._tmp = tempfile.mkdtemp(prefix="vecref_")
        path = os.path.join(self._tmp, os.path.basename(src))
        shutil.copy(src, path)
        self.L = C.CDLL(path)
        self.nt, self.nx = nt, nx
        self.L.vref_setup(C.c_double(m), C.c_double(mu))

    def __del__(self):
        shutil.rmtree(getattr(self, "_tmp", ""), ignore_errors=True)

    def set_field(self, mask):
        self.L.vref_set_field(_ptr(np.ascontiguousarray(mask, dtype=np.int32), _ip))

    def fM(self, v, transpose=False):
        v = _f64(v)
        out = np.empty_like(v)
        self.L.vref_fM(_ptr(v), _ptr(out), int(transpose))
        return out

    def cg_MdM(self, b):
        b = _f64(b)
        x = np.empty_like(b)
        self.L.vref_cg_MdM(_ptr(b), _ptr(x))
        return x

    def calc_Dinv(self):
        """The reference's propagator matrix for the current field, double[2, V/2, V/2]
        (calc_Dinv caches it in a file of the working directory: run in an empty one)."""
        n = self.nt * self.nx // 2
        out = np.empty((2, n, n))
        cwd = os.getcwd()
        work = tempfile.mkdtemp(prefix="dinv_", dir=self._tmp)
        try:
            os.chdir(work)
            self.L.vref_calc_Dinv(_ptr(out))
        finally:
            os.chdir(cwd)
        return out


# ---------------------------------------------------------------------------
# The reference's determinant code (oracle/_ref), when it has been built.
# ---------------------------------------------------------------------------
class RefFullDet:
    """A private instance of the reference's full_determinant.c determinant_mu
    (full_determinant.c:144-186) over fermion_matrix.c's fM_index with the mass
    on the diagonal, on 4 x 4 (antisymmetric boundaries, or open x)."""

    def __init__(self, nt, nx, m, mu, openx):
        from oracle import make_ref
        src = make_ref.det_lib_path(nt, nx, openx)
        if not os.path.exists(src):
            raise FileNotFoundError(f"{src} not built (python oracle/make_ref.py)")
        self._tmp = tempfile.mkdtemp(prefix="detref_")
        path = os.path.join(self._tmp, os.path.basename(src))
        shutil.copy(src, path)
        self.L = C.CDLL(path)
        self.L.dref_determinant_mu.restype = C.c_double
        self.nt, self.nx, self.mu = nt, nx, mu
        self.L.dref_setup(C.c_double(m), C.c_double(mu))

    def __del__(self):
        shutil.rmtree(getattr(self, "_tmp", ""), ignore_errors=True)

    def determinant(self, mask=None):
        """det of fM_index over the sites with mask == 0 (all sites by default)."""
        mask = np.zeros((self.nt, self.nx), np.int32) if mask is None else mask
        self.L.dref_set_field(_ptr(np.ascontiguousarray(mask, dtype=np.int32), _ip))
        return self.L.dref_determinant_mu(C.c_double(self.mu))


def ref_brute(mu: float, m: float = 0.0, U: float = 1.0, seed: int = 54357345) -> dict:
    """Run the reference's brute-force enumeration (tests/thirring_brute.c, 4 x 4,
    open x) and parse its table: arrays [links, monomers] of the sums of det,
    |det|, det*charge, det*chiralcharge and det*chiralsusc."""
    import re
    from oracle import make_ref
    exe = make_ref.brute_path()
    if not os.path.exists(exe):
        raise FileNotFoundError(f"{exe} not built (python oracle/make_ref.py)")
    work = tempfile.mkdtemp(prefix="brute_")
    try:
        r = subprocess.run([exe], input=f"1000000\n1\n100\n{float(m)!r}\n{float(U)!r}\n{float(mu)!r}\n{int(seed)}\n",
                           text=True, capture_output=True, cwd=work, timeout=3600)
    finally:
        shutil.rmtree(work, ignore_errors=True)
    if f" mu {float(mu):f} " not in r.stdout:
        raise RuntimeError("brute-force run did not read mu: " + r.stdout[:500])
    rows = re.findall(r"Links (\d+) Monomers (\d+) det (\S+) abs\(det\) (\S+) det\*charge (\S+) "
                      r"det\*chiralcharge (\S+) det\*chiralsusc (\S+)", r.stdout)
    if not rows or "simulation done" not in r.stdout:
        raise RuntimeError("brute-force run failed: " + r.stdout[-500:] + r.stderr[-500:])
    nl = max(int(x[0]) for x in rows) + 1
    nm = max(int(x[1]) for x in rows) + 1
    out = {k: np.zeros((nl, nm)) for k in ("det", "absdet", "charge", "chiralcharge", "chiralsusc")}
    for row in rows:
        i, j = int(row[0]), int(row[1])
        for k, v in zip(("det", "absdet", "charge", "chiralcharge", "chiralsusc"), row[2:]):
            out[k][i, j] = float(v)
    return out
