"""ctypes binding of libthirring_gpu.so (include/thirring_gpu.h).

The library is loaded from the package directory only.  A missing or
unloadable library raises immediately: there is no CPU fallback.
"""
from __future__ import annotations

import ctypes as C
import os

PKG = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(PKG, "libthirring_gpu.so")

TG_OK, TG_E_NOCONV, TG_E_DIVERGED, TG_E_NAN, TG_E_CUDA, TG_E_ARG, TG_E_ALLOC, TG_E_TIMEOUT = range(8)
STATUS_NAMES = {0: "OK", 1: "NOCONV", 2: "DIVERGED", 3: "NAN", 4: "CUDA", 5: "ARG", 6: "ALLOC", 7: "TIMEOUT"}
SOLVER_DEFAULT, SOLVER_LAUNCHES, SOLVER_PERSISTENT = 0, 1, 2
BC_PERIODIC, BC_ANTIPERIODIC, BC_OPEN = 1, -1, 0
PREC_FP64, PREC_MIXED = 0, 1
RNG_MT, RNG_PHILOX, RNG_EXTERNAL = 0, 1, 2


class LatticeParams(C.Structure):
    _fields_ = [("nt", C.c_int), ("nx", C.c_int), ("m", C.c_double), ("g", C.c_double), ("mu", C.c_double),
                ("bc_t", C.c_int), ("bc_x", C.c_int), ("device", C.c_int)]


class CgParams(C.Structure):
    _fields_ = [("rel_tol", C.c_double), ("abs_tol2", C.c_double), ("maxiter", C.c_int), ("precision", C.c_int),
                ("ru_interval", C.c_int), ("solver", C.c_int)]


class CgResult(C.Structure):
    _fields_ = [("iterations", C.c_int), ("status", C.c_int), ("reliable_updates", C.c_int), ("pad_", C.c_int),
                ("rr", C.c_double), ("rr0", C.c_double)]


class HmcParams(C.Structure):
    _fields_ = [("nsteps", C.c_int), ("tau", C.c_double), ("npf", C.c_int), ("stochastic_term", C.c_int),
                ("rng", C.c_int), ("use_graph", C.c_int), ("seed", C.c_ulonglong), ("cg", CgParams)]


class TrajResult(C.Structure):
    _fields_ = [("dH", C.c_double), ("Sg0", C.c_double), ("Spf0", C.c_double), ("Smd0", C.c_double),
                ("Smom0", C.c_double), ("Sg1", C.c_double), ("Spf1", C.c_double), ("Smd1", C.c_double),
                ("Smom1", C.c_double), ("u_accept", C.c_double), ("accepted", C.c_int), ("status", C.c_int),
                ("cg_solves", C.c_int), ("cg_iterations", C.c_int), ("cg_max_iterations", C.c_int),
                ("reliable_updates", C.c_int), ("cg_ms", C.c_double)]

    def as_dict(self) -> dict:
        return {k: getattr(self, k) for k, _ in self._fields_}


class ChainParams(C.Structure):
    _fields_ = [("nt", C.c_int), ("nx", C.c_int), ("m", C.c_double), ("g", C.c_double), ("mu", C.c_double),
                ("bc_t", C.c_int), ("bc_x", C.c_int), ("seed", C.c_ulonglong)]


class BatchParams(C.Structure):
    _fields_ = [("nsteps", C.c_int), ("tau", C.c_double), ("stochastic_term", C.c_int), ("use_graph", C.c_int),
                ("block", C.c_int), ("cg", CgParams)]


class TGError(RuntimeError):
    def __init__(self, code: int, msg: str):
        super().__init__(f"thirring_gpu error {STATUS_NAMES.get(code, code)}: {msg}")
        self.code = code


_vp = C.c_void_p
_dp = C.POINTER(C.c_double)

# name -> (restype, argtypes)
SIGNATURES = {
    "tg_last_error": (C.c_char_p, []),
    "tg_version": (C.c_char_p, []),
    "tg_create": (C.c_int, [C.POINTER(LatticeParams), C.POINTER(_vp)]),
    "tg_destroy": (C.c_int, [_vp]),
    "tg_set_couplings": (C.c_int, [_vp, C.c_double, C.c_double, C.c_double]),
    "tg_get_params": (C.c_int, [_vp, C.POINTER(LatticeParams)]),
    "tg_synchronize": (C.c_int, [_vp]),
    "tg_stream": (_vp, [_vp]),
    "tg_set_gauge": (C.c_int, [_vp, _dp]),
    "tg_get_gauge": (C.c_int, [_vp, _dp]),
    "tg_set_gauge_dev": (C.c_int, [_vp, _vp]),
    "tg_apply": (C.c_int, [_vp, _dp, _dp, C.c_int]),
    "tg_apply_dev": (C.c_int, [_vp, _vp, _vp, C.c_int, C.c_int]),
    "tg_time_apply": (C.c_int, [_vp, C.c_int, C.c_int, C.c_int, _dp]),
    "tg_cg": (C.c_int, [_vp, C.POINTER(CgParams), _dp, _dp, C.POINTER(CgResult)]),
    "tg_cg_dev": (C.c_int, [_vp, C.POINTER(CgParams), _vp, _vp, C.POINTER(CgResult)]),
    "tg_gauge_action": (C.c_int, [_vp, _dp]),
    "tg_pseudofermion_action": (C.c_int, [_vp, C.POINTER(CgParams), _dp, _dp, C.POINTER(CgResult)]),
    "tg_md_action": (C.c_int, [_vp, _dp, _dp]),
    "tg_force": (C.c_int, [_vp, C.c_int, _dp, _dp, _dp]),
    "tg_momentum_step": (C.c_int, [_vp, C.POINTER(CgParams), _dp, C.c_int, _dp, _dp, C.c_double,
                                   C.POINTER(CgResult)]),
    "tg_gauge_step": (C.c_int, [_vp, _dp, C.c_double]),
    "tg_pf_force": (C.c_int, [_vp, C.POINTER(CgParams), C.c_int, _dp, _dp, C.POINTER(CgResult)]),
    "tg_mt_seed": (C.c_int, [_vp, C.c_long, C.c_long]),
    "tg_mt_uniforms": (C.c_int, [_vp, _dp, C.c_long]),
    "tg_puregauge_sweeps": (C.c_int, [_vp, C.c_int]),
    "tg_puregauge_ext": (C.c_int, [_vp, _dp, C.c_int]),
    "tg_trajectory": (C.c_int, [_vp, C.POINTER(HmcParams), C.POINTER(TrajResult)]),
    "tg_trajectory_ext": (C.c_int, [_vp, C.POINTER(HmcParams), _dp, _dp, _dp, C.c_double, C.POINTER(TrajResult)]),
    "tg_magnetisation": (C.c_int, [_vp, _dp]),
    "tg_fermion_phase": (C.c_int, [_vp, C.c_int, _dp, _dp]),
    "tg_chiral_condensate": (C.c_int, [_vp, C.POINTER(CgParams), C.c_int, C.c_ulonglong, _dp, _dp]),
    "tg_batch_checkpoint_size": (C.c_size_t, [_vp]),
    "tg_batch_checkpoint_save": (C.c_int, [_vp, _vp, C.c_size_t]),
    "tg_batch_checkpoint_load": (C.c_int, [_vp, _vp, C.c_size_t]),
    "tg_checkpoint_size": (C.c_size_t, [_vp]),
    "tg_checkpoint_save": (C.c_int, [_vp, _vp, C.c_size_t]),
    "tg_checkpoint_load": (C.c_int, [_vp, _vp, C.c_size_t]),
    "tg_grid_barrier_check": (C.c_int, [C.c_int, C.c_int, C.POINTER(C.c_int)]),
    "tg_measure_fp64_peak": (C.c_int, [C.c_int, _dp]),
    "tg_stage_faults": (C.c_int, [C.c_int, C.POINTER(C.c_uint)]),
    "tg_fm_propagator": (C.c_int, [_vp, C.POINTER(CgParams), C.POINTER(C.c_int), _dp, C.POINTER(CgResult)]),
    "tg_dense_M": (C.c_int, [_vp, _dp]),
    "tg_log_det": (C.c_int, [_vp, C.c_int, _dp, _dp, _dp]),
    "tg_fm_apply": (C.c_int, [_vp, C.POINTER(C.c_int), _dp, _dp, C.c_int]),
    "tg_cg_mdm_masked": (C.c_int, [_vp, C.POINTER(CgParams), C.POINTER(C.c_int), _dp, _dp, C.POINTER(CgResult)]),
    "tg_cg_noalloc": (C.c_int, [C.POINTER(LatticeParams), C.POINTER(CgParams), _vp, _vp, _vp, C.POINTER(CgResult),
                                _vp]),
    "tg_batch_create": (C.c_int, [C.POINTER(ChainParams), C.c_int, C.c_int, C.POINTER(_vp)]),
    "tg_batch_destroy": (C.c_int, [_vp]),
    "tg_batch_size": (C.c_int, [_vp, C.POINTER(C.c_int), C.POINTER(C.c_longlong)]),
    "tg_batch_set_gauge": (C.c_int, [_vp, C.c_int, _dp]),
    "tg_batch_get_gauge": (C.c_int, [_vp, C.c_int, _dp]),
    "tg_batch_trajectory": (C.c_int, [_vp, C.POINTER(BatchParams), C.POINTER(TrajResult)]),
    "tg_batch_autotune": (C.c_int, [_vp, C.POINTER(BatchParams), C.POINTER(C.c_int), _dp]),
}

_lib = None


def load(path: str = LIB_PATH):
    """Load the CUDA library (raises if it has not been built)."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(path):
        raise ImportError(f"{path} not found: build it with `python -c 'import __graft_entry__ as g; g.build()'`")
    lib = C.CDLL(path)
    for name, (res, args) in SIGNATURES.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    _lib = lib
    return lib


SOLVER_STATUSES = (TG_E_NOCONV, TG_E_DIVERGED, TG_E_NAN)


def check(rc: int, allow_solver_status: bool = False) -> int:
    """Raise TGError for a failed call.  With allow_solver_status, a solve that
    ran but did not converge returns its status instead (outputs are valid)."""
    if rc == TG_OK or (allow_solver_status and rc in SOLVER_STATUSES):
        return rc
    msg = load().tg_last_error()
    raise TGError(rc, msg.decode() if msg else "")


def fp64_peak_tflops(device: int = 0) -> float:
    """Measured FP64 FMA throughput of the GPU (TFLOP/s, tg_measure_fp64_peak)."""
    v = C.c_double()
    check(load().tg_measure_fp64_peak(device, C.byref(v)))
    return v.value


def stage_faults(device: int = 0) -> int:
    """Staged-kernel waits that ran out (tg_stage_faults); 0 in a healthy run."""
    v = C.c_uint()
    check(load().tg_stage_faults(device, C.byref(v)))
    return v.value
