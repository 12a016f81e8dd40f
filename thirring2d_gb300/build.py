"""Build recipe of the native parts (in-tree, no cmake).

  libthirring_gpu.so   csrc/*.cu for sm_103a (nvcc), the C ABI of include/thirring_gpu.h
  libthirring_hmc.so   csrc/hmc_compat.c (gcc), the reference-signature layer of
                       include/thirring_hmc.h, linked against libthirring_gpu.so
  bin/hmc              csrc/hmc_main.c, the drop-in for the reference's `hmc` program

Objects go to thirring2d_gb300/_build/ and are rebuilt only when a source, a
header or the flags change.  Translation units compile in parallel.
"""
from __future__ import annotations

import glob
import hashlib
import os
import subprocess
from concurrent.futures import ThreadPoolExecutor

PKG = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG)
CSRC = os.path.join(PKG, "csrc")
INCLUDE = os.path.join(ROOT, "include")
BUILD = os.path.join(PKG, "_build")
LIB_GPU = os.path.join(PKG, "libthirring_gpu.so")
LIB_HMC = os.path.join(PKG, "libthirring_hmc.so")
BIN_DIR = os.path.join(ROOT, "bin")
HMC_BIN = os.path.join(BIN_DIR, "hmc")

NVCC = os.environ.get("NVCC", "nvcc")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ARCH + ["-lineinfo", "-O3", "-std=c++17", "-Xcompiler", "-fPIC", f"-I{INCLUDE}"]
CC_FLAGS = ["-O2", "-std=gnu99", "-fPIC", "-Wall", "-Wextra", f"-I{INCLUDE}"]


def _digest(paths, flags) -> str:
    h = hashlib.sha256(" ".join(flags).encode())
    for p in sorted(paths):
        with open(p, "rb") as f:
            h.update(f.read())
    return h.hexdigest()


def _headers():
    return glob.glob(os.path.join(CSRC, "*.h")) + glob.glob(os.path.join(CSRC, "*.cuh")) + \
        glob.glob(os.path.join(INCLUDE, "*.h"))


def _stale(target: str, digest: str) -> bool:
    stamp = target + ".sha"
    if not os.path.exists(target) or not os.path.exists(stamp):
        return True
    with open(stamp) as f:
        return f.read().strip() != digest


def _stamp(target: str, digest: str):
    with open(target + ".sha", "w") as f:
        f.write(digest)


def _run(cmd):
    r = subprocess.run(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"build failed: {' '.join(cmd)}\n{r.stdout}")
    return r.stdout


def _compile_cu(src: str) -> str:
    obj = os.path.join(BUILD, os.path.basename(src) + ".o")
    d = _digest([src] + _headers(), [NVCC] + NVCC_FLAGS)
    if _stale(obj, d):
        _run([NVCC] + NVCC_FLAGS + ["-c", src, "-o", obj])
        _stamp(obj, d)
    return obj


def build(verbose: bool = False) -> dict:
    os.makedirs(BUILD, exist_ok=True)
    os.makedirs(BIN_DIR, exist_ok=True)
    cu = sorted(glob.glob(os.path.join(CSRC, "*.cu")))
    with ThreadPoolExecutor(max_workers=max(2, min(len(cu), os.cpu_count() or 2))) as ex:
        objs = list(ex.map(_compile_cu, cu))
    d = _digest(objs, ["link-gpu"])
    if _stale(LIB_GPU, d):
        _run([NVCC] + ARCH + ["-shared", "-o", LIB_GPU] + objs)
        _stamp(LIB_GPU, d)
    compat = os.path.join(CSRC, "hmc_compat.c")
    main = os.path.join(CSRC, "hmc_main.c")
    if os.path.exists(compat):
        d = _digest([compat, LIB_GPU] + _headers(), CC_FLAGS)
        if _stale(LIB_HMC, d):
            _run(["gcc"] + CC_FLAGS + ["-shared", "-o", LIB_HMC, compat, f"-L{PKG}", "-lthirring_gpu",
                                       "-Wl,-rpath,$ORIGIN", "-lm"])
            _stamp(LIB_HMC, d)
    if os.path.exists(main):
        d = _digest([main, LIB_HMC] + _headers(), CC_FLAGS)
        if _stale(HMC_BIN, d):
            _run(["gcc"] + CC_FLAGS + ["-o", HMC_BIN, main, f"-L{PKG}", "-lthirring_hmc", "-lthirring_gpu",
                                       "-Wl,-rpath,$ORIGIN/../thirring2d_gb300", "-lm"])
            _stamp(HMC_BIN, d)
    return {"libthirring_gpu": LIB_GPU, "libthirring_hmc": LIB_HMC, "hmc": HMC_BIN}


if __name__ == "__main__":
    for k, v in build().items():
        print(k, v)
