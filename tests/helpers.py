"""Shared helpers of the test suite (fixtures loading, error norms)."""
from __future__ import annotations

import os

import numpy as np

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
# trajectory fixtures whose nx is a multiple of 32 and nt of 4: they run the
# column-march stencil, the path of the large-lattice workloads
MARCH_CONFIGS = ["march_64x64_px", "march_32x96_apx", "march_32x64_mu_px"]
TRAJ_CONFIGS = ["c1_16x16_apx", "c1_16x16_px", "c1s_16x16_px", "mu_8x8_px", "odd_6x4_apx"] + MARCH_CONFIGS
STABLE = {"c1s_16x16_px", "mu_8x8_px", "odd_6x4_apx"} | set(MARCH_CONFIGS)


def golden(name: str) -> dict:
    with np.load(os.path.join(GOLDEN, f"{name}.npz")) as d:
        return {k: d[k] for k in d.files}


def rel(a, b) -> float:
    """|a - b| / |b| in the L2 norm."""
    a, b = np.asarray(a), np.asarray(b)
    return float(np.linalg.norm((a - b).ravel()) / np.linalg.norm(b.ravel()))


def maxrel(a, b) -> float:
    """max |a - b| / max |b| (the force tolerance form)."""
    a, b = np.asarray(a), np.asarray(b)
    return float(np.abs(a - b).max() / np.abs(b).max())


def lat_args(d: dict):
    return (int(d["nt"]), int(d["nx"]), float(d["m"]), float(d["g"]), float(d["mu"]), int(d["bc_t"]), int(d["bc_x"]))


def dH_ok(got: float, want: float, stable: bool) -> bool:
    """dH parity: 1e-9 absolute where the trajectory is stable (|dH| < 10);
    relative 1e-9 on the reference's unstable 10-step 16^2 trajectories, where
    |dH| reaches 1e5 and the last digits are amplified rounding."""
    if stable:
        return abs(got - want) <= 1e-9
    return abs(got - want) <= 1e-9 * max(1.0, abs(want))
