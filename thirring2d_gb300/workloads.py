"""The benchmark workloads as chain descriptors and starting fields.

Each function returns (chains, fields): chain dicts as tg.Batch takes them
(nt, nx, m, g, mu, bc_t, bc_x, seed) and starting gauge fields
float64[nt, nx, 2], seeded so every run builds the same workload.
"""
from __future__ import annotations

import numpy as np

from . import native as N


def mixed_size_chains(n: int, seed: int = 4, side: int = 0):
    """The batched-chain workload: n chains, sides uniform in {16, 24, 32, 48, 64,
    96, 128} (or all `side`), m ~ U[0.05, 0.5], g ~ U[0.2, 1.2], own seeds,
    A ~ N(0, 0.2^2)."""
    rng = np.random.default_rng(seed)
    sides = np.array([side] if side else [16, 24, 32, 48, 64, 96, 128])
    chains, fields = [], []
    for k in range(n):
        L = int(rng.choice(sides))
        chains.append(dict(nt=L, nx=L, m=float(rng.uniform(0.05, 0.5)), g=float(rng.uniform(0.2, 1.2)), mu=0.0,
                           bc_t=N.BC_ANTIPERIODIC, bc_x=N.BC_PERIODIC, seed=int(seed * 100000 + k)))
        fields.append(rng.normal(0, 0.2, (L, L, 2)))
    return chains, fields


# The 16^2 plain-FP64 workload as the reference's hmc.c runs it: periodic x,
# antiperiodic t, m 0.1, g 0.5, A ~ N(0, 0.1^2), 10 leapfrog steps of a
# trajectory of length 1 (hmc.c:708-716 hard-codes both).
C1 = dict(nt=16, nx=16, m=0.1, g=0.5, mu=0.0, bc_t=N.BC_ANTIPERIODIC, bc_x=N.BC_PERIODIC, sigma=0.1, nsteps=10,
          tau=1.0)


def c1_chains(n: int, seed: int = 16):
    """n independent chains of the 16^2 workload, each with its own seed and
    starting field."""
    rng = np.random.default_rng(seed)
    chains = [dict(nt=C1["nt"], nx=C1["nx"], m=C1["m"], g=C1["g"], mu=C1["mu"], bc_t=C1["bc_t"], bc_x=C1["bc_x"],
                   seed=int(seed * 100000 + k)) for k in range(n)]
    fields = [rng.normal(0, C1["sigma"], (C1["nt"], C1["nx"], 2)) for _ in range(n)]
    return chains, fields
