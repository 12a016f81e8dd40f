"""Generate tests/golden/*.npz from the reference hmc.c itself.

Run from the repository root where the reference tree is available:

    python oracle/make_ref.py && python tests/golden/make_golden.py

Each fixture is produced by the adjoint-corrected build of the reference's own
hmc.c + mersenne_inline.c (oracle/_ref, see oracle/make_ref.py), driven
in-process through oracle/ref_driver.c.  The reference ships no golden vectors
or known-answer tests, so these outputs ARE the pins: the CPU oracle is checked
against them without a GPU, and the CUDA library on the GPU.
"""
from __future__ import annotations

import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)

from oracle import make_ref  # noqa: E402
from oracle.oracle import RefHMC  # noqa: E402

OUT = os.path.dirname(os.path.abspath(__file__))

# name: (nt, nx, m, g, mu, variant, sigma_A, seed, puregauge sweeps, trajectories, nsteps)
CONFIGS = {
    # the 16^2 workload (m 0.1, g 0.5, 10 steps), reference boundary conditions (x antiperiodic)
    "c1_16x16_apx": (16, 16, 0.1, 0.5, 0.0, "fixed_apx", 0.1, 12345, 10, 3, 10),
    # the 16^2 workload with a periodic x direction
    "c1_16x16_px": (16, 16, 0.1, 0.5, 0.0, "fixed_px", 0.1, 4242, 10, 3, 10),
    # the same with a stable step size (40 steps): |dH| < 1, so dH is pinned absolutely
    "c1s_16x16_px": (16, 16, 0.1, 0.5, 0.0, "fixed_px", 0.1, 2024, 10, 3, 40),
    # chemical potential on: exercises e^{+-mu} and the stochastic-term force
    "mu_8x8_px": (8, 8, 0.3, 0.8, 0.3, "fixed_px", 0.3, 777, 5, 3, 10),
    # odd shape, mu on, reference BCs
    "odd_6x4_apx": (6, 4, 0.5, 1.0, 0.2, "fixed_apx", 0.5, 99, 5, 3, 8),
    # column-march shapes (nx a multiple of 32, nt of 4), stable step sizes (|dH| < 1):
    # the stencil path of the large-lattice workloads, against the reference
    "march_64x64_px": (64, 64, 0.1, 0.5, 0.0, "fixed_px", 0.3, 6464, 10, 3, 80),
    "march_32x96_apx": (32, 96, 0.2, 0.5, 0.0, "fixed_apx", 0.3, 3296, 10, 3, 40),
    "march_32x64_mu_px": (32, 64, 0.2, 0.6, 0.2, "fixed_px", 0.3, 3264, 10, 3, 40),
}

MT_SEEDS = [12345, 4354365264, -7]


def make_config(name, nt, nx, m, g, mu, variant, sigma, seed, sweeps, ntraj, nsteps):
    rng = np.random.default_rng(abs(seed) + 1)
    A = rng.normal(0.0, sigma, (nt, nx, 2))
    psi = rng.normal(size=(nt, nx)) + 1j * rng.normal(size=(nt, nx))
    noise = rng.normal(size=(nt, nx)) + 1j * rng.normal(size=(nt, nx))
    mom0 = rng.normal(size=(nt, nx, 2))
    ref = RefHMC(nt, nx, m, g, mu, seed=seed, warmup=543210, variant=variant)
    ref.set_A(A)
    out = dict(nt=nt, nx=nx, m=m, g=g, mu=mu, bc_x=(1 if variant.endswith("_px") else -1), bc_t=-1,
               A=A, psi=psi, noise=noise, mom0=mom0)
    out["M_psi"] = ref.M(psi)
    out["Mdag_psi"] = ref.Mdag(psi)
    out["cg_x"] = ref.cg(psi)
    out["S_gauge"] = ref.gauge_action()
    out["S_pf"] = ref.pseudofermion_action(psi)
    out["S_md"] = ref.md_action(noise)
    out["mom_step"] = ref.momentum_step(mom0, psi, noise, 0.1)
    # trajectory sequence from the reference's own set-up: seed, 543210
    # warm-up draws, A = 0, pure-gauge sweeps, then update_gauge's sequence
    tr = RefHMC(nt, nx, m, g, mu, seed=seed, warmup=543210, variant=variant)
    tr.puregauge(sweeps)
    out["traj_seed"] = seed
    out["traj_sweeps"] = sweeps
    out["traj_nsteps"] = nsteps
    out["traj_A_start"] = tr.get_A()
    stats, As = [], []
    for _ in range(ntraj):
        stats.append(tr.trajectory(nsteps, 1.0))
        As.append(tr.get_A())
    out["traj_stats"] = np.array(stats)
    out["traj_A"] = np.array(As)
    np.savez_compressed(os.path.join(OUT, f"{name}.npz"), **out)
    print(name, "dH", out["traj_stats"][:, 0], "acc", out["traj_stats"][:, 9])


def make_mt():
    out = {}
    for s in MT_SEEDS:
        ref = RefHMC(4, 4, 0.1, 0.5, 0.0, seed=s, warmup=543210)
        out[f"seed_{s}"] = ref.uniforms(3000)
    ref = RefHMC(4, 4, 0.1, 0.5, 0.0, seed=12345, warmup=0)
    out["seed_12345_nowarmup"] = ref.uniforms(1300)
    np.savez_compressed(os.path.join(OUT, "mt_stream.npz"), **out)


def make_dense():
    out = {}
    for name, (nt, nx, m, mu, variant) in {"det_4x4_apx": (4, 4, 0.2, 0.1, "fixed_apx"),
                                           "det_4x4_px": (4, 4, 0.05, 0.0, "fixed_px"),
                                           "det_6x4_apx": (6, 4, 0.3, 0.25, "fixed_apx")}.items():
        rng = np.random.default_rng(nt * 100 + nx)
        A = rng.normal(0, 0.4, (nt, nx, 2))
        ref = RefHMC(nt, nx, m, 0.5, mu, variant=variant, warmup=0)
        ref.set_A(A)
        Md = ref.dense_M()
        sign, logdet = np.linalg.slogdet(Md)
        out[name] = dict(nt=nt, nx=nx, m=m, mu=mu, bc_x=(1 if variant.endswith("_px") else -1), A=A, M=Md,
                         logabsdet=logdet, phase=sign)
    for name, d in out.items():
        np.savez_compressed(os.path.join(OUT, f"{name}.npz"), **d)


VEC_CONFIGS = {  # name: (nt, nx, m, mu, fraction of occupied sites, seed)
    "vecops_8x8": (8, 8, 0.3, 0.2, 0.3, 1),
    "vecops_6x4": (6, 4, 0.5, 0.0, 0.25, 2),
    "vecops_16x16": (16, 16, 0.1, 0.0, 0.1, 3),
}


def make_vecops():
    """fM, fM_transpose and cg_MdM of the reference's vec_ops.c (fermion-bag
    operator, ANTISYMMETRIC boundaries) on random occupations."""
    from oracle.oracle import RefVecOps
    for name, (nt, nx, m, mu, occ, seed) in VEC_CONFIGS.items():
        rng = np.random.default_rng(seed)
        mask = (rng.random((nt, nx)) < occ).astype(np.int32)
        v = rng.normal(size=(nt, nx))
        b = rng.normal(size=(nt, nx))
        ref = RefVecOps(nt, nx, m, mu)
        ref.set_field(mask)
        np.savez_compressed(os.path.join(OUT, f"{name}.npz"), nt=nt, nx=nx, m=m, mu=mu, mask=mask, v=v, b=b,
                            fM_v=ref.fM(v), fMt_v=ref.fM(v, True), cg_x=ref.cg_MdM(b))


def make_free_det():
    """The free (A = 0, no monomers) fermion-bag matrix, built column by column
    from the reference's own vec_ops.c fM, and its log-determinant: the A = 0
    pin of the determinant (fermion_matrix.c:28-64 fM_index, same operator)."""
    from oracle.oracle import RefVecOps
    for name in ("vecops_8x8", "vecops_6x4"):
        nt, nx, m, mu = VEC_CONFIGS[name][:4]
        ref = RefVecOps(nt, nx, m, mu)
        ref.set_field(np.zeros((nt, nx), np.int32))
        V = nt * nx
        Mf = np.empty((V, V))
        for j in range(V):
            e = np.zeros(V)
            e[j] = 1.0
            Mf[:, j] = ref.fM(e.reshape(nt, nx)).ravel()
        sign, logabs = np.linalg.slogdet(Mf)
        np.savez_compressed(os.path.join(OUT, f"free_det_{nt}x{nx}.npz"), nt=nt, nx=nx, m=m, mu=mu, M=Mf,
                            logabsdet=logabs, sign=sign)


PROP_CONFIGS = {  # name: (nt, nx, m, mu, fraction of occupied sites, seed)
    "prop_8x8": (8, 8, 0.0, 0.2, 0.0, 0),
    "prop_6x4_mask": (6, 4, 0.3, 0.0, 0.25, 5),
}


def make_prop():
    """calc_Dinv (fermion_matrix.c:189-351, WITH_MASS_MONOMERS) of the reference:
    the propagator matrix from one cg_propagator solve per source site."""
    from oracle.oracle import RefVecOps
    for name, (nt, nx, m, mu, occ, seed) in PROP_CONFIGS.items():
        rng = np.random.default_rng(seed)
        mask = (rng.random((nt, nx)) < occ).astype(np.int32)
        ref = RefVecOps(nt, nx, m, mu, prop=True)
        ref.set_field(mask)
        np.savez_compressed(os.path.join(OUT, f"{name}.npz"), nt=nt, nx=nx, m=m, mu=mu, mask=mask,
                            Dinv=ref.calc_Dinv())


def make_determinant_pins():
    """The reference's own determinant code on 4 x 4 (its brute-force test size):

      * full_determinant.c's determinant_mu over fermion_matrix.c's fM_index
        (mass on the diagonal), antisymmetric boundaries and open x, for several
        m and mu, on the empty field (det(m + D) at A = 0) and on two monomer
        masks (the determinant over the unoccupied sites);
      * tests/thirring_brute.c's enumeration (open x) at three mu: the sums of
        the fermion-bag weights per (links, monomers).  With no links they give
        det(m + D) = sum_k m^k Z[0][k] / Z[0][16] for every m (the
        principal-minor expansion of det(m + D) with Jacobi's identity).
    """
    from oracle.oracle import RefFullDet, ref_brute
    nt = nx = 4
    rng = np.random.default_rng(44)
    masks = np.stack([np.zeros((nt, nx), np.int32)] +
                     [(rng.random((nt, nx)) < 0.3).astype(np.int32) for _ in range(2)])
    pairs = [(0.1, 0.0), (0.3, 0.1), (0.05, 0.25), (1.0, 0.0)]
    dets = np.zeros((2, len(pairs), len(masks)))
    for b, openx in enumerate((False, True)):
        for i, (m, mu) in enumerate(pairs):
            ref = RefFullDet(nt, nx, m, mu, openx)
            for k, mask in enumerate(masks):
                dets[b, i, k] = ref.determinant(mask)
    np.savez_compressed(os.path.join(OUT, "fulldet_4x4.npz"), nt=nt, nx=nx, boundaries=np.array(["apx", "openx"]),
                        m_mu=np.array(pairs), masks=masks, det=dets)
    mus = np.array([0.1, 0.0, 0.3])
    runs = [ref_brute(float(mu)) for mu in mus]
    Z = np.stack([r["det"] for r in runs])
    Zabs = np.stack([r["absdet"] for r in runs])
    np.savez_compressed(os.path.join(OUT, "brute_4x4_openx.npz"), nt=nt, nx=nx, mu=mus, Z=Z, Zabs=Zabs)
    print("fulldet", dets[:, :, 0], "brute Z[0]", Z[:, 0, :])


if __name__ == "__main__":
    # no arguments: every fixture; "determinants": the determinant pins only;
    # else only the named trajectory configs
    if sys.argv[1:] == ["determinants"]:
        make_ref.build([(4, 4)])
        make_determinant_pins()
        sys.exit(0)
    names = sys.argv[1:] or list(CONFIGS)
    make_ref.build(sorted({(CONFIGS[n][0], CONFIGS[n][1]) for n in names} | {(4, 4), (6, 4)}))
    if not sys.argv[1:]:
        make_vecops()
        make_free_det()
        make_prop()
        make_mt()
        make_dense()
        make_determinant_pins()
    for name in names:
        make_config(name, *CONFIGS[name])
