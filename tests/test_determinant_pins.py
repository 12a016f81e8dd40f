"""The determinant pins from the reference's own determinant code, 4 x 4.

tests/golden/fulldet_4x4.npz holds full_determinant.c's determinant_mu
(full_determinant.c:144-186) over fermion_matrix.c's fM_index with the mass on
the diagonal: det(m + D) at A = 0 on the empty field, and the determinant over
the unoccupied sites of two monomer masks, with antisymmetric boundaries and
with open x.  tests/golden/brute_4x4_openx.npz holds tests/thirring_brute.c's
enumeration (open x): Z[links][monomers], the sum of the fermion-bag weights
det_save over every configuration.  With no links, expanding det(m + D) in its
principal minors and applying Jacobi's identity to each gives, for every m,

    det(m + D) = sum_k m^k Z[0][k] / Z[0][16]

(Z[0][16] = 1 / det D, the all-monomer term).  Both generated by
tests/golden/make_golden.py from builds of the reference's sources
(oracle/make_ref.py).

The CPU tests hold the oracle's dense operator to them; the GPU tests hold the
library's dense operator (tg_dense_M) and batched LU log-determinant
(tg_log_det) at A = 0 with the same boundaries (bc_t = -1; bc_x = -1, or 0 for
open x) to them.
"""
import numpy as np
import pytest

from helpers import golden

BC_X = {"apx": -1, "openx": 0}
M_POLY = [0.0, 0.02, 0.1, 0.3, 0.7, 1.0, 2.5]


def _poly_det(Z0, m):
    """det(m + D) from the brute-force sums with no links."""
    return np.polyval(Z0[::-1], m) / Z0[16]


def test_brute_force_sums_are_the_free_determinant(oracle_lib):
    d = golden("brute_4x4_openx")
    A = np.zeros((4, 4, 2))
    for mu, Z in zip(d["mu"], d["Z"]):
        Z0 = Z[0]
        assert not Z0[1::2].any()       # odd monomer numbers cannot pair up: zero weight
        for m in M_POLY:
            det = np.linalg.det(oracle_lib.Oracle(4, 4, m, 0.5, float(mu), -1, 0).dense_M(A))
            want = _poly_det(Z0, m)
            assert abs(det.imag) <= 1e-14 * abs(det)
            assert abs(det.real - want) <= 1e-12 * abs(want), (mu, m, det, want)


@pytest.mark.parametrize("b", [0, 1])
def test_full_determinant_matches_oracle_operator(oracle_lib, b):
    d = golden("fulldet_4x4")
    bnd = str(d["boundaries"][b])
    A = np.zeros((4, 4, 2))
    for i, (m, mu) in enumerate(d["m_mu"]):
        Md = oracle_lib.Oracle(4, 4, float(m), 0.5, float(mu), -1, BC_X[bnd]).dense_M(A)
        for k, mask in enumerate(d["masks"]):
            keep = np.flatnonzero(mask.ravel() == 0)
            det = np.linalg.det(Md[np.ix_(keep, keep)])
            want = d["det"][b, i, k]
            assert abs(det.imag) <= 1e-14 * abs(det)
            assert abs(det.real - want) <= 1e-12 * abs(want), (bnd, m, mu, k, det, want)


# ---------------------------------------------------------------------------
# the library, on the GPU
# ---------------------------------------------------------------------------
@pytest.fixture(scope="module")
def tg():
    import thirring2d_gb300 as tg
    tg.native.load()
    return tg


@pytest.mark.gpu
def test_gpu_log_det_matches_brute_force(tg):
    """tg_log_det at A = 0, open x, against the brute-force enumeration's
    polynomial in m, for each mu of the fixture (m = 0 included: det D)."""
    d = golden("brute_4x4_openx")
    for mu, Z in zip(d["mu"], d["Z"]):
        for m in M_POLY:
            L = tg.Lattice(4, 4, m, 0.5, float(mu), -1, 0)
            L.set_gauge(np.zeros((4, 4, 2)))
            la, ph = L.log_det()
            L.close()
            want = _poly_det(Z[0], m)
            assert abs(la - np.log(abs(want))) <= 1e-12, (mu, m, la, want)
            assert abs(np.cos(ph) - np.sign(want)) <= 1e-12 and abs(np.sin(ph)) <= 1e-12


@pytest.mark.gpu
@pytest.mark.parametrize("b", [0, 1])
def test_gpu_determinant_matches_full_determinant(tg, b):
    """tg_log_det on the empty field, and det of tg_dense_M's rows and columns
    of the unoccupied sites, against determinant_mu, both boundaries."""
    d = golden("fulldet_4x4")
    bnd = str(d["boundaries"][b])
    for i, (m, mu) in enumerate(d["m_mu"]):
        L = tg.Lattice(4, 4, float(m), 0.5, float(mu), -1, BC_X[bnd])
        L.set_gauge(np.zeros((4, 4, 2)))
        la, ph = L.log_det()
        Md = L.fermion_matrix()
        L.close()
        want0 = d["det"][b, i, 0]
        assert abs(la - np.log(abs(want0))) <= 1e-12, (bnd, m, mu, la, want0)
        assert abs(np.cos(ph) - np.sign(want0)) <= 1e-12 and abs(np.sin(ph)) <= 1e-12
        for k, mask in enumerate(d["masks"]):
            keep = np.flatnonzero(mask.ravel() == 0)
            det = np.linalg.det(Md[np.ix_(keep, keep)])
            want = d["det"][b, i, k]
            assert abs(det - want) <= 1e-12 * abs(want), (bnd, m, mu, k, det, want)
