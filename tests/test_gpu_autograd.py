"""The differentiation check on 64x64 (m 0.1, g 0.5, A ~ N(0, 0.3^2), two
pseudofermions): the hand-derived adjoint force dS_pf/dA, reached through the
torch.autograd wrapper over the C ABI, against central finite differences of
S_pf (step 1e-6, 256 random links) and against the oracle's force, in FP64 and
with the mixed-precision solver."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")

N_SITES = 64
H = 1e-6


@pytest.fixture(scope="module")
def setup(oracle_lib):
    import thirring2d_gb300 as tg
    n = N_SITES
    rng = np.random.default_rng(64)
    A = rng.normal(0, 0.3, (n, n, 2))
    o = oracle_lib.Oracle(n, n, 0.1, 0.5, 0.0, -1, 1)
    etas = [rng.normal(size=(n, n)) + 1j * rng.normal(size=(n, n)) for _ in range(2)]
    phis = np.stack([o.Mdag(A, e) for e in etas])
    links = [(int(rng.integers(n)), int(rng.integers(n)), int(rng.integers(2))) for _ in range(256)]
    return tg, o, A, phis, links


def grad_and_action(tg, A, phis, precision):
    from thirring2d_gb300.autograd import pseudofermion_action
    n = N_SITES
    L = tg.Lattice(n, n, 0.1, 0.5, 0.0, -1, 1)
    # a tight solve keeps the CG error of S far below the finite-difference signal
    cg = tg.cg_params(rel_tol=1e-14, abs_tol2=0.0, precision=precision, ru_interval=50)
    At = torch.tensor(A, dtype=torch.float64, requires_grad=True)
    S = pseudofermion_action(At, torch.from_numpy(phis), L, cg)
    S.backward()
    return L, cg, S.item(), At.grad.numpy().copy()


@pytest.mark.parametrize("precision", [0, 1])
def test_force_vs_central_differences(setup, precision):
    tg, o, A, phis, links = setup
    from thirring2d_gb300.autograd import pseudofermion_action
    L, cg, S0, F = grad_and_action(tg, A, phis, precision)
    phit = torch.from_numpy(phis)
    worst = 0.0
    for (t, x, d) in links:
        Ap, Am = A.copy(), A.copy()
        Ap[t, x, d] += H
        Am[t, x, d] -= H
        Sp = pseudofermion_action(torch.from_numpy(Ap), phit, L, cg).item()
        Sm = pseudofermion_action(torch.from_numpy(Am), phit, L, cg).item()
        fd = (Sp - Sm) / (2 * H)
        err = abs(fd - F[t, x, d]) / max(1.0, abs(F[t, x, d]))
        worst = max(worst, err)
    # central differences at h = 1e-6 of an action of size ~1e4 carry ~1e-6 of
    # rounding; the oracle's own check reaches the same level
    assert worst < 2e-5, worst


@pytest.mark.parametrize("precision", [0, 1])
def test_force_vs_oracle(setup, precision):
    tg, o, A, phis, links = setup
    L, cg, S0, F = grad_and_action(tg, A, phis, precision)
    chis = [o.cg(A, ph, rel_tol=1e-14, abs_tol2=0)[0] for ph in phis]
    F_o = o.pf_force(A, chis)
    err = np.abs(F - F_o).max() / np.abs(F_o).max()
    assert err < (1e-11 if precision == 0 else 1e-10), err
    S_o = sum(float(np.vdot(ph, c).real) for ph, c in zip(phis, chis))
    assert abs(S0 - S_o) <= 1e-11 * abs(S_o)
