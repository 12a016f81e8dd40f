"""torch.autograd view of the pseudofermion action, FOR CHECKING THE FORCE ONLY.

    S_pf(A) = sum_k Re <phi_k, (M^dag M)^-1 phi_k>        (hmc.c:451-463)

`PseudofermionAction.apply(A, phi, lattice, cg)` evaluates S_pf on the GPU
through the C ABI and its backward pass returns the hand-derived adjoint force
dS_pf/dA (tg_pf_force, hmc.c:517-576 restated), recomputing the CG solutions
instead of storing them.  It lets the force be compared with finite
differences and with torch's own gradient machinery; the HMC itself never
goes through torch.
"""
from __future__ import annotations

import numpy as np
import torch

from . import native as N
from .lattice import Lattice, cg_params


class PseudofermionAction(torch.autograd.Function):
    @staticmethod
    def forward(ctx, A: torch.Tensor, phi: torch.Tensor, lattice: Lattice, cg: N.CgParams | None = None):
        cg = cg or cg_params(rel_tol=1e-12, abs_tol2=0.0)
        A_np = A.detach().to("cpu", torch.float64).numpy()
        phi_np = phi.detach().to("cpu", torch.complex128).numpy().reshape(-1, lattice.nt, lattice.nx)
        lattice.set_gauge(A_np)
        S = 0.0
        for k in range(phi_np.shape[0]):
            s, res = lattice.pseudofermion_action(phi_np[k], cg)
            if res.status != N.TG_OK:
                raise N.TGError(res.status, "CG did not converge in the pseudofermion action")
            S += s
        ctx.save_for_backward(A.detach(), phi.detach())
        ctx.lattice, ctx.cg = lattice, cg
        return torch.tensor(S, dtype=torch.float64, device=A.device)

    @staticmethod
    def backward(ctx, grad_out):
        A, phi = ctx.saved_tensors
        L = ctx.lattice
        L.set_gauge(A.to("cpu", torch.float64).numpy())
        F, res = L.pf_force(phi.to("cpu", torch.complex128).numpy().reshape(-1, L.nt, L.nx), ctx.cg)
        if res.status != N.TG_OK:
            raise N.TGError(res.status, "CG did not converge in the force")
        gA = torch.from_numpy(np.ascontiguousarray(F)).to(A.device) * grad_out
        return gA, None, None, None


def pseudofermion_action(A: torch.Tensor, phi: torch.Tensor, lattice: Lattice, cg: N.CgParams | None = None):
    return PseudofermionAction.apply(A, phi, lattice, cg)
