"""torch.autograd.Function harness around the compliance adjoint.

J(kappa, x) = f^T u with K(kappa, x) u = f on a hexahedral mesh.  Forward:
the GPU element pass (hp3dg_batch_*), the condensed global solve (SciPy,
standing in for MUMPS) and the GPU back-substitution.  Backward: the GPU
adjoint kernel (hp3dg_adjoint) gives dJ/dkappa_e and the per-element vertex
contributions dJ/dxvert[e] (each element owns a copy of its 8 vertices).
Test infrastructure: the product is the C ABI.
"""
import numpy as np
import torch

from hp3d_gb300 import hp3dg as H
import fem_harness as FH
from test_gpu_parity import _gpu_elements


def compliance(mesh, integration=0, isol=11):
    """J, the element pass and the full element dof vectors."""
    ep = H.ElementPass(H.FP64, isol=isol, keep_elem=True, integration=integration)
    ep.submit(mesh)
    ep.run()
    ep.download()
    x, _, _ = FH.assemble_solve(mesh, _gpu_elements(ep, mesh))
    ep.backsub(x)
    n = (mesh["p"] + 1) ** 3
    J = 0.0
    dofs = []
    for e in range(mesh["nelem"]):
        _, b = ep.elem(e, n)
        d = ep.dofs(e)
        dofs.append(d)
        J += b @ d
    return J, ep, dofs


class Compliance(torch.autograd.Function):
    @staticmethod
    def forward(ctx, kappa, xvert, mesh):
        m = dict(mesh)
        m["kappa"] = kappa.detach().cpu().numpy().astype(np.float64)
        m["xvert"] = xvert.detach().cpu().numpy().astype(np.float64)
        J, ep, _ = compliance(m)
        dk, dx = ep.adjoint()
        ep.close()
        ctx.save_for_backward(torch.from_numpy(dk), torch.from_numpy(dx))
        return torch.tensor(J, dtype=torch.float64)

    @staticmethod
    def backward(ctx, gJ):
        dk, dx = ctx.saved_tensors
        return gJ * dk, gJ * dx, None
