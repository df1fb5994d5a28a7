"""Post-solve kernels on the GPU: back-substitution (stc_bwd), H1 error
evaluation (element_error) and the compliance adjoint.

Tolerances:
* global solution, back-substituted dof and element errors: 1e-9 relative to
  the oracle path.  Element matrices agree to 1e-13; the oracle condenses with
  LU and the GPU with Cholesky, and the global solve amplifies the difference
  by its conditioning (measured ~1e-11).
* the restated reference pins evaluated entirely on the GPU: poly_pois H1
  error < 1e-15, conv_pois rate in [1.95, 2.05].
* adjoint vs central finite differences (step 1e-6 relative): 1e-6 relative
  plus the rounding floor of the difference quotient, 1e-14 |J| / step.
* adjoint vs an FP64 CPU gradient (oracle element matrices, element-level
  central differences): 1e-7 relative.
"""
import numpy as np
import pytest

from oracle import oracle as O
from hp3d_gb300 import hp3dg as H
from hp3d_gb300 import mesh as M
import fem_harness as FH
from test_gpu_parity import _gpu_elements

pytestmark = pytest.mark.gpu


def _gpu_solve(m, isol, zd=None, prec=H.FP64, keep=False, integration=0):
    ep = H.ElementPass(prec, isol=isol, keep_elem=keep, integration=integration)
    ep.submit(m, zdofd=zd)
    ep.run(); ep.download()
    els = _gpu_elements(ep, m)
    x, lcon, lo = FH.assemble_solve(m, els)
    ep.backsub(x)
    return ep, els, x


@pytest.mark.parametrize("n", [2, 4])
def test_poly_pois_error_on_gpu(n):
    m = M.structured_hexa(n, 1)
    zd = FH.dirichlet_data(m, 12)
    ep, els, x = _gpu_solve(m, 12, zd)
    e2, n2 = ep.element_error(12)
    assert np.sqrt(e2.sum()) < 1e-15
    assert abs(np.sqrt(n2.sum()) - 0.6085806194501846) < 1e-12


def test_conv_pois_rate_on_gpu():
    errs = []
    for n in (2, 4, 8):
        m = M.structured_hexa(n, 2)
        zd = FH.dirichlet_data(m, 2)
        ep, els, x = _gpu_solve(m, 2, zd)
        e2, _ = ep.element_error(2)
        errs.append(np.sqrt(e2.sum()))
        ep.close()
    rate = np.log(errs[-2] / errs[-1]) / np.log(2.0)
    assert 1.95 <= rate <= 2.05


def test_backsub_and_error_match_oracle():
    m = M.random_orientations(M.structured_hexa(3, 4, perturb=0.1, seed=8), seed=2)
    ep, els, x = _gpu_solve(m, 10)
    ref = FH.oracle_element_outputs(m, 10)
    err_o, _, x_o, dofs_o = FH.solve_and_error(m, ref, 10)
    assert np.abs(x - x_o).max() <= 1e-9 * np.abs(x_o).max()
    for e in range(m["nelem"]):
        d = ep.dofs(e)
        assert np.abs(d - dofs_o[e]).max() <= 1e-9 * max(np.abs(dofs_o[e]).max(), 1e-300)
    e2, _ = ep.element_error(10)
    assert abs(np.sqrt(e2.sum()) - err_o) <= 1e-9 * err_o


# ---------------------------------------------------------------------------
# compliance adjoint (config: p=4, vertices perturbed +-0.1h, kappa in [1e-2, 1e2], f = 1)
# ---------------------------------------------------------------------------
def _compliance(m, prec=H.FP64, integration=0):
    ep = H.ElementPass(prec, isol=11, keep_elem=True, integration=integration)
    ep.submit(m)
    ep.run(); ep.download()
    els = _gpu_elements(ep, m)
    x, _, _ = FH.assemble_solve(m, els)
    ep.backsub(x)
    n = (m["p"] + 1) ** 3
    J = 0.0
    dofs = []
    for e in range(m["nelem"]):
        _, b = ep.elem(e, n)
        d = ep.dofs(e)
        dofs.append(d)
        J += b @ d
    return J, ep, dofs


def _set_vertex(m, vid, k, val):
    m2 = dict(m)
    X = m["vertex_xyz"].copy()
    X[vid, k] = val
    m2["vertex_xyz"] = X
    m2["xvert"] = X[m["nodes"][:, :8]]
    return m2


def test_adjoint_against_central_differences():
    m = M.structured_hexa(3, 4, perturb=0.1, kappa_logrange=(-2, 2), seed=31)
    J0, ep, dofs = _compliance(m)
    dk, dx = ep.adjoint()
    rng = np.random.default_rng(5)
    # kappa parameters
    for e in rng.choice(m["nelem"], 6, replace=False):
        h = 1e-6 * m["kappa"][e]
        mp = dict(m); mp["kappa"] = m["kappa"].copy(); mp["kappa"][e] += h
        mm = dict(m); mm["kappa"] = m["kappa"].copy(); mm["kappa"][e] -= h
        fd = (_compliance(mp)[0] - _compliance(mm)[0]) / (2 * h)
        # rounding floor of a central difference: ~eps_solve |J| / h with h = 1e-6 kappa_e
        assert abs(fd - dk[e]) <= 1e-6 * abs(fd) + 1e-14 * abs(J0) / 1e-6 / m["kappa"][e], (e, fd, dk[e])
    # interior vertex coordinates: sum the element contributions of the vertex
    interior = [v for v in range(m["nverts"])
                if np.all((m["vertex_xyz"][v] > 1e-12) & (m["vertex_xyz"][v] < 1 - 1e-12))]
    for v in rng.choice(interior, 3, replace=False):
        for k in range(3):
            g = 0.0
            for e in range(m["nelem"]):
                loc = np.where(m["nodes"][e, :8] == v)[0]
                for q in loc:
                    g += dx[e, q, k]
            x0 = m["vertex_xyz"][v, k]
            h = 1e-6 * max(abs(x0), 1e-3)
            fd = (_compliance(_set_vertex(m, v, k, x0 + h))[0] -
                  _compliance(_set_vertex(m, v, k, x0 - h))[0]) / (2 * h)
            assert abs(fd - g) <= 1e-6 * max(abs(fd), abs(J0)), (v, k, fd, g)


def test_adjoint_against_cpu_gradient():
    """FP64 CPU gradient: dJ/dkappa_e = -u^T K_e u / kappa_e from the oracle's
    element matrix, and element-level central differences of
    -u^T K_e(X) u + 2 u^T b_e(X) with the oracle element routine."""
    m = M.structured_hexa(2, 4, perturb=0.1, kappa_logrange=(-2, 2), seed=33)
    J0, ep, dofs = _compliance(m)
    dk, dx = ep.adjoint()
    for e in range(m["nelem"]):
        K, b, _ = O.elem(1, m["norder"][e], m["nori_edge"][e], m["nori_face"][e], m["xvert"][e],
                         m["kappa"][e], isol=11, integration=0)
        u = dofs[e]
        ref_k = -(u @ K @ u) / m["kappa"][e]
        assert abs(ref_k - dk[e]) <= 1e-10 * abs(ref_k)
        for vq in (0, 6):
            for k in range(3):
                h = 1e-6
                vals = []
                for s in (+1, -1):
                    xv = m["xvert"][e].copy(); xv[vq, k] += s * h
                    Kp, bp, _ = O.elem(1, m["norder"][e], m["nori_edge"][e], m["nori_face"][e],
                                       xv, m["kappa"][e], isol=11, integration=0)
                    vals.append(-(u @ Kp @ u) + 2 * (u @ bp))
                ref = (vals[0] - vals[1]) / (2 * h)
                assert abs(ref - dx[e, vq, k]) <= 1e-7 * max(abs(ref), abs(J0)), (e, vq, k)


def test_autograd_harness_directional_derivative():
    torch = pytest.importorskip("torch")
    from compliance_autograd import Compliance
    m = M.structured_hexa(2, 3, perturb=0.1, kappa_logrange=(-1, 1), seed=41)
    kappa = torch.tensor(m["kappa"], dtype=torch.float64, requires_grad=True)
    xvert = torch.tensor(m["xvert"], dtype=torch.float64, requires_grad=True)
    J = Compliance.apply(kappa, xvert, m)
    J.backward()
    rng = np.random.default_rng(3)
    dk = rng.standard_normal(m["nelem"]) * m["kappa"]
    dxv = np.zeros_like(m["xvert"])
    dxv[:, 6, :] = rng.standard_normal((m["nelem"], 3)) * 0.01  # move each element's v7 copy
    t = 1e-6
    def Jat(s):
        with torch.no_grad():
            return float(Compliance.apply(kappa + s * torch.from_numpy(dk),
                                          xvert + s * torch.from_numpy(dxv), m))
    fd = (Jat(t) - Jat(-t)) / (2 * t)
    ad = float((kappa.grad * torch.from_numpy(dk)).sum() + (xvert.grad * torch.from_numpy(dxv)).sum())
    assert abs(fd - ad) <= 1e-6 * abs(ad) + 1e-12 * abs(float(J.detach())) / t
