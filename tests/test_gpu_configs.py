"""The benchmark configurations at their stated sizes (where a host solve of
that size fits a test), through the C ABI on the GPU.

Config 1 (plain FP64 Galerkin Poisson): 4^3 affine hexahedra of the unit
cube, p = 3, kappa = 1, u = sin(pi x) sin(pi y) sin(pi z), f = 3 pi^2 u,
homogeneous Dirichlet boundary, Gauss rule of order p + 1 per direction
(INTEGRATION = 0), static condensation and the global solve.  The pass's
condensed systems must equal the oracle's (elem_opt + stc_fwd +
celem_systemI) to 1e-12, the interface solution (what MUMPS returns) to
1e-10, and the H1 errors evaluated on the GPU to the oracle path's.

Config 4 (differentiation): 16^3 hexahedra, p = 4, vertices moved by
U(-0.1h, 0.1h), kappa_e = 10**U(-2, 2), f = 1, compliance J = f^T u.  The
adjoint kernel's dJ/dkappa_e is checked on every one of the 4,096 elements
against the FP64 CPU gradient -u_e^T (K_e / kappa_e) u_e with the oracle's
element matrices, and its dJ/dx contributions on 48 elements against
element-level central differences of the oracle's -u^T K_e(x) u + 2 u^T b_e(x)
(the formula is the same for any u, so a random interface vector
back-substituted on the GPU stands in for the solution of the 164k-unknown
system).  Central differences of J itself (step 1e-6 relative; bar 1e-6
relative plus the rounding floor of the quotient, 1e-13 |J| / step) at 64 random
parameters -- 32 element coefficients and 32 interior vertex coordinates --
need 129 solves: they run on the largest mesh of the same kind whose solves
fit the test, 4^3 hexahedra (64 elements, 2,197 H1 dof).
"""
import numpy as np
import pytest

from oracle import oracle as O
from hp3d_gb300 import hp3dg as H
from hp3d_gb300 import mesh as M
import fem_harness as FH

pytestmark = pytest.mark.gpu


def test_config1_plain_fp64_through_the_solve():
    m = M.structured_hexa(4, 3, perturb=0.0, kappa_logrange=None)
    assert np.all(m["kappa"] == 1.0)
    ep = H.ElementPass(H.FP64, integration=0, isol=10)
    ep.submit(m)
    ep.run()
    ep.download()
    gel = FH.gpu_elements(ep, m)
    orc = FH.oracle_element_outputs(m, 10, integration=0, stc_method=0)
    for e in range(m["nelem"]):
        zs, ozs = gel[e]["zastif"], orc[e]["zastif"]
        if ozs.size:
            assert np.abs(zs - ozs).max() <= 1e-12 * np.abs(ozs).max(), e
            assert np.abs(gel[e]["zbload"] - orc[e]["zbload"]).max() <= \
                1e-12 * max(np.abs(orc[e]["zbload"]).max(), 1e-300), e
    x, lcon, _ = FH.assemble_solve(m, gel)
    xo, lcono, _ = FH.assemble_solve(m, orc)
    # 13^3 H1 dof: 11^3 = 1331 free, 512 bubbles, 819 interface unknowns
    assert len(x) == 819 and np.array_equal(lcon, lcono)
    assert np.linalg.norm(x - xo) <= 1e-10 * np.linalg.norm(xo)
    ep.backsub(x)
    e2, n2 = ep.element_error(10)
    err_o, nrm_o, _, _ = FH.solve_and_error(m, orc, 10)
    assert abs(np.sqrt(e2.sum()) - err_o) <= 1e-9 * err_o
    assert abs(np.sqrt(n2.sum()) - nrm_o) <= 1e-12 * nrm_o
    ep.close()


def test_config4_adjoint_every_element_against_cpu_gradient():
    m = M.structured_hexa(16, 4, perturb=0.1, kappa_logrange=(-2, 2), seed=44)
    ep = H.ElementPass(H.FP64, integration=0, isol=11, keep_elem=True)
    ep.submit(m)
    ep.run()
    ep.download()
    nr = ep.index_map()[0]
    rng = np.random.default_rng(8)
    ep.backsub(rng.standard_normal(nr))
    dk, dx = ep.adjoint()
    dofs = [ep.dofs(e) for e in range(m["nelem"])]
    worst = 0.0
    for e in range(m["nelem"]):
        K, b, rc = O.elem(1, m["norder"][e], m["nori_edge"][e], m["nori_face"][e], m["xvert"][e],
                          m["kappa"][e], isol=11, integration=0)
        u = dofs[e]
        ref = -(u @ K @ u) / m["kappa"][e]
        worst = max(worst, abs(ref - dk[e]) / abs(ref))
    assert worst <= 1e-10, worst
    for e in rng.choice(m["nelem"], 48, replace=False):
        u = dofs[e]
        for vq in rng.choice(8, 1):
            for k in range(3):
                h = 1e-6 / 16
                vals = []
                for s in (+1, -1):
                    xv = m["xvert"][e].copy()
                    xv[vq, k] += s * h
                    Kp, bp, _ = O.elem(1, m["norder"][e], m["nori_edge"][e], m["nori_face"][e],
                                       xv, m["kappa"][e], isol=11, integration=0)
                    vals.append(-(u @ Kp @ u) + 2 * (u @ bp))
                ref = (vals[0] - vals[1]) / (2 * h)
                scale = max(abs(ref), abs(vals[0]) / 16)
                assert abs(ref - dx[e, vq, k]) <= 1e-6 * scale, (e, vq, k, ref, dx[e, vq, k])
    ep.close()


def _compliance(m):
    ep = H.ElementPass(H.FP64, isol=11, keep_elem=True, integration=0)
    ep.submit(m)
    ep.run()
    ep.download()
    x, _, _ = FH.assemble_solve(m, FH.gpu_elements(ep, m))
    ep.backsub(x)
    n = (m["p"] + 1) ** 3
    J = sum(ep.elem(e, n)[1] @ ep.dofs(e) for e in range(m["nelem"]))
    return J, ep


def _with_vertex(m, v, k, val):
    m2 = dict(m)
    X = m["vertex_xyz"].copy()
    X[v, k] = val
    m2["vertex_xyz"] = X
    m2["xvert"] = X[m["nodes"][:, :8]]
    return m2


def test_config4_central_differences_at_64_parameters():
    m = M.structured_hexa(4, 4, perturb=0.1, kappa_logrange=(-2, 2), seed=45)
    J0, ep = _compliance(m)
    dk, dx = ep.adjoint()
    ep.close()
    rng = np.random.default_rng(12)
    for e in rng.choice(m["nelem"], 32, replace=False):
        h = 1e-6 * m["kappa"][e]
        Js = []
        for s in (+1, -1):
            mk = dict(m)
            mk["kappa"] = m["kappa"].copy()
            mk["kappa"][e] += s * h
            J, epk = _compliance(mk)
            epk.close()
            Js.append(J)
        fd = (Js[0] - Js[1]) / (2 * h)
        # the difference quotient's rounding floor: J from a sparse direct
        # solve carries ~1e-14 relative error in each evaluation, amplified by
        # the global conditioning, divided by the step
        assert abs(fd - dk[e]) <= 1e-6 * abs(fd) + 1e-13 * abs(J0) / h, (e, fd, dk[e])
    interior = [v for v in range(m["nverts"])
                if np.all((m["vertex_xyz"][v] > 1e-12) & (m["vertex_xyz"][v] < 1 - 1e-12))]
    coords = [(v, k) for v in interior for k in range(3)]
    for idx in rng.choice(len(coords), 32, replace=False):
        v, k = coords[idx]
        g = sum(dx[e, q, k] for e in range(m["nelem"]) for q in np.where(m["nodes"][e, :8] == v)[0])
        x0 = m["vertex_xyz"][v, k]
        h = 1e-6 * max(abs(x0), 1e-3)
        Js = []
        for s in (+1, -1):
            J, epv = _compliance(_with_vertex(m, v, k, x0 + s * h))
            epv.close()
            Js.append(J)
        fd = (Js[0] - Js[1]) / (2 * h)
        assert abs(fd - g) <= 1e-6 * max(abs(fd), abs(J0)), (v, k, fd, g)
