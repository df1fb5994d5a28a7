"""Prism restatement in the oracle (shape3DHPris, the triangle x Gauss rule
of set_3D_int) and the conforming mixed hexa/prism/tet meshes, pinned by:

* the triangle rules of degree 2..12 and the Gauss factor integrate
  monomials of degree <= 2ph in (x, y) and 2pz+1 in z exactly (the
  reference's init_gauss_quadrature checks weight sums and barycentric sums
  to 1e-13, gauss_quadrature.F90:700-735);
* the H1 prism space of orders (ph, pz) is complete (P_ph(x,y) x P_pz(z))
  for random edge / face orientation codes (face orders in the faces' own
  frames); gradients match finite differences;
* end to end through the harness's direct solve: test/poly_pois.F90 (u =
  xyz reproduced) on prism meshes and on the mixed mesh at order 3, and a
  linear solution (isol 13) reproduced on the hp-adaptive mixed mesh --
  which needs every quad / triangle orientation code and min-rule order
  across the hexa-prism and prism-tet interfaces to be consistent.
"""
import math

import numpy as np
import pytest

from oracle import oracle as O
from hp3d_gb300 import mesh as M
import fem_harness as FH


def _no(ph, pz):
    a = np.zeros(19, np.int32)
    a[0:6] = ph; a[6:9] = pz; a[9:11] = ph; a[11:14] = 10 * ph + pz; a[14] = 10 * ph + pz
    return a


@pytest.mark.parametrize("ph,pz", [(1, 1), (2, 3), (4, 2), (6, 6)])
def test_prism_rule_exact(ph, pz):
    xi, w = O.quad_prism(_no(ph, pz))
    for i in range(2 * ph + 1):
        for j in range(2 * ph + 1 - i):
            for k in range(2 * pz + 2):
                ex = math.factorial(i) * math.factorial(j) / math.factorial(i + j + 2) / (k + 1)
                v = (w * xi[:, 0] ** i * xi[:, 1] ** j * xi[:, 2] ** k).sum()
                assert abs(v - ex) <= 1e-13 * ex


@pytest.mark.parametrize("ph,pz", [(1, 1), (3, 2), (6, 5)])
def test_prism_shape_complete(ph, pz):
    rng = np.random.default_rng(ph * 10 + pz)
    no = _no(ph, pz)
    ne = rng.integers(0, 2, 12)
    nf = np.concatenate([rng.integers(0, 6, 2), rng.integers(0, 8, 4)])
    for f in range(3):
        if M.ORIENT_QUAD[nf[2 + f]][0] == 1:
            no[11 + f] = 10 * pz + ph  # the face's own frame has the axes swapped
    n = O.nrdofH(O.PRISM, no)
    assert n == (ph + 1) * (ph + 2) // 2 * (pz + 1)
    x = np.array([0.2, 0.15, 0.3])
    s, g = O.shape_prism(x, no, ne, nf)
    assert abs(s[:6].sum() - 1.0) < 1e-15
    h = 1e-6
    for c in range(3):
        xp, xm = x.copy(), x.copy()
        xp[c] += h; xm[c] -= h
        fd = (O.shape_prism(xp, no, ne, nf)[0] - O.shape_prism(xm, no, ne, nf)[0]) / (2 * h)
        assert np.abs(fd - g[:, c]).max() < 1e-7 * max(1.0, np.abs(g).max())
    pts = rng.random((3000, 3))
    pts = pts[pts[:, 0] + pts[:, 1] < 1][:2 * n + 20]
    A = np.array([O.shape_prism(q, no, ne, nf)[0] for q in pts])
    mons = [(i, j, k) for i in range(ph + 1) for j in range(ph + 1 - i) for k in range(pz + 1)]
    B = np.array([[q[0] ** i * q[1] ** j * q[2] ** k for (i, j, k) in mons] for q in pts])
    coef, _, rank, _ = np.linalg.lstsq(A, B, rcond=None)
    assert rank == n and np.abs(A @ coef - B).max() < 1e-10


@pytest.mark.parametrize("ph,pz,perturb", [(2, 1, 0.0), (3, 3, 0.15)])
def test_poly_pois_prisms(ph, pz, perturb):
    # xyz is in the space of an affine prism for (ph, pz) >= (2, 1); a
    # perturbed prism maps bilinearly in (Nu, Mu), which needs (3, 3)
    m = M.structured_prism(2, ph, pz, perturb=perturb, seed=5)
    zd = FH.dirichlet_data(m, 12)
    ref = FH.oracle_element_outputs(m, 12, zdofd=zd)
    err, nrm, _, _ = FH.solve_and_error(m, ref, 12, zdofd=zd)
    assert err < 1e-12 * nrm


def test_poly_pois_mixed_mesh():
    m = M.mixed_mesh(4, a=0.5, b=0.5, p=3, perturb=0.1, seed=7, kappa_logrange=None)
    assert set(np.unique(m["etype"])) == {1, 2, 3}
    zd = FH.dirichlet_data(m, 12)
    ref = FH.oracle_element_outputs(m, 12, zdofd=zd)
    err, nrm, _, _ = FH.solve_and_error(m, ref, 12, zdofd=zd)
    assert err < 1e-12 * nrm


def test_linear_solution_hp_mixed_mesh():
    m = M.mixed_mesh(4, a=0.5, b=0.5, perturb=0.1, seed=9, kappa_logrange=None)
    assert len({tuple(o) for o in m["orders"]}) > 10
    zd = FH.dirichlet_data(m, 13)
    ref = FH.oracle_element_outputs(m, 13, zdofd=zd)
    err, nrm, _, _ = FH.solve_and_error(m, ref, 13, zdofd=zd)
    assert err < 1e-12 * nrm


def test_poly_pois_corner_mixed_mesh():
    """The corner layout (tetrahedra in a corner block, prisms extruded along
    x, y and z beside it, hexahedra elsewhere) is conforming: u = xyz is
    reproduced (test/poly_pois.F90:101) at p = 3 on a perturbed mesh."""
    m = M.mixed_mesh(4, a=0.5, b=0.5, cy=0.5, p=3, perturb=0.1, seed=7, kappa_logrange=None)
    assert set(np.unique(m["etype"])) == {1, 2, 3}
    zd = FH.dirichlet_data(m, 12)
    ref = FH.oracle_element_outputs(m, 12, zdofd=zd)
    err, nrm, _, _ = FH.solve_and_error(m, ref, 12, zdofd=zd)
    assert err < 1e-12 * nrm


def test_linear_solution_hp_corner_mixed_mesh():
    m = M.mixed_mesh(4, a=0.5, b=0.5, cy=0.5, perturb=0.1, seed=9, kappa_logrange=None)
    assert len({tuple(o) for o in m["orders"]}) > 10
    zd = FH.dirichlet_data(m, 13)
    ref = FH.oracle_element_outputs(m, 13, zdofd=zd)
    err, nrm, _, _ = FH.solve_and_error(m, ref, 13, zdofd=zd)
    assert err < 1e-12 * nrm


def test_batching_mesh_composition():
    """The hp batching workload: 25^3 cells, tetrahedra in a 6 x 6 x 7 corner
    block: 19,129 elements, 68.6 / 23.5 / 7.9 % hexa / prism / tet (the
    conforming layout's closest split to 70 / 20 / 10 near 20,000 elements:
    prism columns bound the tetrahedra's share)."""
    m = M.mixed_mesh(25, a=19 / 25, b=18 / 25, cy=19 / 25, pmax=6, perturb=0.1,
                     kappa_logrange=(-1, 1), seed=12345)
    cnt = np.bincount(m["etype"], minlength=4)[1:]
    assert m["nelem"] == 19129 and list(cnt) == [13129, 4488, 1512]
    assert np.all(m["kappa"] >= 0.1 - 1e-12) and np.all(m["kappa"] <= 10 + 1e-12)
