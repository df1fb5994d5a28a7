"""Pins of the CPU oracle against the reference's own tests and self-checks.

* test/poly_pois.F90:82-101  -- u = xyz, p = 1, two uniform refinements of
  the unit cube, H1 error < 1e-15 after every solve.
* test/conv_pois.F90:84-114  -- u = sin(pi x) sinh(pi y) z^2 (ISOL=2), p = 2,
  three refinements, H1 convergence rate of the last two in [1.95, 2.05].
* set_3D_int.F90:407-457 (HP3D_DEBUG self-check) -- Gauss rules integrate
  monomials to 1e-14.
Plus the known-answer properties of the element matrices: symmetry, the
constant function in the kernel of the Poisson stiffness, partition of unity
of the vertex functions, and agreement of the BLAS-3 (elem_opt) and scalar
(elem_poisson) element forms.
"""
import numpy as np
import pytest

from oracle import oracle as O
from hp3d_gb300 import mesh as M
import fem_harness as H


@pytest.mark.parametrize("n", [2, 4])
def test_poly_pois(n):
    m = M.structured_hexa(n, 1)
    zd = H.dirichlet_data(m, 12)
    els = H.oracle_element_outputs(m, 12, zdofd=zd)
    err, nrm, _, _ = H.solve_and_error(m, els, 12, zdofd=zd)
    assert err < 1e-15 * max(1.0, 1.0)


def test_conv_pois_rate():
    errs = []
    for n in (2, 4, 8):
        m = M.structured_hexa(n, 2)
        zd = H.dirichlet_data(m, 2)
        els = H.oracle_element_outputs(m, 2, zdofd=zd)
        err, _, _, _ = H.solve_and_error(m, els, 2, zdofd=zd)
        errs.append(err)
    rate = np.log(errs[-2] / errs[-1]) / np.log(2.0)
    assert 1.95 <= rate <= 2.05


@pytest.mark.parametrize("p,integration", [(1, 0), (3, 0), (5, 0), (5, 1), (6, 1)])
def test_monomial_integration(p, integration):
    xi, w = O.quad_hexa(M.pack_order_hexa(p), integration=integration)
    nq = min(p + integration, 6) + 1
    assert len(w) == nq ** 3
    deg = 2 * nq - 1
    for (i, j, k) in [(0, 0, 0), (deg, 0, 0), (deg, deg, deg), (1, deg - 1, 2)]:
        v = (xi[:, 0] ** i * xi[:, 1] ** j * xi[:, 2] ** k * w).sum()
        assert abs(v - 1.0 / ((i + 1) * (j + 1) * (k + 1))) < 1e-14


@pytest.mark.parametrize("p", [1, 2, 3, 5, 6])
def test_element_known_answers(p):
    m = M.random_orientations(M.structured_hexa(2, p, perturb=0.15, kappa_logrange=(-2, 2)), seed=p)
    e = 5
    K, b, rc = O.elem(1, m["norder"][e], m["nori_edge"][e], m["nori_face"][e], m["xvert"][e],
                      m["kappa"][e], isol=10, integration=0)
    K2, b2, _ = O.elem(1, m["norder"][e], m["nori_edge"][e], m["nori_face"][e], m["xvert"][e],
                       m["kappa"][e], isol=10, integration=0, variant=1)
    n = K.shape[0]
    assert rc == 0 and n == (p + 1) ** 3
    assert np.array_equal(K, K.T)
    c = np.zeros(n); c[:8] = 1.0
    assert np.abs(K @ c).max() <= 1e-13 * np.abs(K).max()
    assert np.abs(K - K2).max() <= 1e-13 * np.abs(K).max()
    assert np.abs(b - b2).max() <= 1e-13 * np.abs(b).max()
    s, g = O.shape_hexa([0.3, 0.6, 0.1], m["norder"][e], m["nori_edge"][e], m["nori_face"][e])
    assert abs(s[:8].sum() - 1.0) < 1e-15 and np.abs(g[:8].sum(0)).max() < 1e-15


def test_lu_vs_cholesky_condensation():
    m = M.structured_hexa(2, 5, perturb=0.15, kappa_logrange=(-2, 2))
    K, b, _ = O.elem(1, m["norder"][0], m["nori_edge"][0], m["nori_face"][0], m["xvert"][0],
                     m["kappa"][0], isol=10, integration=1)
    nb = O.nrdof_bubble(1, m["norder"][0])
    a1, b1, s1, t1, r1 = O.stc_fwd(K, b, nb, 0)
    a2, b2, s2, t2, r2 = O.stc_fwd(K, b, nb, 1)
    assert r1 == 0 and r2 == 0
    assert np.abs(a1 - a2).max() <= 1e-12 * np.abs(a1).max()
    assert np.abs(s1 - s2).max() <= 1e-12 * np.abs(s1).max()
    assert np.abs(b1 - b2).max() <= 1e-12 * np.abs(b1).max()


def test_index_maps_first_visit():
    m = M.structured_hexa(3, 2)
    ne = m["nelem"]
    nd = np.stack([O.node_ndof(1, m["norder"][e]) for e in range(ne)])
    ndofm = (nd * (1 - m["bcflag"])).astype(np.int32)
    nrdof, nfirst, lcon, off, nnz = O.index_maps(np.full(ne, 26), m["nodes"], ndofm, m["nnodes"])
    # every active global dof appears, numbering is 1..nrdof
    assert set(np.unique(lcon)) == set(range(1, nrdof + 1))
    # first element's connectivities: nodes in reverse order
    lc0 = lcon[off[0]:off[1]]
    assert lc0[0] == nfirst[m["nodes"][0, 25]] + 1 or ndofm[0, 25] == 0
