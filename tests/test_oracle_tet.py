"""Tetrahedron restatement in the oracle (shape3DHTet, the Duffy rule of
set_3D_int) pinned by properties the reference checks or relies on:

* the Duffy rule integrates monomials of degree <= 2p exactly -- the
  reference's own self-check compares it with the triangle rule to 1e-13
  (quadrature/gauss_quadrature.F90:789-841);
* the H1 space of order p is complete (all polynomials of degree <= p);
* vertex functions are a partition of unity; gradients match finite
  differences; edge / face / bubble functions vanish where H1 conformity
  needs them to; orientation codes {0,4}, {1,5}, {2,3} differ by (-1)^i;
* end to end: test/poly_pois.F90 (u = xyz reproduced, H1 error < 1e-13)
  and test/conv_pois.F90 (p=2, H1 rate ~2) restated on conforming Kuhn
  tetrahedral meshes through the harness's direct solve.
"""
import math

import numpy as np
import pytest

from oracle import oracle as O
from hp3d_gb300 import mesh as M
import fem_harness as FH


def _no(p):
    a = np.zeros(19, np.int32)
    a[:11] = p
    return a


@pytest.mark.parametrize("p", [1, 2, 3, 4, 5, 6])
def test_duffy_rule_exact_to_degree_2p(p):
    xi, w = O.quad_tet(_no(p))
    assert len(w) == (p + 1) ** 2 * (p + 2)
    for i in range(2 * p + 1):
        for j in range(2 * p + 1 - i):
            for k in range(2 * p + 1 - i - j):
                ex = math.factorial(i) * math.factorial(j) * math.factorial(k) / math.factorial(i + j + k + 3)
                v = (w * xi[:, 0] ** i * xi[:, 1] ** j * xi[:, 2] ** k).sum()
                assert abs(v - ex) <= 1e-13 * ex


@pytest.mark.parametrize("p", [1, 3, 6])
def test_tet_shape_complete_and_consistent(p):
    rng = np.random.default_rng(p)
    no = _no(p)
    ne, nf = rng.integers(0, 2, 12), rng.integers(0, 6, 6)
    n = O.nrdofH(O.TET, no)
    assert n == (p + 1) * (p + 2) * (p + 3) // 6
    x = np.array([0.2, 0.15, 0.3])
    s, g = O.shape_tet(x, no, ne, nf)
    assert abs(s[:4].sum() - 1.0) < 1e-15
    h = 1e-6
    for c in range(3):
        xp, xm = x.copy(), x.copy()
        xp[c] += h; xm[c] -= h
        fd = (O.shape_tet(xp, no, ne, nf)[0] - O.shape_tet(xm, no, ne, nf)[0]) / (2 * h)
        assert np.abs(fd - g[:, c]).max() < 1e-7 * max(1.0, np.abs(g).max())
    pts = rng.random((4000, 3))
    pts = pts[pts.sum(1) < 1][:2 * n + 20]
    A = np.array([O.shape_tet(q, no, ne, nf)[0] for q in pts])
    mons = [(i, j, k) for i in range(p + 1) for j in range(p + 1 - i) for k in range(p + 1 - i - j)]
    B = np.array([[q[0] ** i * q[1] ** j * q[2] ** k for (i, j, k) in mons] for q in pts])
    coef, _, rank, _ = np.linalg.lstsq(A, B, rcond=None)
    assert rank == n and np.abs(A @ coef - B).max() < 1e-10


def test_tet_orientation_classes_and_traces():
    p = 6
    no = _no(p)
    rng = np.random.default_rng(1)
    x = np.array([0.1, 0.2, 0.3])
    nfun = (p - 1) * (p - 2) // 2
    off = 4 + 6 * (p - 1)
    for a, b in [(0, 4), (1, 5), (2, 3)]:
        sa, _ = O.shape_tet(x, no, None, np.full(6, a))
        sb, _ = O.shape_tet(x, no, None, np.full(6, b))
        k = 0
        for nij in range(3, p + 1):
            for i in range(2, nij):
                for f in range(4):
                    q = off + f * nfun + k
                    assert abs(sb[q] - (-1) ** i * sa[q]) < 1e-15
                k += 1
    V = np.array([[0, 0, 0], [1, 0, 0], [0, 1, 0], [0, 0, 1]], float)
    for f, (a, b, c) in enumerate(M.TET_FACES):
        u, v = 0.3, 0.5
        q = V[a] + u * (V[b] - V[a]) + v * (V[c] - V[a])
        s, _ = O.shape_tet(q, no, rng.integers(0, 2, 12), rng.integers(0, 6, 6))
        assert np.abs(s[off + 4 * nfun:]).max() < 1e-14  # bubbles
        for g in range(4):
            if g != f:
                assert np.abs(s[off + g * nfun: off + (g + 1) * nfun]).max() < 1e-14


@pytest.mark.parametrize("p", [3, 4])
def test_poly_pois_tets(p):
    """u = xyz is in the space for p >= 3: the solution is reproduced."""
    m = M.structured_tet(2, p, perturb=0.15, seed=3)
    zd = FH.dirichlet_data(m, 12)
    ref = FH.oracle_element_outputs(m, 12, zdofd=zd)
    err, nrm, _, _ = FH.solve_and_error(m, ref, 12, zdofd=zd)
    assert err < 1e-12 * nrm


def test_conv_pois_tets_rate():
    # Kuhn meshes are pre-asymptotic below n = 4 (rates 1.02, 1.77, 1.91)
    errs = []
    for n in (4, 8):
        m = M.structured_tet(n, 2)
        ref = FH.oracle_element_outputs(m, 10)
        err, _, _, _ = FH.solve_and_error(m, ref, 10)
        errs.append(err)
    rate = math.log(errs[0] / errs[1], 2)
    assert 1.85 < rate < 2.1, rate
