"""Constrained approximation (hanging nodes) on CPU: the restated transform
of celem_systemI.F90:541-760 with logic's coefficients.

Pin (the end-to-end form of test/poly_pois.F90 on a mesh with hanging
nodes): the centre element of a 3^3 mesh refined into 8 children, whose
nodes on the coarse faces are constrained; u = xyz and u = 1 + x + 2y + 3z
are reproduced to round-off.  A wrong coefficient (planted in the oracle's
inputs) breaks the reproduction, so the pin sees the constraints.
"""
import numpy as np
import pytest

import fem_harness as FH
import hanging_harness as HH
from oracle import oracle as O


@pytest.mark.parametrize("p,isol", [(1, 12), (2, 12), (3, 12), (2, 13)])
def test_polynomial_reproduced_with_hanging_nodes(p, isol):
    m, cons = HH.hanging_mesh(p)
    assert sum(c is not None for c in cons) == 8
    zd = FH.dirichlet_data(m, isol)
    els = HH.oracle_outputs(m, cons, isol, zd)
    err, nrm, _ = HH.solve_error(m, cons, els, isol, zd)
    assert err / nrm < 1e-12, err / nrm


def test_wrong_coefficient_is_seen():
    m, cons = HH.hanging_mesh(2)
    zd = FH.dirichlet_data(m, 12)
    c = next(c for c in cons if c is not None)
    q = int(np.argmax(np.abs(c["cv"]) < 0.99))  # a genuine (non-identity) coefficient
    c["cv"] = c["cv"].copy()
    c["cv"][q] *= 1.1
    els = HH.oracle_outputs(m, cons, 12, zd)
    err, nrm, _ = HH.solve_error(m, cons, els, 12, zd)
    assert err / nrm > 1e-6


def test_identity_constraints_change_nothing():
    rng = np.random.default_rng(0)
    ni = 26
    A = rng.standard_normal((ni, ni)); A = A + A.T
    b = rng.standard_normal(ni)
    k = np.arange(ni, dtype=np.int32)
    am, bm = O.constrain(A, b, k, k, np.ones(ni), ni)
    assert np.array_equal(am, A) and np.array_equal(bm, b)
