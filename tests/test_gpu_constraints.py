"""Constrained approximation on the GPU (hp3dg_batch_submit_constrained)
against the oracle: the centre element of a 3^3 mesh refined into 8
children with hanging nodes on the coarse faces.

- the constrained, compressed element systems of every element equal the
  oracle's (celem_systemI.F90:541-760 restated) within 1e-12 in FP64 and
  1e-10 in mixed precision (relative to the matrix norm);
- NFIRST_DOF / LCON over the modified nodes are bit-exact;
- u = xyz is reproduced from the GPU outputs;
- identity constraints on a conforming mesh change nothing.
"""
import numpy as np
import pytest

import fem_harness as FH
import hanging_harness as HH
from hp3d_gb300 import hp3dg as H
from hp3d_gb300 import mesh as M

pytestmark = pytest.mark.gpu


def _rel(a, b):
    return np.abs(a - b).max() / max(np.abs(b).max(), 1e-300)


@pytest.mark.parametrize("prec,tol", [(H.FP64, 1e-12), (H.MIXED, 1e-10)])
@pytest.mark.parametrize("p", [2, 3])
def test_constrained_outputs_match_oracle(prec, tol, p):
    m, cons = HH.hanging_mesh(p)
    zd = FH.dirichlet_data(m, 12)
    ref = HH.oracle_outputs(m, cons, 12, zd)
    ep = H.ElementPass(prec, isol=12)
    ep.submit(m, zdofd=zd, constraints=cons)
    ep.run(); ep.download()
    for e in range(m["nelem"]):
        zb, zs = ep.condensed(e)
        assert zs.shape == ref[e]["zastif"].shape, e
        assert _rel(zs, ref[e]["zastif"]) < tol, (e, _rel(zs, ref[e]["zastif"]))
        assert _rel(zb, ref[e]["zbload"]) < tol, e
    nr, nf, lc, lo, en = ep.index_map()
    _, _, (nr0, nf0, lc0, lo0, en0) = HH.solve_error(m, cons, ref, 12, zd)
    assert nr == nr0
    assert np.array_equal(lc, lc0) and np.array_equal(lo, lo0) and np.array_equal(en, en0)
    vis = nf0 >= 0
    assert np.array_equal(nf[vis], nf0[vis])
    ep.close()


def test_polynomial_reproduced_from_gpu_outputs():
    m, cons = HH.hanging_mesh(3)
    zd = FH.dirichlet_data(m, 12)
    ref = HH.oracle_outputs(m, cons, 12, zd)
    ep = H.ElementPass(H.MIXED, isol=12)
    ep.submit(m, zdofd=zd, constraints=cons)
    ep.run(); ep.download()
    els = []
    for e in range(m["nelem"]):
        zb, zs = ep.condensed(e)
        asch, bsch = ep.schur(e)
        el = dict(ref[e])
        el.update(zbload=zb, zastif=zs, aschur=asch, bschur=bsch)
        els.append(el)
    err, nrm, _ = HH.solve_error(m, cons, els, 12, zd)
    assert err / nrm < 1e-9, err / nrm
    with pytest.raises(H.HP3DGError):
        ep.backsub(np.zeros(10))
    ep.close()


def test_identity_constraints_change_nothing():
    m = M.structured_hexa(3, 2, perturb=0.1, seed=1)
    ref = H.ElementPass(H.FP64, isol=10)
    ref.submit(m); ref.run(); ref.download()
    cons = [None] * m["nelem"]
    for e in (4, 13, 22):  # interior and boundary elements
        nd = np.array([1] * 8 + [1] * 12 + [1] * 6, np.int32)
        ni = int(nd.sum())
        cons[e] = dict(nodm=m["nodes"][e, :26], ndof=nd, bc=m["bcflag"][e, :26],
                       ck=np.arange(ni), cl=np.arange(ni), cv=np.ones(ni))
    ep = H.ElementPass(H.FP64, isol=10)
    ep.submit(m, constraints=cons)
    ep.run(); ep.download()
    for e in range(m["nelem"]):
        zb0, zs0 = ref.condensed(e)
        zb, zs = ep.condensed(e)
        assert np.array_equal(zs, zs0) and np.array_equal(zb, zb0), e
    assert ref.index_map()[0] == ep.index_map()[0]
    assert all(np.array_equal(x, y) for x, y in zip(ref.index_map()[1:], ep.index_map()[1:]))
    ep.close(); ref.close()
