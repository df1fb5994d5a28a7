"""hp-adaptive batches: per-element anisotropic orders (min rule) and random
orientations, many bins in one pass (FP64 and mixed precision).

Each element is binned by its per-axis maximum orders; its dof are a signed
permutation of a subset of the bin element's dof.  Tolerances as in
test_gpu_parity (FP64 1e-12) and test_gpu_mixed (mixed 1e-12 element,
1e-10 condensed); index maps bit-exact.
"""
import numpy as np
import pytest

from oracle import oracle as O
from hp3d_gb300 import hp3dg as H
from hp3d_gb300 import mesh as M
import fem_harness as FH

pytestmark = pytest.mark.gpu


def _rel(a, b):
    return np.abs(a - b).max() / max(np.abs(b).max(), 1e-300)


@pytest.mark.parametrize("prec,orient", [(H.FP64, False), (H.FP64, True), (H.MIXED, True)])
def test_hp_element_and_condensed_parity(prec, orient):
    m = M.hp_hexa(3, seed=5, perturb=0.1, kappa_logrange=(-1, 1))
    if orient:
        m = M.random_orientations(m, seed=9)
    ep = H.ElementPass(prec, integration=0, isol=10, keep_elem=True)
    ep.submit(m)
    ep.run(); ep.download()
    ref = FH.oracle_element_outputs(m, 10)
    tol_c = 1e-12 if prec == H.FP64 else 1e-10
    for e in range(m["nelem"]):
        K, b, _ = O.elem(1, m["norder"][e], m["nori_edge"][e], m["nori_face"][e], m["xvert"][e],
                         m["kappa"][e], isol=10, integration=0)
        Kg, bg = ep.elem(e, K.shape[0])
        assert _rel(Kg, K) < 1e-12, (e, m["norder"][e], _rel(Kg, K))
        assert _rel(bg, b) < 1e-12
        zb, zs = ep.condensed(e)
        if zs.size:
            assert _rel(zs, ref[e]["zastif"]) < tol_c, e
            assert _rel(zb, ref[e]["zbload"]) < tol_c, e
        a, bs = ep.schur(e)
        if a.size:
            assert _rel(a, ref[e]["aschur"]) < 1e-10, e
    nrdof, nf, lc, lo, en = ep.index_map()
    ndofm = np.stack([r["ndofm"] for r in ref]).astype(np.int32)
    onr, onf, olc, olo, oen = O.index_maps(np.full(m["nelem"], 26), m["nodes"], ndofm, m["nnodes"])
    assert nrdof == onr and np.array_equal(nf, onf) and np.array_equal(lc, olc)


def test_hp_global_solution_matches_oracle():
    m = M.hp_hexa(4, seed=11, perturb=0.1, kappa_logrange=(-1, 1))
    ep = H.ElementPass(H.MIXED, integration=0, isol=10)
    ep.submit(m)
    ep.run(); ep.download()
    from test_gpu_parity import _gpu_elements
    x, _, _ = FH.assemble_solve(m, _gpu_elements(ep, m))
    ref = FH.oracle_element_outputs(m, 10)
    _, _, x_o, _ = FH.solve_and_error(m, ref, 10)
    assert np.abs(x - x_o).max() <= 1e-9 * np.abs(x_o).max()
