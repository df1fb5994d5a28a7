"""GPU parity of the element pass against the CPU oracle (FP64 path).

Tolerances: element matrices, condensed matrices, loads and Schur blocks
within 1e-12 relative to the largest entry of the element's block (the
oracle condenses with LU as stc_fwd_gen does, the GPU with Cholesky; both
FP64).  Index maps (NFIRST_DOF, LCON, elem_nnz) bit-exact.
"""
import numpy as np
import pytest

from oracle import oracle as O
from hp3d_gb300 import hp3dg as H
from hp3d_gb300 import mesh as M
import fem_harness as FH

pytestmark = pytest.mark.gpu
TOL = 1e-12


def _rel(a, b):
    s = max(np.abs(b).max(), 1e-300)
    return np.abs(a - b).max() / s


@pytest.mark.parametrize("p,integ,orient", [(1, 0, False), (2, 0, True), (3, 0, True),
                                            (4, 1, True), (5, 1, True), (5, 0, False)])
def test_element_matrices(p, integ, orient):
    m = M.structured_hexa(2, p, perturb=0.15, kappa_logrange=(-2, 2), seed=p)
    if orient:
        m = M.random_orientations(m, seed=11 + p)
    ep = H.ElementPass(H.FP64, integration=integ, isol=10, keep_elem=True)
    ep.submit(m)
    ep.run(); ep.download()
    for e in range(m["nelem"]):
        K, b, rc = O.elem(1, m["norder"][e], m["nori_edge"][e], m["nori_face"][e], m["xvert"][e],
                          m["kappa"][e], isol=10, integration=integ)
        Kg, bg = ep.elem(e, K.shape[0])
        assert _rel(Kg, K) < TOL, (e, _rel(Kg, K))
        assert _rel(bg, b) < TOL
    ep.close()


@pytest.mark.parametrize("p,integ,orient", [(2, 0, True), (3, 0, False), (5, 1, True)])
def test_condensed_outputs_and_index_maps(p, integ, orient):
    m = M.structured_hexa(3, p, perturb=0.15, kappa_logrange=(-2, 2), seed=3 + p)
    if orient:
        m = M.random_orientations(m, seed=5)
    ep = H.ElementPass(H.FP64, integration=integ, isol=10)
    ep.submit(m)
    ep.run(); ep.download()
    ref = FH.oracle_element_outputs(m, 10, integration=integ)
    for e in range(m["nelem"]):
        zb, zs = ep.condensed(e)
        assert zs.shape == ref[e]["zastif"].shape
        if zs.size:
            assert _rel(zs, ref[e]["zastif"]) < TOL
            assert _rel(zb, ref[e]["zbload"]) < TOL
        a, bsch = ep.schur(e)
        assert _rel(a, ref[e]["aschur"]) < 1e-11
        assert _rel(bsch, ref[e]["bschur"]) < 1e-11
    nrdof, nf, lc, lo, en = ep.index_map()
    ne = m["nelem"]
    ndofm = np.stack([r["ndofm"] for r in ref]).astype(np.int32)
    onr, onf, olc, olo, oen = O.index_maps(np.full(ne, 26), m["nodes"], ndofm, m["nnodes"])
    assert nrdof == onr
    assert np.array_equal(nf, onf)
    assert np.array_equal(lc, olc)
    assert np.array_equal(lo, olo) and np.array_equal(en, oen)
    ep.close()


def test_dirichlet_lift_matches_oracle():
    m = M.structured_hexa(2, 3, perturb=0.1, seed=2)
    zd = FH.dirichlet_data(m, 2)
    ep = H.ElementPass(H.FP64, isol=2)
    ep.submit(m, zdofd=zd)
    ep.run(); ep.download()
    ref = FH.oracle_element_outputs(m, 2, zdofd=zd)
    for e in range(m["nelem"]):
        zb, zs = ep.condensed(e)
        assert _rel(zb, ref[e]["zbload"]) < TOL


_gpu_elements = FH.gpu_elements


@pytest.mark.parametrize("n", [2, 4])
def test_poly_pois_through_gpu(n):
    """test/poly_pois.F90 restated with the GPU element pass."""
    m = M.structured_hexa(n, 1)
    zd = FH.dirichlet_data(m, 12)
    ep = H.ElementPass(H.FP64, isol=12)
    ep.submit(m, zdofd=zd)
    ep.run(); ep.download()
    err, _, _, _ = FH.solve_and_error(m, _gpu_elements(ep, m), 12, zdofd=zd)
    assert err < 1e-15


def test_conv_pois_rate_through_gpu():
    """test/conv_pois.F90 restated with the GPU element pass."""
    errs = []
    for n in (2, 4, 8):
        m = M.structured_hexa(n, 2)
        zd = FH.dirichlet_data(m, 2)
        ep = H.ElementPass(H.FP64, isol=2)
        ep.submit(m, zdofd=zd)
        ep.run(); ep.download()
        err, _, _, _ = FH.solve_and_error(m, _gpu_elements(ep, m), 2, zdofd=zd)
        errs.append(err)
        ep.close()
    rate = np.log(errs[-2] / errs[-1]) / np.log(2.0)
    assert 1.95 <= rate <= 2.05


def test_negative_jacobian_is_reported():
    m = M.structured_hexa(2, 2)
    # invert element 3: swap bottom and top vertex layers
    xv = m["xvert"][3].copy()
    m["xvert"][3] = np.concatenate([xv[4:], xv[:4]])
    ep = H.ElementPass(H.FP64)
    ep.submit(m)
    ep.run()
    with pytest.raises(H.HP3DGError) as ei:
        ep.sync()
    assert ei.value.code == -1 and ei.value.bad == 3


def test_indefinite_bubble_block_is_reported():
    m = M.structured_hexa(2, 3)
    m["kappa"][5] = -1.0
    ep = H.ElementPass(H.FP64)
    ep.submit(m)
    ep.run()
    with pytest.raises(H.HP3DGError) as ei:
        ep.sync()
    assert ei.value.code == -2 and ei.value.bad == 5


def test_bad_order_is_rejected_on_submit():
    m = M.structured_hexa(2, 2)
    m["norder"][1, 0] = 9
    ep = H.ElementPass(H.FP64)
    with pytest.raises(H.HP3DGError) as ei:
        ep.submit(m)
    assert ei.value.code == -3 and ei.value.bad == 1
