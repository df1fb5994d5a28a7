"""Prisms and the mixed hexa/prism/tet batch on the GPU against the oracle.

Element matrices and loads (1e-12 relative), condensed systems and Schur
blocks (1e-12 FP64 / 1e-10 mixed), index maps bit-exact; random triangle
(0..5) and quad (0..7) orientation codes on prisms; the hp-adaptive mixed
mesh (per-element orders, min rule, orientation codes from the conforming
builder) in one submit with many bins; end to end: poly_pois at order 3 on
the mixed mesh and the linear solution on the hp mixed mesh through the GPU
pass (H1 error < 1e-12 of the norm).
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


def _random_prism_orientations(m, seed):
    rng = np.random.default_rng(seed)
    m = dict(m)
    ne = m["nelem"]
    m["nori_edge"] = np.zeros((ne, 12), np.int32)
    m["nori_face"] = np.zeros((ne, 6), np.int32)
    m["nori_edge"][:, :9] = rng.integers(0, 2, (ne, 9))
    m["nori_face"][:, :2] = rng.integers(0, 6, (ne, 2))
    m["nori_face"][:, 2:5] = rng.integers(0, 8, (ne, 3))
    return m


def _check(m, prec, isol=10):
    ep = H.ElementPass(prec, isol=isol, keep_elem=True)
    ep.submit(m)
    ep.run(); ep.download()
    ref = FH.oracle_element_outputs(m, isol)
    tol_c = 1e-12 if prec == H.FP64 else 1e-10
    for e in range(m["nelem"]):
        et = int(m["etype"][e])
        nv = FH.type_info(et)[0]
        K, b, _ = O.elem(et, m["norder"][e], m["nori_edge"][e], m["nori_face"][e],
                         m["xvert"][e][:nv], m["kappa"][e], isol=isol)
        Kg, bg = ep.elem(e, K.shape[0])
        assert _rel(Kg, K) < 1e-12, (e, et, _rel(Kg, K))
        assert _rel(bg, b) < 1e-12, (e, et)
        zb, zs = ep.condensed(e)
        if zs.size:
            assert _rel(zs, ref[e]["zastif"]) < tol_c, (e, et)
            assert _rel(zb, ref[e]["zbload"]) < tol_c, (e, et)
        a, _ = ep.schur(e)
        if a.size:
            assert _rel(a, ref[e]["aschur"]) < 1e-10, (e, et)
    nrdof, nf, lc, lo, en = ep.index_map()
    ndofm = np.stack([r["ndofm"] for r in ref]).astype(np.int32)
    onr, onf, olc, olo, oen = O.index_maps(FH.nnode_of(m), m["nodes"], ndofm, m["nnodes"])
    assert nrdof == onr and np.array_equal(nf, onf) and np.array_equal(lc, olc)
    ep.close()


@pytest.mark.parametrize("ph,pz", [(3, 2), (6, 5)])
def test_prism_parity_random_orientations(ph, pz):
    m = _random_prism_orientations(
        M.structured_prism(2, ph, pz, perturb=0.15, kappa_logrange=(-2, 2), seed=2), 11)
    _check(m, H.FP64)


@pytest.mark.parametrize("prec", [H.FP64, H.MIXED])
def test_hp_mixed_mesh_parity(prec):
    m = M.mixed_mesh(4, a=0.5, b=0.5, perturb=0.1, seed=13)
    _check(m, prec)


def test_poly_pois_mixed_mesh_gpu():
    m = M.mixed_mesh(4, a=0.5, b=0.5, p=3, perturb=0.1, seed=7, kappa_logrange=None)
    zd = FH.dirichlet_data(m, 12)
    ep = H.ElementPass(H.FP64, isol=12)
    ep.submit(m, zdofd=zd)
    ep.run(); ep.download()
    err, nrm, _, _ = FH.solve_and_error(m, FH.gpu_elements(ep, m), 12, zdofd=zd)
    assert err < 1e-12 * nrm


def test_linear_solution_hp_mixed_mesh_gpu():
    m = M.mixed_mesh(4, a=0.5, b=0.5, perturb=0.1, seed=9, kappa_logrange=None)
    zd = FH.dirichlet_data(m, 13)
    ep = H.ElementPass(H.MIXED, isol=13)
    ep.submit(m, zdofd=zd)
    ep.run(); ep.download()
    err, nrm, x, _ = FH.solve_and_error(m, FH.gpu_elements(ep, m), 13, zdofd=zd)
    assert err < 1e-11 * nrm
    # the post-solve kernels on the mixed batch
    ep.backsub(x)
    e2, n2 = ep.element_error(13)
    assert np.sqrt(e2.sum()) < 1e-11 * np.sqrt(n2.sum())
