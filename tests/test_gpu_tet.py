"""Tetrahedra on the GPU: element matrices and loads, condensed systems,
Schur blocks and index maps against the oracle (shape3DHTet, the Duffy rule
of set_3D_int), with random edge/face orientation codes (all six OrientTri
codes) and per-element orders (min rule), in FP64 and mixed precision; the
end-to-end pins (poly_pois, a global solve, element errors) through the GPU.

Tolerances: element matrices 1e-12 relative (FP64 pass; the mixed pass
recombines to FP64 round-off as well), condensed outputs 1e-12 (FP64) /
1e-10 (mixed), index maps bit-exact.
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


def _random_tet_orientations(m, seed):
    rng = np.random.default_rng(seed)
    m = dict(m)
    ne = m["nelem"]
    m["nori_edge"] = np.zeros((ne, 12), np.int32)
    m["nori_face"] = np.zeros((ne, 6), np.int32)
    m["nori_edge"][:, :6] = rng.integers(0, 2, (ne, 6))
    m["nori_face"][:, :4] = rng.integers(0, 6, (ne, 4))
    return m


@pytest.mark.parametrize("prec,kind", [(H.FP64, "uniform"), (H.FP64, "hp"), (H.MIXED, "hp")])
def test_tet_parity(prec, kind):
    if kind == "uniform":
        m = _random_tet_orientations(M.structured_tet(2, 5, perturb=0.15, kappa_logrange=(-2, 2)), 3)
    else:
        m = _random_tet_orientations(M.hp_tet(2, seed=4, perturb=0.15), 5)
    ep = H.ElementPass(prec, isol=10, keep_elem=True)
    ep.submit(m)
    ep.run(); ep.download()
    ref = FH.oracle_element_outputs(m, 10)
    tol_c = 1e-12 if prec == H.FP64 else 1e-10
    for e in range(m["nelem"]):
        K, b, _ = O.elem(3, m["norder"][e], m["nori_edge"][e], m["nori_face"][e],
                         m["xvert"][e][:4], m["kappa"][e], isol=10)
        Kg, bg = ep.elem(e, K.shape[0])
        assert _rel(Kg, K) < 1e-12, (e, _rel(Kg, K))
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
    onr, onf, olc, olo, oen = O.index_maps(FH.nnode_of(m), m["nodes"], ndofm, m["nnodes"])
    assert nrdof == onr and np.array_equal(nf, onf) and np.array_equal(lc, olc)
    assert np.array_equal(en, oen)


@pytest.mark.parametrize("p", [3, 5])
def test_poly_pois_tets_gpu(p):
    m = M.structured_tet(2, p, perturb=0.15, seed=3)
    zd = FH.dirichlet_data(m, 12)
    ep = H.ElementPass(H.FP64, isol=12)
    ep.submit(m, zdofd=zd)
    ep.run(); ep.download()
    err, nrm, _, _ = FH.solve_and_error(m, FH.gpu_elements(ep, m), 12, zdofd=zd)
    assert err < 1e-12 * nrm


def test_tet_solution_error_and_backsub_match_oracle():
    m = M.hp_tet(3, seed=6, perturb=0.1)
    ep = H.ElementPass(H.MIXED, isol=10)
    ep.submit(m)
    ep.run(); ep.download()
    x, _, _ = FH.assemble_solve(m, FH.gpu_elements(ep, m))
    ref = FH.oracle_element_outputs(m, 10)
    err_o, nrm_o, x_o, dofs_o = FH.solve_and_error(m, ref, 10)
    assert np.abs(x - x_o).max() <= 1e-10 * np.abs(x_o).max()
    ep.backsub(x_o)
    for e in range(m["nelem"]):
        d = ep.dofs(e)
        assert np.abs(d - dofs_o[e]).max() <= 1e-9 * max(np.abs(dofs_o[e]).max(), 1e-30)
    e2, n2 = ep.element_error(10)
    assert abs(np.sqrt(e2.sum()) - err_o) <= 1e-9 * err_o
    assert abs(np.sqrt(n2.sum()) - nrm_o) <= 1e-12 * nrm_o
