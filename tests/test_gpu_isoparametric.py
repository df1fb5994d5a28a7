"""Isoparametric (curved) geometry: the element pass with the elements'
nrdofH geometry dof (nodcor, constrs/nodcor.F90:19-196, as geom3D consumes
them, element/util/geom3D.F90:30-112) against the oracle's elem_opt with the
same Xnod.

- Geometry dof equal to the vertex coordinates with zero higher-order dof
  reproduce the vertex-geometry pass (hexahedra, prisms, tetrahedra).
- Curved elements (random higher-order geometry dof, every element's own
  orientation codes): element matrices and loads within 1e-12 of the oracle
  (FP64; 1e-9 for the mixed contraction), condensed systems and Schur blocks
  within 1e-12 / 1e-11.
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


def _xnod(m, amp, seed):
    """Per element (nrdofH, 3): the vertex coordinates, then random
    higher-order dof of size amp times the element size."""
    rng = np.random.default_rng(seed)
    out = []
    for e in range(m["nelem"]):
        et = int(m["etype"][e]) if "etype" in m else 1
        nv = FH.type_info(et)[0]
        n = O.nrdofH(et, m["norder"][e])
        x = np.zeros((n, 3))
        xv = np.asarray(m["xvert"][e])[:nv]
        x[:nv] = xv
        h = np.ptp(xv, axis=0).max()
        x[nv:] = amp * h * rng.uniform(-1, 1, (n - nv, 3))
        out.append(x)
    return out


def _meshes():
    hexa = M.random_orientations(M.structured_hexa(2, 3, perturb=0.1, seed=4), seed=9)
    return [("hexa", hexa), ("prism", M.structured_prism(2, 3, 2, perturb=0.1, seed=5)),
            ("tet", M.structured_tet(2, 3, perturb=0.1, seed=6))]


@pytest.mark.parametrize("which", [0, 1, 2])
def test_vertex_dofs_reproduce_vertex_geometry(which):
    name, m = _meshes()[which]
    ep = H.ElementPass(H.FP64, isol=10, keep_elem=True)
    ep.submit(m)
    ep.run(); ep.download()
    ref = []
    for e in range(m["nelem"]):
        n = O.nrdofH(int(m["etype"][e]) if "etype" in m else 1, m["norder"][e])
        ref.append(ep.elem(e, n))
    ep.set_geometry(_xnod(m, 0.0, 1))
    ep.run(); ep.download()
    for e in range(m["nelem"]):
        K, b = ep.elem(e, ref[e][0].shape[0])
        assert _rel(K, ref[e][0]) < 1e-13 and _rel(b, ref[e][1]) < 1e-13, (name, e)
    ep.close()


@pytest.mark.parametrize("which,prec,tol", [(0, H.FP64, 1e-12), (1, H.FP64, 1e-12),
                                            (2, H.FP64, 1e-12), (0, H.MIXED, 1e-9)])
def test_curved_element_matrices_match_oracle(which, prec, tol):
    name, m = _meshes()[which]
    xn = _xnod(m, 0.01, 2 + which)
    ep = H.ElementPass(prec, isol=10, keep_elem=True)
    ep.submit(m)
    ep.set_geometry(xn)
    ep.run(); ep.download()
    for e in range(m["nelem"]):
        et = int(m["etype"][e]) if "etype" in m else 1
        K, b, rc = O.elem(et, m["norder"][e], m["nori_edge"][e], m["nori_face"][e], xn[e],
                          m["kappa"][e], isol=10)
        assert rc == 0
        Kg, bg = ep.elem(e, K.shape[0])
        assert _rel(Kg, K) < tol and _rel(bg, b) < tol, (name, e, _rel(Kg, K), _rel(bg, b))
    ep.close()


def test_curved_condensed_outputs_match_oracle():
    m = M.random_orientations(M.structured_hexa(3, 4, perturb=0.1, seed=8), seed=3)
    xn = _xnod(m, 0.01, 7)
    ep = H.ElementPass(H.FP64, isol=10)
    ep.submit(m)
    ep.set_geometry(xn)
    ep.run(); ep.download()
    for e in range(m["nelem"]):
        K, b, rc = O.elem(1, m["norder"][e], m["nori_edge"][e], m["nori_face"][e], xn[e],
                          m["kappa"][e], isol=10)
        nb = O.nrdof_bubble(1, m["norder"][e])
        aii, bi, asch, bsch, rc = O.stc_fwd(K, b, nb, 0)
        assert rc == 0
        _, zb, zs, _ = O.celem_compress(1, m["norder"][e], m["bcflag"][e], aii, bi, None)
        zbg, zsg = ep.condensed(e)
        assert _rel(zsg, zs) < 1e-12 and _rel(zbg, zb) < 1e-12, e
        a, bs = ep.schur(e)
        assert _rel(a, asch) < 1e-11 and _rel(bs, bsch) < 1e-11, e
    # back to the vertex geometry: the post kernels are available again
    ep.set_geometry(None)
    ep.run(); ep.download()
    ep.close()
