"""Geometry dof by projection of a geometry-block map on the GPU
(hp3dg_gdof_points + hp3dg_update_gdof, the reference's update_gdof) against
the oracle's restatement, and the projected geometry driving the pass.

The block is the unit cube of a spherical-shell sector (tests/gdof_harness.py
plays the reference's GMP block routine); the elements are the boxes of a
conforming mesh in the block with rotated local frames (every orientation
code).  Checked:
- every element's geometry dof equal the oracle's per-element projection
  (1e-12 relative), at p = 2, 4 and 6, and each node holds the values of its
  first element;
- 'Linear' elements keep vertex dof only for the nodes they visit first;
- with apply = 1 the pass runs on the projected geometry: the volume from the
  vertex loads with f = 1 converges to the shell sector's volume with p, and
  equals the pass with the same dof given through hp3dg_batch_set_geometry.
"""
import numpy as np
import pytest

import dpg_harness as DH
import gdof_harness as GH
from hp3d_gb300 import hp3dg as H
from hp3d_gb300 import mesh as M
from oracle import oracle as O

pytestmark = pytest.mark.gpu


def _maps(ep, m):
    eta = ep.gdof_points(m["xvert"])
    x, J = GH.shell_map(eta)
    return x, J


@pytest.mark.parametrize("p", [2, 4, 6])
def test_gdof_matches_the_oracle(p):
    m = DH.rotated_hexa_mesh(2 if p == 6 else 3, p, seed=p, grading=1.2)
    ep = H.ElementPass(H.FP64, integration=1, isol=11)
    ep.submit(m)
    x, J = _maps(ep, m)
    xn = ep.update_gdof(m["xvert"], x, J)
    scale = 1.5
    first = {}
    for e in range(m["nelem"]):
        ref = O.gdof_hexa(m["norder"][e], m["nori_edge"][e], m["nori_face"][e], m["xvert"][e],
                          GH.shell_map, integration=1)
        assert xn[e].shape == ref.shape
        assert np.abs(xn[e] - ref).max() <= 1e-12 * scale, (p, e)
        nd = O.node_ndof(M.HEXA, m["norder"][e])
        f = np.concatenate([[0], np.cumsum(nd)]).astype(int)
        for i in range(26):
            node = int(m["nodes"][e, i])
            v = xn[e][f[i]:f[i + 1]]
            if node in first:
                assert np.array_equal(v, first[node]), (e, i)  # copied from the first element
            else:
                first[node] = v
    ep.close()


def test_linear_elements():
    m = DH.rotated_hexa_mesh(2, 3, seed=1)
    ep = H.ElementPass(H.FP64, integration=1, isol=11)
    ep.submit(m)
    x, J = _maps(ep, m)
    lin = np.zeros(m["nelem"], np.int32)
    lin[0] = 1
    xn = ep.update_gdof(m["xvert"], x, J, linear=lin)
    nd = O.node_ndof(M.HEXA, m["norder"][0])
    f = np.concatenate([[0], np.cumsum(nd)]).astype(int)
    # element 0 is every one of its nodes' first element: vertices only
    assert np.abs(xn[0][8:]).max() == 0.0
    assert np.allclose(xn[0][:8], GH.shell_map(m["xvert"][0])[0], rtol=0, atol=1e-15)
    # a neighbour's shared edge carries element 0's (zero) values, its own
    # interior is projected
    shared = set(m["nodes"][0, 8:20].tolist())
    for e in range(1, m["nelem"]):
        nde = O.node_ndof(M.HEXA, m["norder"][e])
        fe = np.concatenate([[0], np.cumsum(nde)]).astype(int)
        for i in range(8, 20):
            if int(m["nodes"][e, i]) in shared:
                assert np.abs(xn[e][fe[i]:fe[i + 1]]).max() == 0.0
        assert np.abs(xn[e][fe[26]:]).max() > 0.0
    ep.close()


def _volume(m, apply=True):
    ep = H.ElementPass(H.FP64, integration=1, isol=11, keep_elem=True)
    ep.submit(m)
    x, J = _maps(ep, m)
    xn = ep.update_gdof(m["xvert"], x, J, apply=apply)
    if not apply:
        ep.set_geometry(xn)
    ep.run()
    ep.download()
    n = (m["p"] + 1) ** 3
    vol = sum(ep.elem(e, n)[1][:8].sum() for e in range(m["nelem"]))
    out = [ep.condensed(e) for e in range(m["nelem"])]
    ep.close()
    return vol, out


def test_projected_geometry_drives_the_pass():
    exact = GH.shell_volume()
    err = {}
    for p in (2, 4):
        m = M.structured_hexa(3, p, perturb=0.0, kappa_logrange=None, seed=3)
        vol, out = _volume(m)
        err[p] = abs(vol - exact) / exact
        vol2, out2 = _volume(m, apply=False)
        assert vol2 == vol
        for (zb, zs), (zb2, zs2) in zip(out, out2):
            assert np.array_equal(zb, zb2) and np.array_equal(zs, zs2)
    assert err[4] < err[2] / 20 and err[4] < 1e-5, err
