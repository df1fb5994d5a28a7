"""Geometry dof by projection-based interpolation of a block map (update_gdof,
hpinterp/update_gdof.F90 with hpvert / hpedge / hpface / hpmdle) restated in
the oracle, on CPU:

- a polynomial block map inside the element's space is reproduced exactly,
  on sub-boxes of the block and under every orientation code;
- a spherical-shell map converges with p (max point error falls by more than
  an order of magnitude from p = 2 to p = 4 and again to p = 6);
- every element sharing a node computes the same dof for it (the reference
  projects each node once), on a conforming mesh with rotated local frames;
- a 'Linear' block keeps vertex dof only.
"""
import numpy as np
import pytest

import dpg_harness as DH
import gdof_harness as GH
from hp3d_gb300 import mesh as M
from oracle import oracle as O


def _box(lo, hi):
    off = np.array([(0, 0, 0), (1, 0, 0), (1, 1, 0), (0, 1, 0), (0, 0, 1), (1, 0, 1), (1, 1, 1),
                    (0, 1, 1)], float)
    return lo + off * (np.asarray(hi) - np.asarray(lo))


@pytest.mark.parametrize("p", [2, 3, 4])
def test_polynomial_map_reproduced(p):
    rng = np.random.default_rng(p)
    norder = [p] * 12 + [p * 11] * 6 + [p * 111]
    for trial in range(4):
        ne = rng.integers(0, 2, 12)
        nf = rng.integers(0, 8, 6)
        lo = rng.uniform(0, 0.5, 3)
        etav = _box(lo, lo + rng.uniform(0.2, 0.5, 3))
        xn = O.gdof_hexa(norder, ne, nf, etav, GH.poly_map)
        for xi in rng.uniform(0, 1, (6, 3)):
            x = GH.eval_geometry(O, xn, norder, ne, nf, xi)
            want, _ = GH.poly_map(GH.eta_of(etav, xi))
            assert np.abs(x - want).max() < 1e-12, (p, trial)


def test_shell_map_converges_with_p():
    etav = _box([0.25, 0.0, 0.5], [0.5, 0.5, 1.0])
    rng = np.random.default_rng(3)
    pts = rng.uniform(0, 1, (40, 3))
    err = {}
    for p in (2, 4, 6):
        norder = [p] * 12 + [p * 11] * 6 + [p * 111]
        xn = O.gdof_hexa(norder, [0] * 12, [0] * 6, etav, GH.shell_map)
        err[p] = max(np.abs(GH.eval_geometry(O, xn, norder, [0] * 12, [0] * 6, xi)
                            - GH.shell_map(GH.eta_of(etav, xi))[0]).max() for xi in pts)
    assert err[4] < err[2] / 10 and err[6] < err[4] / 10 and err[6] < 1e-5, err


def test_node_dof_agree_between_elements():
    m = DH.rotated_hexa_mesh(2, 4, seed=5, grading=1.3)
    assert len(np.unique(m["nori_face"])) >= 4
    seen = {}
    for e in range(m["nelem"]):
        xn = O.gdof_hexa(m["norder"][e], m["nori_edge"][e], m["nori_face"][e], m["xvert"][e],
                         GH.shell_map)
        nd = O.node_ndof(M.HEXA, m["norder"][e])
        first = np.concatenate([[0], np.cumsum(nd)]).astype(int)
        for i in range(26):
            if nd[i] == 0:
                continue
            v = xn[first[i]:first[i + 1]]
            node = int(m["nodes"][e, i])
            if node in seen:
                assert np.abs(v - seen[node]).max() < 1e-12 * max(1.0, np.abs(v).max()), (e, i)
            else:
                seen[node] = v


def test_linear_block_keeps_vertices_only():
    norder = [3] * 12 + [33] * 6 + [333]
    etav = _box([0, 0, 0], [0.5, 0.5, 0.5])
    xn = O.gdof_hexa(norder, [0] * 12, [0] * 6, etav, GH.shell_map, linear=True)
    assert np.array_equal(xn[8:], np.zeros_like(xn[8:]))
    for v in range(8):
        assert np.allclose(xn[v], GH.shell_map(etav[v])[0], rtol=0, atol=1e-15)
