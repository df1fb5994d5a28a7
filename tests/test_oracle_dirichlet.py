"""Dirichlet data by projection-based interpolation (update_Ddof,
hpinterp/update_Ddof.F90 with dhpvert / dhpedgeH / dhpfaceH) restated in the
oracle, on CPU:

- data in the trace space are interpolated exactly (they agree with the
  harness's independent least-squares projection);
- the values of a node depend only on its trace: every element sharing a
  boundary node computes the same dof (the reference computes each node once),
  on a perturbed mesh with every orientation code and non-polynomial data.
"""
import numpy as np
import pytest

import dpg_harness as DH
import fem_harness as FH
from hp3d_gb300 import mesh as M
from oracle import oracle as O


@pytest.mark.parametrize("isol", [12, 13])
def test_in_space_data_interpolated_exactly(isol):
    m = M.structured_hexa(3, 4, perturb=0.0, seed=2)
    z2 = FH.dirichlet_data(m, isol)
    for e in range(m["nelem"]):
        z1 = O.dirichlet_hexa(m["norder"][e], m["nori_edge"][e], m["nori_face"][e], m["xvert"][e],
                              m["bcflag"][e], isol)
        assert np.abs(z1 - z2[e]).max() < 1e-12


def test_node_values_agree_between_elements():
    m = DH.rotated_hexa_mesh(3, 4, seed=9, grading=1.2)
    assert len(np.unique(m["nori_face"])) >= 4
    seen = {}
    for e in range(m["nelem"]):
        z = O.dirichlet_hexa(m["norder"][e], m["nori_edge"][e], m["nori_face"][e], m["xvert"][e],
                             m["bcflag"][e], 10)
        nd = O.node_ndof(M.HEXA, m["norder"][e])
        first = np.concatenate([[0], np.cumsum(nd)]).astype(int)
        for i in range(26):
            if not m["bcflag"][e, i] or nd[i] == 0:
                continue
            g = int(m["nodes"][e, i])
            v = z[first[i]:first[i + 1]]
            if g in seen:
                assert np.abs(seen[g] - v).max() < 1e-12 * max(1.0, np.abs(v).max())
            else:
                seen[g] = v
    assert len(seen) > 50
