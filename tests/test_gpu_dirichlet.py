"""update_Ddof on the GPU (hp3dg_dirichlet_dofs) against the oracle, and the
projected data used end to end."""
import numpy as np
import pytest

import dpg_harness as DH
import fem_harness as FH
from hp3d_gb300 import hp3dg as H
from hp3d_gb300 import mesh as M
from oracle import oracle as O

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("p", [2, 4, 6])
def test_dirichlet_dofs_match_oracle(p):
    m = DH.rotated_hexa_mesh(3, p, seed=9, grading=1.2)
    ep = H.ElementPass(H.FP64, isol=10)
    ep.submit(m)
    zg = ep.dirichlet_dofs(10)
    for e in range(m["nelem"]):
        z = O.dirichlet_hexa(m["norder"][e], m["nori_edge"][e], m["nori_face"][e], m["xvert"][e],
                             m["bcflag"][e], 10)
        assert len(zg[e]) == len(z)
        assert np.abs(zg[e] - z).max() <= 1e-12 * max(1.0, np.abs(z).max()), e
    ep.close()


def test_projected_data_solve_end_to_end():
    m = M.structured_hexa(3, 3, perturb=0.0, seed=2)
    ep = H.ElementPass(H.FP64, isol=12)
    ep.submit(m)
    zd = ep.dirichlet_dofs(12)
    ep.submit(m, zdofd=zd)
    ep.run(); ep.download()
    err, nrm, _, _ = FH.solve_and_error(m, FH.gpu_elements(ep, m), 12, zdofd=zd)
    assert err / nrm < 1e-12
    ep.close()
