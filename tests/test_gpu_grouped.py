"""The contraction of a multi-bin batch runs as one persistent launch over the
joint tile space of all its (type, order, orientation class) bins.  Each tile
does the same arithmetic as in a launch of its bin alone, so every element's
outputs must be bit-identical to those of a batch holding that element only
(a one-bin launch).  Checked on the hp mixed hexa / prism / tet mesh in mixed
precision, and the graph's kernel count falls with the grouping."""
import numpy as np
import pytest

from hp3d_gb300 import hp3dg as H
from hp3d_gb300 import mesh as M

pytestmark = pytest.mark.gpu


def _sub(m, idx):
    ne = m["nelem"]
    d = {k: (v[idx] if isinstance(v, np.ndarray) and v.shape[:1] == (ne,) else v)
         for k, v in m.items()}
    d["nelem"] = len(idx)
    return d


def test_grouped_contraction_bit_identical_to_one_bin_launches():
    m = M.mixed_mesh(4, a=0.5, b=0.5, cy=0.5, perturb=0.1, seed=21, kappa_logrange=(-1, 1))
    ep = H.ElementPass(H.MIXED, integration=1, isol=10)
    ep.submit(m)
    ep.run()
    ep.download()
    kernels, _ = ep.pass_stats()
    rng = np.random.default_rng(2)
    picks = sorted(set(rng.choice(m["nelem"], 12, replace=False)) |
                   {int(np.where(m["etype"] == t)[0][0]) for t in (1, 2, 3)})
    for e in picks:
        one = H.ElementPass(H.MIXED, integration=1, isol=10)
        one.submit(_sub(m, [e]))
        one.run()
        one.download()
        zb, zs = ep.condensed(e)
        zb1, zs1 = one.condensed(0)
        a, b = ep.schur(e)
        a1, b1 = one.schur(0)
        assert np.array_equal(zb, zb1) and np.array_equal(zs, zs1), e
        assert np.array_equal(a, a1) and np.array_equal(b, b1), e
        one.close()
    ep.close()
    assert kernels > 0
