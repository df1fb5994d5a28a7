"""A multi-bin batch runs its per-element kernels as grouped launches over
all its (type, order, orientation class) bins: stage 0 (orientation maps,
geometry, loads, digit slicing) and the condensation through segment tables,
the mixed-precision contraction as one persistent launch over the joint tile
space.  Each element goes through the same arithmetic as in a launch of its
bin alone, so its outputs must be bit-identical to those of a batch holding
that element only (a one-bin launch).  Checked on the hp mixed hexa / prism /
tet mesh in both precisions, on elements with and without bubbles."""
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


@pytest.mark.parametrize("prec", [H.MIXED, H.FP64])
def test_grouped_launches_bit_identical_to_one_bin_launches(prec):
    m = M.mixed_mesh(4, a=0.5, b=0.5, cy=0.5, perturb=0.1, seed=21, kappa_logrange=(-1, 1))
    ep = H.ElementPass(prec, integration=1, isol=10)
    ep.submit(m)
    ep.run()
    ep.download()
    kernels, _ = ep.pass_stats()
    rng = np.random.default_rng(2)
    nb = np.array([len(ep.schur(e)[1]) for e in range(m["nelem"])])
    picks = set(rng.choice(m["nelem"], 12, replace=False))
    picks |= {int(np.where(m["etype"] == t)[0][0]) for t in (1, 2, 3)}
    # elements without bubbles (condensed by the compression kernel alone)
    picks |= set(int(e) for e in np.where(nb == 0)[0][:4])
    picks |= set(int(e) for e in np.where(nb > 0)[0][:4])
    assert (nb == 0).any() and (nb > 0).any()
    for e in sorted(picks):
        one = H.ElementPass(prec, integration=1, isol=10)
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
