"""Failure paths of the element pass, made on purpose without faulting the GPU.

The reference stops on a LAPACK info /= 0 (modules/stc.F90:462-464) and
retries MUMPS with more workspace (solver/omp_mumps/mumps_sc.F90:402-410);
here every failure becomes a status code and the context stays usable.

- Timeout: with hp3dg_opts.fault_inject = 1 the contraction's loader never
  fills one stage of its ring.  The MMA thread's bounded wait on that stage
  runs out (a short iteration limit in this mode), every role of the kernel
  stops, the thread that issued copies waits for them, TMEM is freed, and the
  kernel returns: hp3dg_batch_sync reports HP3DG_ERR_TIMEOUT.  The same
  context then runs a correct pass after a resubmit without the fault (a
  new context), and the GPU context is unharmed.
- Allocation: with fault_inject = 2 every device allocation of the submit
  fails; the submit returns HP3DG_ERR_ALLOC, the context can be ended, and a
  new context works.
"""
import numpy as np
import pytest

from oracle import oracle as O
from hp3d_gb300 import hp3dg as H
from hp3d_gb300 import mesh as M

pytestmark = pytest.mark.gpu

TIMEOUT, ALLOC = -6, -4


def _check_pass(mesh, precision):
    ep = H.ElementPass(precision, integration=1, isol=10)
    ep.submit(mesh)
    ep.run()
    ep.download()
    for e in range(mesh["nelem"]):
        K, b, rc = O.elem(1, mesh["norder"][e], mesh["nori_edge"][e], mesh["nori_face"][e],
                          mesh["xvert"][e], mesh["kappa"][e], isol=10, integration=1)
        nb = O.nrdof_bubble(1, mesh["norder"][e])
        aii, bi, _, _, _ = O.stc_fwd(K, b, nb, 0)
        _, zb, zs, _ = O.celem_compress(1, mesh["norder"][e], mesh["bcflag"][e], aii, bi)
        gzb, gzs = ep.condensed(e)
        if zs.size:
            assert np.abs(gzs - zs).max() <= 1e-10 * np.abs(zs).max()
    ep.close()


def test_contraction_wait_runs_out_and_reports_timeout():
    mesh = M.structured_hexa(3, 3, perturb=0.1, kappa_logrange=(-1, 1), seed=8)
    # FP64 condensation: the stage after the contraction reads whatever the
    # stopped kernel left in the stiffness buffer, and its indexing does not
    # depend on those values
    ep = H.ElementPass(H.MIXED, integration=1, isol=10, schur_tc=False, fault_inject=1)
    ep.submit(mesh)
    ep.run()
    with pytest.raises(H.HP3DGError) as ei:
        ep.sync()
    assert ei.value.code == TIMEOUT
    # the context stays usable: run again (the fault is injected again)
    ep.run()
    with pytest.raises(H.HP3DGError) as ei:
        ep.sync()
    assert ei.value.code == TIMEOUT
    ep.close()
    # a context without the fault on the same device computes the right pass
    _check_pass(mesh, H.MIXED)


def test_allocation_failure_reports_alloc_and_context_closes():
    mesh = M.structured_hexa(2, 2, perturb=0.1, seed=4)
    ep = H.ElementPass(H.FP64, integration=1, isol=10, fault_inject=2)
    with pytest.raises(H.HP3DGError) as ei:
        ep.submit(mesh)
    assert ei.value.code == ALLOC
    with pytest.raises(H.HP3DGError) as ei:
        ep.run()                      # nothing submitted
    ep.close()
    _check_pass(mesh, H.FP64)
