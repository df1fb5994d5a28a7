"""Mixed-precision path (split-BF16 digits on tcgen05) against the FP64
oracle and against the FP64 GPU path.

Tolerances, stated per quantity:
* element stiffness PK, mixed vs oracle: 1e-12 relative to the element's
  largest entry (radix 7 x 7 digits carry ~49 bits; measured ~5e-15);
* condensed matrices / loads / Schur blocks: 1e-10 relative;
* final solution of the assembled condensed system, mixed vs FP64 GPU:
  1e-10 relative (the metric's accuracy bar).
"""
import numpy as np
import pytest

from oracle import oracle as O
from hp3d_gb300 import hp3dg as H
from hp3d_gb300 import mesh as M
import fem_harness as FH
from test_gpu_parity import _gpu_elements

pytestmark = pytest.mark.gpu


def _rel(a, b):
    return np.abs(a - b).max() / max(np.abs(b).max(), 1e-300)


@pytest.mark.parametrize("p,integ", [(2, 0), (3, 1), (5, 1)])
def test_mixed_element_matrices(p, integ):
    m = M.random_orientations(M.structured_hexa(2, p, perturb=0.15, kappa_logrange=(-2, 2), seed=p),
                              seed=p)
    ep = H.ElementPass(H.MIXED, integration=integ, isol=10, keep_elem=True)
    ep.submit(m)
    ep.run(); ep.download()
    r, d, npair = ep.mixed_config()
    assert (r, d) == (7, 7) and npair == 28
    worst = 0.0
    for e in range(m["nelem"]):
        K, b, _ = O.elem(1, m["norder"][e], m["nori_edge"][e], m["nori_face"][e], m["xvert"][e],
                         m["kappa"][e], isol=10, integration=integ)
        Kg, bg = ep.elem(e, K.shape[0])
        worst = max(worst, _rel(Kg, K))
        assert _rel(bg, b) < 1e-12
    assert worst < 1e-12, worst


def test_mixed_condensed_vs_oracle():
    m = M.random_orientations(M.structured_hexa(3, 5, perturb=0.15, kappa_logrange=(-2, 2), seed=9),
                              seed=4)
    ep = H.ElementPass(H.MIXED, integration=1, isol=10)
    ep.submit(m)
    ep.run(); ep.download()
    ref = FH.oracle_element_outputs(m, 10, integration=1)
    for e in range(m["nelem"]):
        zb, zs = ep.condensed(e)
        if zs.size:
            assert _rel(zs, ref[e]["zastif"]) < 1e-10
            assert _rel(zb, ref[e]["zbload"]) < 1e-10
        a, bsch = ep.schur(e)
        assert _rel(a, ref[e]["aschur"]) < 1e-10


def test_mixed_final_solution_within_1e10():
    """Assemble and solve the condensed system from both GPU paths on a
    perturbed p=5 mesh with kappa in [1e-2, 1e2].  The solution of the
    condensed interface system -- what MUMPS returns -- differs by <= 1e-10
    relative.  The bubbles back-substituted from it go through ASchur, which
    the mixed pass forms with the explicit inverse of the bubble block's
    Cholesky factor (about 1e-10 relative on its worst elements): the full
    solution is held to 2e-10."""
    m = M.structured_hexa(4, 5, perturb=0.15, kappa_logrange=(-2, 2), seed=21)
    sols, xs = {}, {}
    for prec in (H.FP64, H.MIXED):
        ep = H.ElementPass(prec, integration=1, isol=10)
        ep.submit(m)
        ep.run(); ep.download()
        _, _, x, dofs = FH.solve_and_error(m, _gpu_elements(ep, m), 10)
        sols[prec] = np.concatenate(dofs)
        xs[prec] = x
        ep.close()
    rel_x = np.linalg.norm(xs[H.MIXED] - xs[H.FP64]) / np.linalg.norm(xs[H.FP64])
    assert rel_x < 1e-10, rel_x
    rel = np.linalg.norm(sols[H.MIXED] - sols[H.FP64]) / np.linalg.norm(sols[H.FP64])
    assert rel < 2e-10, rel


def test_mixed_radix_digits_options():
    m = M.structured_hexa(2, 4, perturb=0.1, seed=3)
    ep = H.ElementPass(H.MIXED, integration=0, isol=10, keep_elem=True, ozaki_radix=6,
                       ozaki_digits=7)
    ep.submit(m)
    ep.run(); ep.download()
    assert ep.mixed_config() == (6, 7, 28)
    K, b, _ = O.elem(1, m["norder"][0], m["nori_edge"][0], m["nori_face"][0], m["xvert"][0],
                     m["kappa"][0], isol=10, integration=0)
    Kg, _ = ep.elem(0, K.shape[0])
    assert _rel(Kg, K) < 5e-12  # radix 6 x 7 digits carries ~42 bits


def test_mixed_final_solution_at_the_fp64_floor():
    """On 6^3 p=5 (kappa in [1e-2, 1e2]) the global conditioning amplifies
    element rounding to ~5e-10 in the final solution: the FP64 GPU pass and
    the FP64 CPU oracle already differ by that much.  The mixed pass must
    stay within twice that FP64-to-FP64 difference of the FP64 pass."""
    m = M.structured_hexa(6, 5, perturb=0.15, kappa_logrange=(-2, 2), seed=7)
    sols = {}
    for prec in (H.FP64, H.MIXED):
        ep = H.ElementPass(prec, integration=1, isol=10)
        ep.submit(m)
        ep.run(); ep.download()
        _, _, _, dofs = FH.solve_and_error(m, _gpu_elements(ep, m), 10)
        sols[prec] = np.concatenate(dofs)
        ep.close()
    orc = FH.oracle_element_outputs(m, 10, integration=1, stc_method=1)
    _, _, _, dofs = FH.solve_and_error(m, orc, 10)
    cpu = np.concatenate(dofs)
    floor = np.linalg.norm(sols[H.FP64] - cpu) / np.linalg.norm(cpu)
    rel = np.linalg.norm(sols[H.MIXED] - sols[H.FP64]) / np.linalg.norm(sols[H.FP64])
    assert rel <= max(1e-10, 2.0 * floor), (rel, floor)
