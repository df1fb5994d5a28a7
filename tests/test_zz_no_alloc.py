"""hp3dg_condense_noalloc: static condensation with no allocation.

Callers that cannot allocate device memory (an element loop inside an OpenMP
region of a host solver, an application whose GPU memory belongs to its own
pool) hand the library their element matrices and output buffers; the entry
point keeps its scratch in a fixed device array.  These tests call it through
the C ABI, several calls in a row, and check each result against the batch
entry point (hp3dg_batch_* / hp3dg_get_condensed / hp3dg_get_schur) within
the FP64 tolerance of the other parity tests, 1e-12 relative, and against the
oracle's stc_fwd on the same element matrices.  They also cover the largest
batch the scratch array accepts at p = 5, the first oversized batch, a bubble
block that is not positive definite, and an empty batch.  The file runs last
(file name) and needs nothing from earlier tests.
"""
import ctypes

import numpy as np
import pytest

from oracle import oracle as O
from hp3d_gb300 import hp3dg as H
from hp3d_gb300 import mesh as M

pytestmark = pytest.mark.gpu
TOL = 1e-12          # FP64 parity bar of the condensed matrix and load
TOL_SCHUR = 1e-11    # Schur blocks carry cond(K_bb) (Cholesky here, LU in stc_fwd)
SCRATCH = 1 << 20    # HP3DG_NOALLOC_SCRATCH_DOUBLES


def _rel(a, b):
    return np.abs(a - b).max() / max(np.abs(b).max(), 1e-300)


def _bind():
    L = H.lib()
    f = L.hp3dg_condense_noalloc
    f.argtypes = [ctypes.c_int32, ctypes.c_int32, ctypes.c_int32] + [ctypes.c_void_p] * 6 + \
        [ctypes.POINTER(ctypes.c_int32), ctypes.c_void_p]
    f.restype = ctypes.c_int
    return f


def _element_matrices(p, nx):
    """FP64 element matrices of a perturbed p-hexa mesh from the batch pass,
    and the pass itself (for its condensed outputs)."""
    m = M.structured_hexa(nx, p, perturb=0.15, kappa_logrange=(-2, 2), seed=17, dirichlet=False)
    n = (p + 1) ** 3
    ep = H.ElementPass(H.FP64, integration=1, isol=10, keep_elem=True)
    ep.submit(m)
    ep.run()
    ep.download()
    Ks, bs = zip(*[ep.elem(e, n) for e in range(m["nelem"])])
    nd = O.node_ndof(1, m["norder"][0])
    first = np.concatenate([[0], np.cumsum(nd)])
    nxt = np.array([first[i] + q for i in range(25, -1, -1) for q in range(nd[i])])
    return m, ep, Ks, bs, nxt


def _call(f, torch, Ks, bs, idx, n, nb, stream):
    dev = torch.device("cuda", 0)
    ni = n - nb
    K = torch.tensor(np.stack([Ks[e].T for e in idx]), dtype=torch.float64, device=dev)
    b = torch.tensor(np.stack([bs[e] for e in idx]), dtype=torch.float64, device=dev)
    aii = torch.empty((len(idx), ni, ni), dtype=torch.float64, device=dev)
    bi = torch.empty((len(idx), ni), dtype=torch.float64, device=dev)
    asch = torch.empty((len(idx), ni, nb), dtype=torch.float64, device=dev)
    bsch = torch.empty((len(idx), nb), dtype=torch.float64, device=dev)
    bad = ctypes.c_int32(-5)
    rc = f(len(idx), n, nb, K.data_ptr(), b.data_ptr(), aii.data_ptr(), bi.data_ptr(),
           asch.data_ptr(), bsch.data_ptr(), ctypes.byref(bad), ctypes.c_void_p(stream))
    # per element column-major blocks -> [e, col, row]
    return rc, bad.value, aii.cpu().numpy(), bi.cpu().numpy(), asch.cpu().numpy(), \
        bsch.cpu().numpy()


def _check(ep, Ks, bs, idx, nb, nxt, A, Bi, AS, BS):
    for k, e in enumerate(idx):
        zb, zs = ep.condensed(e)
        a_ref, b_ref = ep.schur(e)
        Ae = A[k].T
        assert _rel(Ae[np.ix_(nxt, nxt)], zs) < TOL, e
        assert _rel(Bi[k][nxt], zb) < TOL, e
        assert _rel(AS[k].T, a_ref) < TOL, e
        assert _rel(BS[k], b_ref) < TOL, e
        # the oracle's stc_fwd (LU, stc.F90:443-509) on the same element matrix
        aii, bi, asch, bsch, rc = O.stc_fwd(Ks[e], bs[e], nb, 0)
        assert rc == 0
        assert _rel(Ae, aii) < TOL, e
        assert _rel(Bi[k], bi) < TOL, e
        assert _rel(AS[k].T, asch) < TOL_SCHUR, e
        assert _rel(BS[k], bsch) < TOL_SCHUR, e


def test_condense_noalloc_matches_batch_entry_point():
    torch = pytest.importorskip("torch")
    f = _bind()
    p = 3
    n, nb = (p + 1) ** 3, (p - 1) ** 3
    m, ep, Ks, bs, nxt = _element_matrices(p, 2)
    stream = torch.cuda.current_stream(torch.device("cuda", 0)).cuda_stream
    for calln, elems in enumerate([range(0, 4), range(4, 8)]):
        idx = list(elems)
        rc, bad, A, Bi, AS, BS = _call(f, torch, Ks, bs, idx, n, nb, stream)
        assert rc == 0 and bad == -1, (calln, rc, bad)
        _check(ep, Ks, bs, idx, nb, nxt, A, Bi, AS, BS)
    ep.close()


def test_condense_noalloc_largest_batch_p5():
    """p = 5 (ni = 152, the largest triangle of the packed-index decode) at the
    largest batch the scratch array accepts, then one element more."""
    torch = pytest.importorskip("torch")
    f = _bind()
    p = 5
    n, nb = (p + 1) ** 3, (p - 1) ** 3
    ni = n - nb
    cap = (SCRATCH - 1) // (ni * (ni + 1) // 2)
    assert cap == 90
    m, ep, Ks, bs, nxt = _element_matrices(p, 5)
    stream = torch.cuda.current_stream(torch.device("cuda", 0)).cuda_stream
    idx = list(range(cap))
    rc, bad, A, Bi, AS, BS = _call(f, torch, Ks, bs, idx, n, nb, stream)
    assert rc == 0 and bad == -1, (rc, bad)
    _check(ep, Ks, bs, idx, nb, nxt, A, Bi, AS, BS)
    # a second call in a row on other elements reuses the same scratch
    idx2 = list(range(cap, m["nelem"]))
    rc, bad, A, Bi, AS, BS = _call(f, torch, Ks, bs, idx2, n, nb, stream)
    assert rc == 0 and bad == -1, (rc, bad)
    _check(ep, Ks, bs, idx2, nb, nxt, A, Bi, AS, BS)
    rc, bad, *_ = _call(f, torch, Ks, bs, list(range(cap + 1)), n, nb, stream)
    assert rc == -7 and bad == -1
    ep.close()


def test_condense_noalloc_not_spd_reports_first_bad_element():
    torch = pytest.importorskip("torch")
    f = _bind()
    p = 3
    n, nb = (p + 1) ** 3, (p - 1) ** 3
    ni = n - nb
    m, ep, Ks, bs, nxt = _element_matrices(p, 2)
    ep.close()
    Ks = [K.copy() for K in Ks]
    for e in (5, 2):             # two bad elements: the first index is reported
        Ks[e][ni, ni] = -abs(Ks[e][ni, ni])
    stream = torch.cuda.current_stream(torch.device("cuda", 0)).cuda_stream
    rc, bad, *_ = _call(f, torch, Ks, bs, list(range(8)), n, nb, stream)
    assert rc == -2 and bad == 2, (rc, bad)
    # the status is reset per call: a good batch right after succeeds
    rc, bad, *_ = _call(f, torch, Ks, bs, [0, 1, 3, 4], n, nb, stream)
    assert rc == 0 and bad == -1, (rc, bad)


def test_condense_noalloc_rejects_oversized_batch_and_accepts_empty():
    f = _bind()
    # 2^20 doubles of scratch: 100 elements of p=6 (ni = 218) need more
    bad = ctypes.c_int32(0)
    rc = f(100, 343, 125, ctypes.c_void_p(16), ctypes.c_void_p(16), ctypes.c_void_p(16),
           ctypes.c_void_p(16), ctypes.c_void_p(16), ctypes.c_void_p(16), ctypes.byref(bad), None)
    assert rc == -7 and bad.value == -1
    bad = ctypes.c_int32(7)
    rc = f(0, 64, 8, ctypes.c_void_p(16), ctypes.c_void_p(16), ctypes.c_void_p(16),
           ctypes.c_void_p(16), ctypes.c_void_p(16), ctypes.c_void_p(16), ctypes.byref(bad), None)
    assert rc == 0 and bad.value == -1
    # a p = 6 hexahedron's bubble block does not fit in shared memory
    bad = ctypes.c_int32(0)
    rc = f(1, 343, 125, ctypes.c_void_p(16), ctypes.c_void_p(16), ctypes.c_void_p(16),
           ctypes.c_void_p(16), ctypes.c_void_p(16), ctypes.c_void_p(16), ctypes.byref(bad), None)
    assert rc == -9 and bad.value == -1
