"""hp3dg_condense_noalloc: static condensation with no allocation.

Callers that cannot allocate device memory (an element loop inside an OpenMP
region of a host solver, an application whose GPU memory belongs to its own
pool) hand the library their element matrices and output buffers; the entry
point keeps its scratch in a fixed device array.  This test calls it through
the C ABI twice in a row, on different elements, and checks each result
against the batch entry point (hp3dg_batch_* / hp3dg_get_condensed /
hp3dg_get_schur) within the FP64 tolerance of the other parity tests, 1e-12
relative.  It runs last (file name) and needs nothing from earlier tests.
"""
import ctypes

import numpy as np
import pytest

from oracle import oracle as O
from hp3d_gb300 import hp3dg as H
from hp3d_gb300 import mesh as M

pytestmark = pytest.mark.gpu
TOL = 1e-12


def _rel(a, b):
    return np.abs(a - b).max() / max(np.abs(b).max(), 1e-300)


def _bind():
    L = H.lib()
    f = L.hp3dg_condense_noalloc
    f.argtypes = [ctypes.c_int32, ctypes.c_int32, ctypes.c_int32] + [ctypes.c_void_p] * 6 + \
        [ctypes.POINTER(ctypes.c_int32), ctypes.c_void_p]
    f.restype = ctypes.c_int
    return f


def test_condense_noalloc_matches_batch_entry_point():
    torch = pytest.importorskip("torch")
    f = _bind()
    p = 3
    m = M.structured_hexa(2, p, perturb=0.15, kappa_logrange=(-2, 2), seed=17, dirichlet=False)
    n = (p + 1) ** 3
    nb = (p - 1) ** 3
    ni = n - nb
    ep = H.ElementPass(H.FP64, integration=1, isol=10, keep_elem=True)
    ep.submit(m)
    ep.run()
    ep.download()
    Ks, bs = zip(*[ep.elem(e, n) for e in range(m["nelem"])])
    nd = O.node_ndof(1, m["norder"][0])
    first = np.concatenate([[0], np.cumsum(nd)])
    nx = np.array([first[i] + q for i in range(25, -1, -1) for q in range(nd[i])])
    dev = torch.device("cuda", 0)
    stream = torch.cuda.current_stream(dev)
    for calln, elems in enumerate([range(0, 4), range(4, 8)]):
        idx = list(elems)
        K = torch.tensor(np.stack([Ks[e].T for e in idx]), dtype=torch.float64, device=dev)
        b = torch.tensor(np.stack([bs[e] for e in idx]), dtype=torch.float64, device=dev)
        aii = torch.empty((len(idx), ni, ni), dtype=torch.float64, device=dev)
        bi = torch.empty((len(idx), ni), dtype=torch.float64, device=dev)
        asch = torch.empty((len(idx), ni, nb), dtype=torch.float64, device=dev)
        bsch = torch.empty((len(idx), nb), dtype=torch.float64, device=dev)
        bad = ctypes.c_int32(-5)
        rc = f(len(idx), n, nb, K.data_ptr(), b.data_ptr(), aii.data_ptr(), bi.data_ptr(),
               asch.data_ptr(), bsch.data_ptr(), ctypes.byref(bad), ctypes.c_void_p(stream.cuda_stream))
        assert rc == 0 and bad.value == -1, (calln, rc, bad.value)
        A = aii.cpu().numpy()      # per element column-major ni x ni -> [e, col, row]
        Bi = bi.cpu().numpy()
        AS = asch.cpu().numpy()    # per element column-major nb x ni -> [e, col, row]
        BS = bsch.cpu().numpy()
        for k, e in enumerate(idx):
            zb, zs = ep.condensed(e)
            a_ref, b_ref = ep.schur(e)
            Ae = A[k].T
            assert _rel(Ae[np.ix_(nx, nx)], zs) < TOL
            assert _rel(Bi[k][nx], zb) < TOL
            assert _rel(AS[k].T, a_ref) < TOL
            assert _rel(BS[k], b_ref) < TOL
    ep.close()


def test_condense_noalloc_rejects_oversized_batch():
    f = _bind()
    # 2^20 doubles of scratch: 100 elements of p=6 (ni = 218) need more
    bad = ctypes.c_int32(0)
    rc = f(100, 343, 125, ctypes.c_void_p(16), ctypes.c_void_p(16), ctypes.c_void_p(16),
           ctypes.c_void_p(16), ctypes.c_void_p(16), ctypes.c_void_p(16), ctypes.byref(bad), None)
    assert rc == -7
