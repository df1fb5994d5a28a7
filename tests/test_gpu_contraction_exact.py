"""Exactness of the mixed-precision contraction on worst-case operands.

The split-BF16 contraction (k_ozaki.cu) sums the digit products of each level
in FP32 tensor-core accumulators.  It restarts every accumulator after at most
`kchunk` k-blocks, with kchunk * 16 * max_s sum_{i+j=s} b_i b_j <= 2^24, so no
partial sum can reach 2^24 whatever the data.  These tests drive the kernel
through hp3dg_mixed_contract with operands built to make the level sums as
large as the digit bounds allow: every entry just below its power-of-two
scale, so the leading digits are 127 or 128 and all products of a level have
the same sign.  Summed over K = 2058 (p = 5, INTEGRATION = 1) without the
restarts, level 2 alone reaches 2058 * 128^2 = 3.4e7 > 2^24, which FP32 would
round (about 6e-8 relative).  The bar is the FP64 product, 1e-13 relative to
sum |D||M|, the FP64 rounding of a K-term dot product; and the element-level
case the reference computes (elem_opt.F90:131) against the oracle at 1e-12.
"""
import ctypes
import math

import numpy as np
import pytest

from oracle import oracle as O
from hp3d_gb300 import hp3dg as H
from hp3d_gb300 import mesh as M

pytestmark = pytest.mark.gpu


def _contract(torch, D, Mt, radix=0, digits=0):
    dev = torch.device("cuda", 0)
    d = torch.tensor(D, dtype=torch.float64, device=dev)
    m = torch.tensor(Mt, dtype=torch.float64, device=dev)
    out = torch.empty((D.shape[0], Mt.shape[1]), dtype=torch.float64, device=dev)
    st = torch.cuda.current_stream(dev).cuda_stream
    rc = H.lib().hp3dg_mixed_contract(D.shape[0], D.shape[1], Mt.shape[1], d.data_ptr(),
                                      m.data_ptr(), out.data_ptr(), radix, digits,
                                      ctypes.c_void_p(st))
    assert rc == 0, rc
    return out.cpu().numpy()


def _near_scale(rng, shape, sign=False):
    """Entries in [0.99, 1): every row / column maximum just below 1, its
    scale 1, so the leading digit of every entry is 127 or 128."""
    v = 0.99 + 0.0099 * rng.random(shape)
    if sign:
        v *= rng.choice([-1.0, 1.0], size=shape)
    return v


@pytest.mark.parametrize("radix,digits", [(7, 7), (6, 7), (8, 6), (7, 5)])
def test_same_sign_worst_case_levels_exact(radix, digits):
    torch = pytest.importorskip("torch")
    rng = np.random.default_rng(11 + radix * 10 + digits)
    K = 2058
    D = _near_scale(rng, (200, K))
    Mt = _near_scale(rng, (K, 300))
    got = _contract(torch, D, Mt, radix, digits)
    ref = D @ Mt
    # level 2 without restarts would exceed 2^24 here
    assert K * 127 * 127 > 2 ** 24
    bits = radix * digits
    tol = max(1e-13, 2.0 ** (1 - bits) * 4)  # FP64 dot rounding, or the digit truncation
    err = np.abs(got - ref).max() / np.abs(ref).max()
    assert err < tol, (radix, digits, err)
    # exact sums of a few entries (math.fsum is correctly rounded)
    for r, c in ((0, 0), (199, 299), (57, 123)):
        ex = math.fsum(D[r, :] * Mt[:, c])  # products exact to 2^-106: fsum of the doubles
        assert abs(got[r, c] - ex) <= tol * abs(ex)


def test_signed_worst_case_and_zero_rows():
    torch = pytest.importorskip("torch")
    rng = np.random.default_rng(5)
    K = 2058
    D = _near_scale(rng, (130, K), sign=True)
    Mt = _near_scale(rng, (K, 150), sign=True)
    D[7] = 0.0                      # a zero row: scale 1, all digits zero
    Mt[:, 11] = 0.0
    got = _contract(torch, D, Mt)
    ref = D @ Mt
    scale = np.abs(D) @ np.abs(Mt)
    assert np.all(np.abs(got - ref) <= 1e-13 * scale + 0.0)
    assert np.all(got[7] == 0.0) and np.all(got[:, 11] == 0.0)


def test_ragged_sizes():
    """K, rows and columns that are not multiples of the tiles (16, 64, 128)."""
    torch = pytest.importorskip("torch")
    rng = np.random.default_rng(9)
    for nr, K, nc in ((1, 17, 1), (65, 100, 129), (300, 343 * 6, 7)):
        D = rng.standard_normal((nr, K)) * 10.0 ** rng.uniform(-3, 3, (nr, 1))
        Mt = rng.standard_normal((K, nc)) * 10.0 ** rng.uniform(-3, 3, (1, nc))
        got = _contract(torch, D, Mt)
        scale = np.abs(D) @ np.abs(Mt)
        assert np.all(np.abs(got - D @ Mt) <= 1e-13 * scale), (nr, K, nc)


def test_affine_uniform_kappa_p6_element_matches_oracle():
    """An affine element with uniform kappa: D per point is kappa w_l detJ
    J^-1 J^-T, constant up to the weights and diagonal, so every product of
    a diagonal column (a, a) of M = G_i[l,a]^2 has one sign.  p = 6,
    INTEGRATION = 1 (the rule of order 6, 343 points, K = 2058)."""
    m = M.structured_hexa(2, 6, perturb=0.0, kappa_logrange=None, seed=3)
    ep = H.ElementPass(H.MIXED, integration=1, isol=10, keep_elem=True)
    ep.submit(m)
    ep.run()
    ep.download()
    n = 7 ** 3
    for e in range(m["nelem"]):
        K, b, rc = O.elem(1, m["norder"][e], m["nori_edge"][e], m["nori_face"][e], m["xvert"][e],
                          m["kappa"][e], isol=10, integration=1)
        Kg, bg = ep.elem(e, n)
        err = np.abs(Kg - K).max() / np.abs(K).max()
        assert err < 1e-12, (e, err)
    ep.close()
