"""Pins of the DPG Maxwell oracle (problems/MAXWELL/ULTRAWEAK_DPG) on CPU.

- H(curl) trace shapes: curls equal finite-difference curls of the values,
  and the element space spans the whole Nedelec space Q(p-1,p,p) x
  Q(p,p-1,p) x Q(p,p,p-1) under every orientation code;
- the broken test space has full rank;
- the DPG element matrix is Hermitian positive semi-definite;
- end to end: the reference's polynomial solution (mfd_solutions.F90 case 2,
  E_x = -100 xyz(x-1)(y-1)(z-1), H = curl E / (-i omega mu)) lies in the
  trial space at p = 3, so the DPG solution reproduces it to round-off, on a
  mesh with every kind of orientation code, graded boxes, per-element complex
  permittivity, perfect-conductor walls and an impedance face.
"""
import numpy as np
import pytest

import dpg_harness as D
from oracle import oracle as O


def _fd_curl(fn, x, h=1e-6):
    J = np.zeros(fn(x).shape + (3,))
    for d in range(3):
        xp = x.copy(); xp[d] += h
        xm = x.copy(); xm[d] -= h
        J[..., d] = (fn(xp) - fn(xm)) / (2 * h)
    return np.stack([J[:, 2, 1] - J[:, 1, 2], J[:, 0, 2] - J[:, 2, 0], J[:, 1, 0] - J[:, 0, 1]], 1)


@pytest.mark.parametrize("p", [1, 2, 3, 4])
def test_hcurl_curl_is_fd_curl(p):
    rng = np.random.default_rng(p)
    no = np.array([p] * 12 + [11 * p] * 6 + [111 * p])
    for _ in range(3):
        ne = rng.integers(0, 2, 12); nf = rng.integers(0, 8, 6)
        x = rng.uniform(0.1, 0.9, 3)
        s, c = O.shapeE_hexa(x, no, ne, nf)
        fd = _fd_curl(lambda y: O.shapeE_hexa(y, no, ne, nf)[0], x)
        assert np.abs(fd - c).max() < 1e-8 * max(1.0, np.abs(c).max())
    s, c = O.shapeEE_hexa(x, 111 * (p + 1))
    fd = _fd_curl(lambda y: O.shapeEE_hexa(y, 111 * (p + 1))[0], x)
    assert np.abs(fd - c).max() < 1e-8 * max(1.0, np.abs(c).max())


@pytest.mark.parametrize("p", [2, 3])
def test_hcurl_space_is_complete_under_orientations(p):
    rng = np.random.default_rng(10 + p)
    no = np.array([p] * 12 + [11 * p] * 6 + [111 * p])
    pts = rng.uniform(0, 1, (160, 3))
    for _ in range(2):
        ne = rng.integers(0, 2, 12); nf = rng.integers(0, 8, 6)
        A = np.stack([O.shapeE_hexa(q, no, ne, nf)[0] for q in pts]).transpose(0, 2, 1)
        A = A.reshape(3 * len(pts), -1)
        assert A.shape[1] == 3 * p * (p + 1) ** 2 == O.lib().orc_nrdofE_hexa(
            O._p(O._i32(no), O._i32p))
        res = 0.0
        for comp in range(3):
            degs = [p, p, p]
            degs[comp] = p - 1
            for i in range(degs[0] + 1):
                for j in range(degs[1] + 1):
                    for k in range(degs[2] + 1):
                        f = np.zeros((len(pts), 3))
                        f[:, comp] = pts[:, 0] ** i * pts[:, 1] ** j * pts[:, 2] ** k
                        coef, *_ = np.linalg.lstsq(A, f.reshape(-1), rcond=None)
                        res = max(res, np.abs(A @ coef - f.reshape(-1)).max())
        assert res < 1e-11


def test_broken_test_space_full_rank():
    pts = np.random.default_rng(3).uniform(0, 1, (200, 3))
    for nordP in (222, 333, 444):
        A = np.stack([O.shapeEE_hexa(q, nordP)[0] for q in pts]).transpose(0, 2, 1)
        A = A.reshape(600, -1)
        q = nordP // 111
        assert A.shape[1] == 3 * q * (q + 1) ** 2
        assert np.linalg.matrix_rank(A) == A.shape[1]


def test_sizes_of_config_p3():
    s = O.dpg_sizes([3] * 12 + [33] * 6 + [333])
    assert (s["ntest"], s["ntrial"], s["nEi"], s["nQ"]) == (600, 378, 108, 27)


def test_element_matrix_hermitian_psd():
    m = D.rotated_hexa_mesh(1, 2, seed=5)
    prm = O.maxw_params(isol=1)
    A, b, rc = O.dpg_elem(m["norder"][0], m["nori_edge"][0], m["nori_face"][0],
                          m["xvert"][0], 2.0 - 0.1j, 0, prm)
    assert rc == A.shape[0]
    assert np.abs(A - A.conj().T).max() <= 1e-13 * np.abs(A).max()
    ev = np.linalg.eigvalsh(A)
    assert ev.min() > -1e-12 * ev.max()
    prm0 = O.maxw_params(isol=0)
    _, b0, _ = O.dpg_elem(m["norder"][0], m["nori_edge"][0], m["nori_face"][0],
                          m["xvert"][0], 2.0 - 0.1j, 0, prm0)
    assert np.all(b0 == 0)


@pytest.mark.parametrize("imp_planes", [(), ((0, 1),)])
def test_polynomial_solution_reproduced(imp_planes):
    m = D.rotated_hexa_mesh(2, 3, seed=3, grading=1.3)
    assert len(np.unique(m["nori_face"])) >= 4 and np.any(m["nori_edge"] == 1)
    prm = O.maxw_params(isol=2, ibcflag=2 if imp_planes else 0)
    rng = np.random.default_rng(1)
    eps = rng.uniform(1, 4, m["nelem"]) * (1 - 1j * rng.uniform(0, 0.1, m["nelem"]))
    bc, imp = D.boundary_flags(m, imp_planes)
    assert (imp != 0).any() == bool(imp_planes)
    cond, schur, ni_e = D.oracle_condense(m, prm, eps, bc, imp)
    u, lcon, lcon_off, _ = D.solve_condensed(m, cond, m["nnodes"])
    ee, eh = D.field_errors(m, prm, eps, cond, schur, u, lcon, lcon_off, ni_e)
    assert ee < 1e-11 and eh < 1e-11, (ee, eh)
