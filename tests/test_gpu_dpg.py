"""The ultraweak DPG Maxwell pass on the GPU against the oracle
(problems/MAXWELL/ULTRAWEAK_DPG restated in oracle/hp3d_oracle_dpg.c).

- the DPG element matrix B^H G^-1 B and its load, element by element, on a
  mesh with every kind of edge and face orientation code, graded boxes and a
  complex permittivity per element;
- the condensed and compressed systems, the Schur blocks, and the index maps
  (bit-exact) of the EHtrc unknowns with perfect-conductor walls;
- the impedance penalty on one face;
- end to end: the reference's polynomial solution is reproduced from the GPU
  outputs to round-off.
Tolerances: the element matrices and condensed systems agree with the FP64
oracle to 1e-10 relative to their norms (same mathematics, another order of
summation and another factorisation order).
"""
import numpy as np
import pytest

import dpg_harness as D
from hp3d_gb300 import hp3dg as H
from oracle import oracle as O

pytestmark = pytest.mark.gpu


def _setup(n, p, imp_planes=(), isol=1, seed=3):
    m = D.rotated_hexa_mesh(n, p, seed=seed, grading=1.3)
    prm = O.maxw_params(isol=isol, ibcflag=2 if imp_planes else 0)
    rng = np.random.default_rng(seed)
    eps = rng.uniform(1, 4, m["nelem"]) * (1 - 1j * rng.uniform(0, 0.1, m["nelem"]))
    bc, imp = D.boundary_flags(m, imp_planes)
    flags = bc.copy()
    for e in range(m["nelem"]):
        for f in range(6):
            if (imp[e] >> f) & 1:
                flags[e, 20 + f] |= 4
    return m, prm, eps, bc, imp, flags


def _gpu(m, prm, eps, flags, keep=True):
    ep = H.DPGPass(omega=prm.omega, mu=prm.mu, epsilon=prm.epsilon, gamma=prm.gamma,
                   alpha=prm.alpha, ibcflag=prm.ibcflag, nord_add=prm.nord_add, isol=prm.isol,
                   icomp=prm.icomp, keep_elem=keep)
    ep.submit(m, eps, flags)
    ep.run()
    ep.download()
    return ep


def _rel(a, b):
    return np.abs(a - b).max() / max(np.abs(b).max(), 1e-300)


@pytest.mark.parametrize("p,imp_planes", [(1, ()), (2, ()), (3, ()), (2, ((0, 1),))])
def test_element_matrices_match_oracle(p, imp_planes):
    m, prm, eps, bc, imp, flags = _setup(2, p, imp_planes)
    ep = _gpu(m, prm, eps, flags)
    ntrial, ni, nb = ep.sizes()
    s = O.dpg_sizes(m["norder"][0])
    assert (ntrial, ni, nb) == (s["ntrial"], 2 * s["nEi"], 6 * s["nQ"])
    for e in range(m["nelem"]):
        A, b, rc = O.dpg_elem(m["norder"][e], m["nori_edge"][e], m["nori_face"][e],
                              m["xvert"][e], eps[e], int(imp[e]), prm)
        Ag, bg = ep.elem(e)
        assert _rel(Ag, A) < 1e-10, (e, _rel(Ag, A))
        assert _rel(bg, b) < 1e-10, (e, _rel(bg, b))
    ep.close()


@pytest.mark.parametrize("p,imp_planes", [(2, ()), (3, ((0, 1),))])
def test_condensed_schur_and_index_maps_match_oracle(p, imp_planes):
    m, prm, eps, bc, imp, flags = _setup(2, p, imp_planes)
    ep = _gpu(m, prm, eps, flags, keep=False)
    cond, schur, ni_e = D.oracle_condense(m, prm, eps, bc, imp)
    for e in range(m["nelem"]):
        nx, zb, zs, _ = cond[e]
        zbg, zsg = ep.condensed(e)
        assert zsg.shape == zs.shape
        assert _rel(zsg, zs) < 1e-10 and _rel(zbg, zb) < 1e-10, e
        ag, bg = ep.schur(e)
        assert _rel(ag, schur[e][0]) < 1e-10 and _rel(bg, schur[e][1]) < 1e-10, e
    nr, nf, lc, lo, en = ep.index_map()
    ndofm = np.array([c[3] for c in cond], np.int32)
    nr0, nf0, lc0, lo0, en0 = O.index_maps(np.full(m["nelem"], 26, np.int32),
                                           m["nodes"][:, :26], ndofm, m["nnodes"])
    assert nr == nr0
    assert np.array_equal(lo, lo0) and np.array_equal(en, en0) and np.array_equal(lc, lc0)
    vis = nf0 >= 0
    assert np.array_equal(nf[vis], nf0[vis])
    ep.close()


@pytest.mark.parametrize("imp_planes", [(), ((0, 1),)])
def test_polynomial_solution_from_gpu_outputs(imp_planes):
    m, prm, eps, bc, imp, flags = _setup(2, 3, imp_planes, isol=2)
    ep = _gpu(m, prm, eps, flags, keep=False)
    ntrial, ni, nb = ep.sizes()
    cond, schur = [], []
    for e in range(m["nelem"]):
        zb, zs = ep.condensed(e)
        # the extraction vector is the host's (celem_systemI order); take it
        # from the oracle compression of the same flags
        nx = O.celem_compress_z(m["norder"][e], bc[e], np.eye(ni, dtype=complex),
                                np.zeros(ni, complex))[0]
        ndofm = O.celem_compress_z(m["norder"][e], bc[e], np.eye(ni, dtype=complex),
                                   np.zeros(ni, complex))[3]
        cond.append((nx, zb, zs, ndofm))
        schur.append(ep.schur(e))
    u, lcon, lcon_off, _ = D.solve_condensed(m, cond, m["nnodes"])
    ee, eh = D.field_errors(m, prm, eps, cond, schur, u, lcon, lcon_off, [ni] * m["nelem"])
    assert ee < 1e-10 and eh < 1e-10, (ee, eh)
    ep.close()


def test_rejects_anisotropic_or_mixed_orders():
    m = D.rotated_hexa_mesh(1, 2)
    m2 = dict(m)
    no = m["norder"].copy()
    no[0, 18] = 223
    m2["norder"] = no
    ep = H.DPGPass()
    with pytest.raises(H.HP3DGError):
        ep.submit(m2, np.ones(1, complex), np.zeros((1, 26), np.int32))
    ep.close()


@pytest.mark.parametrize("p,imp_planes", [(1, ()), (2, ((0, 1),)), (3, ())])
def test_tensor_core_dense_algebra_matches_oracle(p, imp_planes):
    """precision = MIXED: the Gram Cholesky's trailing updates, the solve's
    block updates and X^H X on tensor cores from split-BF16 digits (FP64
    diagonal blocks); element matrices and condensed systems within 1e-10 of
    the FP64 oracle."""
    m, prm, eps, bc, imp, flags = _setup(2, p, imp_planes)
    ep = H.DPGPass(omega=prm.omega, ibcflag=prm.ibcflag, isol=prm.isol, keep_elem=True,
                   precision=H.MIXED)
    ep.submit(m, eps, flags)
    ep.run(); ep.download()
    # per panel of the augmented matrix: the diagonal block, the digit slices
    # and the tensor-core updates are separate launches
    assert ep.pass_stats() > 40
    cond, schur, ni_e = D.oracle_condense(m, prm, eps, bc, imp)
    for e in range(m["nelem"]):
        A, b, rc = O.dpg_elem(m["norder"][e], m["nori_edge"][e], m["nori_face"][e],
                              m["xvert"][e], eps[e], int(imp[e]), prm)
        Ag, bg = ep.elem(e)
        assert _rel(Ag, A) < 1e-10 and _rel(bg, b) < 1e-10, (e, _rel(Ag, A), _rel(bg, b))
        zb, zs = ep.condensed(e)
        assert _rel(zs, cond[e][2]) < 1e-10 and _rel(zb, cond[e][1]) < 1e-10, e
    ep.close()


def test_tensor_core_polynomial_solution():
    m, prm, eps, bc, imp, flags = _setup(2, 3, ((0, 1),), isol=2)
    ep = H.DPGPass(omega=prm.omega, ibcflag=prm.ibcflag, isol=prm.isol, precision=H.MIXED)
    ep.submit(m, eps, flags)
    ep.run(); ep.download()
    ntrial, ni, nb = ep.sizes()
    cond, schur = [], []
    for e in range(m["nelem"]):
        zb, zs = ep.condensed(e)
        nx, _, _, ndofm = O.celem_compress_z(m["norder"][e], bc[e], np.eye(ni, dtype=complex),
                                             np.zeros(ni, complex))
        cond.append((nx, zb, zs, ndofm))
        schur.append(ep.schur(e))
    u, lcon, lcon_off, _ = D.solve_condensed(m, cond, m["nnodes"])
    ee, eh = D.field_errors(m, prm, eps, cond, schur, u, lcon, lcon_off, [ni] * m["nelem"])
    assert ee < 1e-10 and eh < 1e-10, (ee, eh)
    ep.close()


@pytest.mark.parametrize("precision", [H.FP64, H.MIXED])
def test_resubmit_same_mesh_matches_fresh_context(precision):
    """A resubmit with the same descriptors only uploads the new vertices and
    permittivities; its outputs equal those of a new context."""
    m, prm, eps, bc, imp, flags = _setup(2, 2, ((0, 1),))
    eps2 = eps * (1.5 - 0.2j)
    ep = H.DPGPass(omega=prm.omega, ibcflag=prm.ibcflag, isol=prm.isol, precision=precision)
    ep.submit(m, eps, flags)
    ep.run(); ep.download()
    ep.submit(m, eps2, flags)
    ep.run(); ep.download()
    fresh = H.DPGPass(omega=prm.omega, ibcflag=prm.ibcflag, isol=prm.isol, precision=precision)
    fresh.submit(m, eps2, flags)
    fresh.run(); fresh.download()
    for e in range(m["nelem"]):
        zb, zs = ep.condensed(e)
        zb0, zs0 = fresh.condensed(e)
        assert np.array_equal(zs, zs0) and np.array_equal(zb, zb0), e
        a, b = ep.schur(e)
        a0, b0 = fresh.schur(e)
        assert np.array_equal(a, a0) and np.array_equal(b, b0), e
    ep.close(); fresh.close()


def test_tensor_core_p4_element_matrices():
    """p = 4 (test order 5: augmented size 1849, Gram table of 146k packed
    columns) on the mixed path: two elements with different orientation
    codes against the oracle (one oracle element takes seconds)."""
    m, prm, eps, bc, imp, flags = _setup(2, 4, ((0, 1),))
    ep = H.DPGPass(omega=prm.omega, ibcflag=prm.ibcflag, isol=prm.isol, keep_elem=True,
                   precision=H.MIXED)
    ep.submit(m, eps, flags)
    ep.run(); ep.download()
    for e in (0, 5):
        A, b, rc = O.dpg_elem(m["norder"][e], m["nori_edge"][e], m["nori_face"][e],
                              m["xvert"][e], eps[e], int(imp[e]), prm)
        Ag, bg = ep.elem(e)
        assert _rel(Ag, A) < 1e-10 and _rel(bg, b) < 1e-10, (e, _rel(Ag, A), _rel(bg, b))
    ep.close()
