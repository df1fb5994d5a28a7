"""Host-side assembly and solve of the ultraweak DPG Maxwell system for the
parity tests (the stand-in for the reference's MUMPS driver).

The element matrices come from the oracle (or from the GPU pass); the
condensed interface systems are assembled through LCON into a SciPy sparse
complex matrix, solved, and the L2 fields recovered element by element from
the Schur blocks (stc_bwd).  Errors are measured against the manufactured
solution at the element quadrature points.
"""
from __future__ import annotations

import itertools

import numpy as np
import scipy.sparse as sp
import scipy.sparse.linalg as spla

from hp3d_gb300 import mesh as M
from oracle import oracle as O

_VOFF = np.array([[0, 0, 0], [1, 0, 0], [1, 1, 0], [0, 1, 0],
                  [0, 0, 1], [1, 0, 1], [1, 1, 1], [0, 1, 1]])


def _rotations():
    """The 24 proper rotations of the cube as signed permutation matrices."""
    out = []
    for perm in itertools.permutations(range(3)):
        for signs in itertools.product((1, -1), repeat=3):
            R = np.zeros((3, 3), int)
            for r, (c, s) in enumerate(zip(perm, signs)):
                R[r, c] = s
            if round(np.linalg.det(R)) == 1:
                out.append(R)
    return out


def rotated_hexa_mesh(n, p, seed=0, grading=1.0, rotate=True):
    """n^3 box hexahedra of the unit cube, each with a random proper rotation
    of its local vertex numbering (so that edge and face orientation codes of
    every kind occur), isotropic order p.  grading != 1 maps the grid
    coordinates by x -> x**grading (boxes of different sizes: still affine
    elements)."""
    rng = np.random.default_rng(seed)
    rots = _rotations()
    nv1 = n + 1
    idx = np.arange(nv1)
    I, J, K = np.meshgrid(idx, idx, idx, indexing="ij")
    grid = np.stack([I.ravel(order="F"), J.ravel(order="F"), K.ravel(order="F")], axis=1)
    X = (grid / n) ** grading
    vid = lambda c: int(c[0] + nv1 * (c[1] + nv1 * c[2]))  # noqa: E731
    et, verts, orders = [], [], []
    for k in range(n):
        for j in range(n):
            for i in range(n):
                c = np.array([i, j, k])
                R = rots[rng.integers(len(rots))] if rotate else np.eye(3, dtype=int)
                loc = [(R @ (2 * v - 1) + 1) // 2 for v in _VOFF]
                et.append(M.HEXA)
                verts.append([vid(c + q) for q in loc])
                orders.append((p, p, p))
    return M.build_mesh(et, verts, X, grid, n, orders)


def boundary_flags(mesh, imp_planes=()):
    """Per element: bcflag (26 nodes; bit 0 = E trace known) and the impedance
    face mask, from the library's node flags (hp3d_gb300.mesh)."""
    fl = M.dpg_boundary_flags(mesh, imp_planes)
    bc = fl & 3
    imp = np.zeros(mesh["nelem"], np.int32)
    for f in range(6):
        imp |= ((fl[:, 20 + f] >> 2) & 1) << f
    return bc, imp


def solve_condensed(mesh, cond, nnodes):
    """Assemble the condensed complex interface systems through LCON and solve.
    cond: per element (nextract, zbload, zastif, ndofm)."""
    ne = mesh["nelem"]
    ndofm = np.array([c[3] for c in cond], np.int32)
    nnode = np.full(ne, 26, np.int32)
    nrdof, nfirst, lcon, lcon_off, elem_nnz = O.index_maps(nnode, mesh["nodes"][:, :26], ndofm,
                                                           nnodes)
    rows, cols, vals = [], [], []
    F = np.zeros(nrdof, np.complex128)
    for e in range(ne):
        lc = lcon[lcon_off[e]:lcon_off[e + 1]] - 1
        _, zb, zs, _ = cond[e]
        rows.append(np.repeat(lc, len(lc)))
        cols.append(np.tile(lc, len(lc)))
        vals.append(zs.reshape(-1))
        np.add.at(F, lc, zb)
    A = sp.csc_matrix((np.concatenate(vals), (np.concatenate(rows), np.concatenate(cols))),
                      shape=(nrdof, nrdof))
    u = spla.spsolve(A, F)
    return u, lcon, lcon_off, nfirst


def field_errors(mesh, prm, eps, cond, schur, u, lcon, lcon_off, ni_e):
    """Relative L2 errors of the recovered E and H fields."""
    num_e = den_e = num_h = den_h = 0.0
    one = np.array([1] * 12 + [11] * 6 + [111])
    for e in range(mesh["nelem"]):
        norder = mesh["norder"][e]
        nx, _, _, _ = cond[e]
        asch, bsch = schur[e]
        xi = np.zeros(ni_e[e], np.complex128)
        xi[nx] = u[lcon[lcon_off[e]:lcon_off[e + 1]] - 1]
        xb = bsch - asch @ xi
        nq = len(xb) // 6
        coef = xb.reshape(nq, 6)
        xq, wq = O.quad_hexa(norder, integration=1)
        xv = mesh["xvert"][e, :8]
        for q, w in zip(xq, wq):
            sh, gr = O.shape_hexa(q, one)
            x = sh @ xv
            J = xv.T @ gr
            dj = np.linalg.det(J)
            qv = O.shapeQ_hexa(q, norder) / dj
            Eh = qv @ coef[:, 0:3]
            Hh = qv @ coef[:, 3:6]
            E, H, _ = O.maxw_exact(x, prm, eps[e])
            num_e += w * dj * np.sum(np.abs(Eh - E) ** 2)
            den_e += w * dj * np.sum(np.abs(E) ** 2)
            num_h += w * dj * np.sum(np.abs(Hh - H) ** 2)
            den_h += w * dj * np.sum(np.abs(H) ** 2)
    return np.sqrt(num_e / den_e), np.sqrt(num_h / den_h)


def oracle_condense(mesh, prm, eps, bc, imp):
    """Element matrices, condensation and compression by the oracle."""
    cond, schur, ni_e = [], [], []
    for e in range(mesh["nelem"]):
        no = mesh["norder"][e]
        A, b, rc = O.dpg_elem(no, mesh["nori_edge"][e], mesh["nori_face"][e],
                              mesh["xvert"][e], eps[e], int(imp[e]), prm)
        assert rc > 0, rc
        nb = 6 * O.dpg_sizes(no, prm.nord_add)["nQ"]
        aii, bi, asch, bsch, rc = O.stc_fwd_z(A, b, nb)
        assert rc == 0
        cond.append(O.celem_compress_z(no, bc[e], aii, bi))
        schur.append((asch, bsch))
        ni_e.append(aii.shape[0])
    return cond, schur, ni_e
