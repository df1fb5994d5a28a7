"""Meshes with hanging nodes and their constraint coefficients, for the
constrained-approximation tests (constrs/logic.F90 + celem_systemI.F90:541-760).

The mesh is nc^3 box hexahedra of the unit cube with the centre element
refined into 8 children.  The children's nodes on the centre cube's faces
that no coarse element has (edge midpoints, face centres, half edges, quarter
faces) are constrained by the coarse neighbour's face trace: the constraint
coefficients C(k, l) express every coarse trace function psi_l restricted to
a child face in the child's trace basis (an exact polynomial identity,
computed by least squares on a Gauss rule of the child face).  The modified
element of a child is its unconstrained nodes followed by the coarse parent
nodes, each node's dof numbered forward (logic's Nodm / nacH / constrH).
"""
from __future__ import annotations

import numpy as np
import scipy.sparse as sp
import scipy.sparse.linalg as spla

from hp3d_gb300 import mesh as M
from oracle import oracle as O

_VOFF = np.array([[0, 0, 0], [1, 0, 0], [1, 1, 0], [0, 1, 0],
                  [0, 0, 1], [1, 0, 1], [1, 1, 1], [0, 1, 1]])
_EDGES = [e for e, _ in M._HEXA_EDGES]
_FACES = [f for f, _ in M._HEXA_FACES]


def _face_nodes(f):
    """Element node indices (vertices, edges, the face) of hexa face f."""
    fv = set(_FACES[f])
    nodes = sorted(fv)
    nodes += [8 + q for q, (a, b) in enumerate(_EDGES) if a in fv and b in fv]
    nodes.append(20 + f)
    return nodes


def hanging_mesh(p, nc=3, perturb=0.0):
    """nc^3 coarse boxes, the centre one refined into 8 children; returns the
    mesh dict and the per-element constraint data (None for unconstrained
    elements)."""
    assert nc % 2 == 1
    n = 2 * nc
    nv1 = n + 1
    idx = np.arange(nv1)
    I, J, K = np.meshgrid(idx, idx, idx, indexing="ij")
    grid = np.stack([I.ravel(order="F"), J.ravel(order="F"), K.ravel(order="F")], axis=1)
    X = grid / n
    vid = lambda c: int(c[0] + nv1 * (c[1] + nv1 * c[2]))  # noqa: E731
    ctr = np.array([nc // 2] * 3)
    et, verts, orders, kind = [], [], [], []
    for k in range(nc):
        for j in range(nc):
            for i in range(nc):
                c = np.array([i, j, k])
                if np.array_equal(c, ctr):
                    continue
                et.append(M.HEXA)
                verts.append([vid(2 * (c + v)) for v in _VOFF])
                orders.append((p, p, p))
                kind.append(("coarse", c))
    for o in _VOFF:
        cf = 2 * ctr + o
        et.append(M.HEXA)
        verts.append([vid(cf + v) for v in _VOFF])
        orders.append((p, p, p))
        kind.append(("child", o))
    m = M.build_mesh(et, verts, X, grid, n, orders)
    cons = _constraints(m, kind, ctr, n)
    return m, cons


def _xi_of(xv, x):
    """Reference coordinates of x in an axis-aligned box element whose local
    vertex 0 is its lower corner and vertex 6 its upper corner."""
    lo, hi = xv[0], xv[6]
    return (x - lo) / (hi - lo)


def _constraints(m, kind, ctr, n):
    ne = m["nelem"]
    no = m["norder"]
    coarse_nodes = set()
    for e in range(ne):
        if kind[e][0] == "coarse":
            coarse_nodes.update(int(g) for g in m["nodes"][e, :26])
    lo_c, hi_c = ctr / (n // 2), (ctr + 1) / (n // 2)
    out = []
    for e in range(ne):
        if kind[e][0] != "child":
            out.append(None)
            continue
        xv = m["xvert"][e][:8]
        nd = O.node_ndof(M.HEXA, no[e])
        first = np.concatenate([[0], np.cumsum(nd)]).astype(int)
        ni = int(first[-1])
        gid = [int(g) for g in m["nodes"][e, :26]]
        constrained = [i >= 8 and gid[i] not in coarse_nodes and _on_ctr_boundary(
            _node_point(xv, i), lo_c, hi_c) for i in range(26)]
        # vertices too: a child vertex at an edge midpoint / face centre of the
        # centre cube is not a coarse vertex
        for i in range(8):
            constrained[i] = gid[i] not in coarse_nodes and _on_ctr_boundary(xv[i], lo_c, hi_c)
        # modified nodes: the child's unconstrained nodes, then parents
        nodm, ndof, bc = [], [], []
        mod_first = {}
        for i in range(26):
            if not constrained[i]:
                mod_first[("own", i)] = sum(ndof)
                nodm.append(gid[i]); ndof.append(int(nd[i])); bc.append(int(m["bcflag"][e, i]))
        coef = {}
        for i in range(26):
            if not constrained[i]:
                for j in range(nd[i]):
                    coef[(first[i] + j, mod_first[("own", i)] + j)] = 1.0
        for f in range(6):
            pts_c = np.array([xv[q] for q in _FACES[f]])
            ax = [a for a in range(3) if np.ptp(pts_c[:, a]) < 1e-14]
            if not ax:
                continue
            a = ax[0]
            val = pts_c[0, a]
            if not (abs(val - lo_c[a]) < 1e-14 or abs(val - hi_c[a]) < 1e-14):
                continue
            # coarse neighbour across this centre-cube face and its face
            step = np.zeros(3, int)
            step[a] = 1 if abs(val - hi_c[a]) < 1e-14 else -1
            cn = ctr + step
            en = [q for q in range(ne) if kind[q][0] == "coarse" and np.array_equal(kind[q][1], cn)]
            assert len(en) == 1
            en = en[0]
            xvn = m["xvert"][en][:8]
            fn = [g for g in range(6)
                  if np.ptp(np.array([xvn[q] for q in _FACES[g]])[:, a]) < 1e-14
                  and abs(xvn[_FACES[g][0]][a] - val) < 1e-14][0]
            ndn = O.node_ndof(M.HEXA, no[en])
            firstn = np.concatenate([[0], np.cumsum(ndn)]).astype(int)
            cols_c = [first[i] + j for i in _face_nodes(f) for j in range(nd[i])]
            par = [(i, j) for i in _face_nodes(fn) for j in range(ndn[i])]
            # sample points on the child face (a 2D Gauss rule in its plane)
            g1, _ = O.gauss1d(int(no[e][0]) + 3)
            t = [q for q in range(3) if q != a]
            lo_f, hi_f = pts_c.min(0), pts_c.max(0)
            A, Bm = [], []
            for s1 in g1:
                for s2 in g1:
                    x = np.array(lo_f, float)
                    x[t[0]] = lo_f[t[0]] + s1 * (hi_f[t[0]] - lo_f[t[0]])
                    x[t[1]] = lo_f[t[1]] + s2 * (hi_f[t[1]] - lo_f[t[1]])
                    sc, _ = O.shape_hexa(_xi_of(xv, x), no[e], m["nori_edge"][e], m["nori_face"][e])
                    sn, _ = O.shape_hexa(_xi_of(xvn, x), no[en], m["nori_edge"][en],
                                         m["nori_face"][en])
                    A.append(sc[cols_c])
                    Bm.append([sn[firstn[i] + j] for i, j in par])
            A = np.array(A); Bm = np.array(Bm)
            sol, res, rank, _ = np.linalg.lstsq(A, Bm, rcond=None)
            assert rank == A.shape[1]
            assert np.abs(A @ sol - Bm).max() < 1e-11
            for (i, j) in par:
                g = int(m["nodes"][en, i])
                if ("par", g) not in mod_first:
                    mod_first[("par", g)] = sum(ndof)
                    nodm.append(g); ndof.append(int(ndn[i])); bc.append(int(m["bcflag"][en, i]))
            for r, k in enumerate(cols_c):
                inode = int(np.searchsorted(first, k, side="right") - 1)
                if not constrained[inode]:
                    continue
                for q, (i, j) in enumerate(par):
                    v = sol[r, q]
                    if abs(v) < 1e-13:
                        continue
                    l = mod_first[("par", int(m["nodes"][en, i]))] + j
                    key = (k, l)
                    if key in coef:
                        assert abs(coef[key] - v) < 1e-10
                    coef[key] = v
        items = sorted(coef.items())
        ck = np.array([k for (k, _), _ in items], np.int32)
        cl = np.array([l for (_, l), _ in items], np.int32)
        cv = np.array([v for _, v in items])
        out.append(dict(nodm=np.array(nodm, np.int32), ndof=np.array(ndof, np.int32),
                        bc=np.array(bc, np.int32), ck=ck, cl=cl, cv=cv, ni=ni,
                        nmod=int(sum(ndof))))
    return out


def _node_point(xv, i):
    if i < 8:
        return xv[i]
    if i < 20:
        a, b = _EDGES[i - 8]
        return 0.5 * (xv[a] + xv[b])
    return np.mean([xv[q] for q in _FACES[i - 20]], axis=0)


def _on_ctr_boundary(x, lo, hi, tol=1e-12):
    inside = np.all(x >= lo - tol) and np.all(x <= hi + tol)
    on = np.any(np.abs(x - lo) < tol) or np.any(np.abs(x - hi) < tol)
    return bool(inside and on)


def oracle_outputs(m, cons, isol, zdofd):
    """Condensed, constrained and compressed element systems by the oracle,
    with the node lists the index maps walk; zdofd: per element Dirichlet
    values of the interface dof (the children are interior)."""
    res = []
    for e in range(m["nelem"]):
        K, b, rc = O.elem(M.HEXA, m["norder"][e], m["nori_edge"][e], m["nori_face"][e],
                          m["xvert"][e][:8], m["kappa"][e], isol=isol)
        assert rc == 0
        nb = O.nrdof_bubble(M.HEXA, m["norder"][e])
        aii, bi, asch, bsch, rc = O.stc_fwd(K, b, nb, 1)
        assert rc == 0
        c = cons[e]
        if c is None:
            nx, zb, zs, ndofm = O.celem_compress(M.HEXA, m["norder"][e], m["bcflag"][e], aii, bi,
                                                 zdofd[e])
            nodes = m["nodes"][e, :26]
            nd_act = ndofm[:26]
        else:
            am, bm = O.constrain(aii, bi, c["ck"], c["cl"], c["cv"], c["nmod"])
            nx, zb, zs, ndofm = O.celem_compress_nodes(c["ndof"], c["bc"], am, bm)
            nodes = c["nodm"]
            nd_act = ndofm
        res.append(dict(nextract=nx, zbload=zb, zastif=zs, nodes=np.asarray(nodes),
                        ndofm=np.asarray(nd_act), aschur=asch, bschur=bsch, ni=aii.shape[0]))
    return res


def solve_error(m, cons, elems, isol, zdofd):
    """Assemble through LCON over the (modified) node lists, solve, recover
    element dof (x_elem = C x_mod for constrained elements), back-substitute
    the bubbles and return the H1 error and norm."""
    ne = m["nelem"]
    nmax = max(len(el["nodes"]) for el in elems)
    nodes = -np.ones((ne, nmax), np.int32)
    ndofm = np.zeros((ne, nmax), np.int32)
    nnode = np.zeros(ne, np.int32)
    for e, el in enumerate(elems):
        k = len(el["nodes"])
        nodes[e, :k] = el["nodes"]; ndofm[e, :k] = el["ndofm"]; nnode[e] = k
    nrdof, nfirst, lcon, lcon_off, elem_nnz = O.index_maps(nnode, nodes, ndofm, m["nnodes"])
    rows, cols, vals = [], [], []
    rhs = np.zeros(nrdof)
    for e in range(ne):
        lc = lcon[lcon_off[e]:lcon_off[e + 1]] - 1
        rows.append(np.repeat(lc, len(lc))); cols.append(np.tile(lc, len(lc)))
        vals.append(elems[e]["zastif"].ravel())
        np.add.at(rhs, lc, elems[e]["zbload"])
    A = sp.coo_matrix((np.concatenate(vals), (np.concatenate(rows), np.concatenate(cols))),
                      shape=(nrdof, nrdof)).tocsc()
    x = spla.spsolve(A, rhs)
    err2 = nrm2 = 0.0
    L = O.lib()
    for e in range(ne):
        el = elems[e]
        c = cons[e]
        lc = lcon[lcon_off[e]:lcon_off[e + 1]] - 1
        if c is None:
            xi = zdofd[e].copy()
            xi[el["nextract"]] = x[lc]
        else:
            xm = np.zeros(c["nmod"])
            xm[el["nextract"]] = x[lc]
            xi = np.zeros(el["ni"])
            np.add.at(xi, c["ck"], c["cv"] * xm[c["cl"]])
        xb = O.stc_bwd(el["aschur"], el["bschur"], xi)
        dof = np.concatenate([xi, xb])
        xn = np.zeros((len(dof), 3)); xn[:8] = m["xvert"][e][:8]
        e2 = np.zeros(1); r2 = np.zeros(1)
        L.orc_element_error(M.HEXA, O._p(O._i32(m["norder"][e]), O._i32p),
                            O._p(O._i32(m["nori_edge"][e]), O._i32p),
                            O._p(O._i32(m["nori_face"][e]), O._i32p),
                            O._p(O._f64(xn), O._f64p), O._p(O._f64(dof), O._f64p), isol,
                            O._p(e2, O._f64p), O._p(r2, O._f64p))
        err2 += e2[0]; nrm2 += r2[0]
    return np.sqrt(err2), np.sqrt(nrm2), (nrdof, nfirst, lcon, lcon_off, elem_nnz)
