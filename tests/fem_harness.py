"""End-to-end finite-element harness for the restated reference tests.

The reference pins its element pass only end to end: test/poly_pois.F90 and
test/conv_pois.F90 refine, interpolate Dirichlet data (update_Ddof), assemble
and solve through mumps_sc + MUMPS, back-substitute the bubbles (solout ->
stc_bwd) and integrate the H1 error (element_error).  MUMPS is not available,
so this harness assembles the same triplets (mumps_sc.F90:300-321) into a
SciPy sparse matrix and solves it directly.  Element outputs come either from
the CPU oracle or from the GPU library; both feed the same assembly.
"""
from __future__ import annotations

import numpy as np
import scipy.sparse as sp
import scipy.sparse.linalg as spla

from oracle import oracle as O
from hp3d_gb300 import mesh as M

# local vertex numbers of each hexa edge / face (element_data.F90 hexa tables)
HEXA_EDGE_V = [(0, 1), (1, 2), (3, 2), (0, 3), (4, 5), (5, 6), (7, 6), (4, 7),
               (0, 4), (1, 5), (2, 6), (3, 7)]
# reference coordinate parametrisation of each face: fixed axis/value, (s,t) axes
HEXA_FACE = [(2, 0.0, 0, 1), (2, 1.0, 0, 1), (1, 0.0, 0, 2), (0, 1.0, 1, 2),
             (1, 1.0, 0, 2), (0, 0.0, 1, 2)]
_VREF = np.array([[0, 0, 0], [1, 0, 0], [1, 1, 0], [0, 1, 0],
                  [0, 0, 1], [1, 0, 1], [1, 1, 1], [0, 1, 1]], dtype=float)
# tetrahedron and prism reference vertices (BlendProject.F90 BlendTetV, BlendPrisV)
TET_VREF = np.array([[0, 0, 0], [1, 0, 0], [0, 1, 0], [0, 0, 1]], dtype=float)
PRISM_VREF = np.array([[0, 0, 0], [1, 0, 0], [0, 1, 0], [0, 0, 1], [1, 0, 1], [0, 1, 1]],
                      dtype=float)
TET_EDGE_V = [(0, 1), (1, 2), (0, 2), (0, 3), (1, 3), (2, 3)]
TET_FACE_V = [(0, 1, 2), (0, 1, 3), (1, 2, 3), (0, 2, 3)]

HEXA, PRISM, TET = 1, 2, 3


def type_info(etype):
    """(vertex count, node count, reference vertices, edge vertex pairs,
    face vertex lists in the element's frame order)."""
    nv, edges, faces = M._TOPO[etype]
    vref = {HEXA: _VREF, PRISM: PRISM_VREF, TET: TET_VREF}[etype]
    return nv, nv + len(edges) + len(faces), vref, [e for e, _ in edges], [f for f, _ in faces]


def nnode_of(mesh):
    return np.array([type_info(int(t))[1] for t in mesh["etype"]], dtype=np.int32)


def _xmap(xv, shap):
    return shap[: len(xv)] @ xv


def _face_points(etype, f):
    """Quadrature points (reference coordinates) and weights on face f:
    a collapsed Gauss rule on triangles, a bilinear map of the unit square
    through the face's vertices on quadrilaterals."""
    vref, fv = type_info(etype)[2], type_info(etype)[4][f]
    gs, gw = O.gauss1d(8)
    pts, wts = [], []
    V = [vref[q] for q in fv]
    for s1, w1 in zip(gs, gw):
        for t1, w2 in zip(gs, gw):
            if len(V) == 3:
                u, v = s1 * (1 - t1), t1
                pts.append(V[0] + u * (V[1] - V[0]) + v * (V[2] - V[0]))
                wts.append(w1 * w2 * (1 - t1))
            else:
                pts.append((1 - s1) * (1 - t1) * V[0] + s1 * (1 - t1) * V[1] + s1 * t1 * V[2]
                           + (1 - s1) * t1 * V[3])
                wts.append(w1 * w2)
    return pts, wts


def dirichlet_data(mesh, isol):
    """Per element, per interface dof (element order) Dirichlet values:
    vertex values, then discrete L2 projections on edges and faces of what
    the vertex (and edge) interpolant leaves -- a projection-based
    interpolant of the boundary trace in the spirit of update_Ddof."""
    ne = mesh["nelem"]
    no = mesh["norder"]
    nodes = mesh["nodes"]
    bc = mesh["bcflag"]
    known = {}
    out = []
    for e in range(ne):
        et = int(mesh["etype"][e])
        nv, nn, vref, edges, _ = type_info(et)
        nd = O.node_ndof(et, no[e])
        first = np.concatenate([[0], np.cumsum(nd)])
        ni = int(first[-1])
        z = np.zeros(ni)
        xv = mesh["xvert"][e][:nv]
        ne_, nf_ = mesh["nori_edge"][e], mesh["nori_face"][e]
        nedge = len(edges)
        for i in range(nn):
            if not bc[e, i] or nd[i] == 0:
                continue
            g = int(nodes[e, i])
            if g in known:
                z[first[i]:first[i + 1]] = known[g]
                continue
            if i < nv:
                s, _ = O.shape(et, vref[i], no[e], ne_, nf_)
                u, _ = O.exact(isol, _xmap(xv, s))
                val = np.array([u])
            elif i < nv + nedge:
                a, b = edges[i - nv]
                gs, gw = O.gauss1d(8)
                rows, rhs = [], []
                for t, w in zip(gs, gw):
                    xi = (1 - t) * vref[a] + t * vref[b]
                    s, _ = O.shape(et, xi, no[e], ne_, nf_)
                    u, _ = O.exact(isol, _xmap(xv, s))
                    uv = s[a] * z[first[a]] + s[b] * z[first[b]]
                    rows.append(np.sqrt(w) * s[first[i]:first[i + 1]])
                    rhs.append(np.sqrt(w) * (u - uv))
                val = np.linalg.lstsq(np.array(rows), np.array(rhs), rcond=None)[0]
            else:
                pts, wts = _face_points(et, i - nv - nedge)
                rows, rhs = [], []
                for xi, w in zip(pts, wts):
                    s, _ = O.shape(et, xi, no[e], ne_, nf_)
                    u, _ = O.exact(isol, _xmap(xv, s))
                    known_part = s[:first[nv + nedge]] @ z[:first[nv + nedge]]
                    rows.append(np.sqrt(w) * s[first[i]:first[i + 1]])
                    rhs.append(np.sqrt(w) * (u - known_part))
                val = np.linalg.lstsq(np.array(rows), np.array(rhs), rcond=None)[0]
            known[g] = val
            z[first[i]:first[i + 1]] = val
        out.append(z)
    return out


def oracle_element_outputs(mesh, isol, integration=0, zdofd=None, stc_method=0):
    """Per-element outputs of the oracle: list of dicts with the condensed
    compressed system, Schur blocks and per-node active dof counts."""
    res = []
    for e in range(mesh["nelem"]):
        et = int(mesh["etype"][e])
        nv = type_info(et)[0]
        K, b, rc = O.elem(et, mesh["norder"][e], mesh["nori_edge"][e], mesh["nori_face"][e],
                          mesh["xvert"][e][:nv], mesh["kappa"][e], isol=isol,
                          integration=integration)
        assert rc == 0
        nb = O.nrdof_bubble(et, mesh["norder"][e])
        if nb > 0:
            aii, bi, asch, bsch, rc = O.stc_fwd(K, b, nb, stc_method)
            assert rc == 0
        else:
            aii, bi = K, b
            asch = np.zeros((0, K.shape[0])); bsch = np.zeros(0)
        zd = None if zdofd is None else zdofd[e]
        nextract, zb, zs, ndofm = O.celem_compress(et, mesh["norder"][e], mesh["bcflag"][e],
                                                   aii, bi, zd)
        nd26 = np.zeros(26, dtype=np.int32)
        nd26[: len(ndofm)] = ndofm[:26]
        res.append(dict(nextract=nextract, zbload=zb, zastif=zs, ndofm=nd26,
                        aschur=asch, bschur=bsch, ni=aii.shape[0], nb=nb))
    return res


def assemble_solve(mesh, elems):
    """Assemble the condensed interface system from per-element outputs
    (mumps_sc.F90:300-321 triplets) and solve it; returns the global interface
    solution x and the index maps."""
    ne = mesh["nelem"]
    nnode = nnode_of(mesh)
    ndofm = np.stack([el["ndofm"] for el in elems]).astype(np.int32)
    nrdof, nfirst, lcon, lcon_off, elem_nnz = O.index_maps(nnode, mesh["nodes"], ndofm,
                                                           mesh["nnodes"])
    rows, cols, vals = [], [], []
    rhs = np.zeros(nrdof)
    for e in range(ne):
        lc = lcon[lcon_off[e]:lcon_off[e + 1]] - 1
        nc = len(lc)
        if nc == 0:
            continue
        rows.append(np.repeat(lc, nc)); cols.append(np.tile(lc, nc))
        vals.append(elems[e]["zastif"].ravel())
        np.add.at(rhs, lc, elems[e]["zbload"])
    A = sp.coo_matrix((np.concatenate(vals), (np.concatenate(rows), np.concatenate(cols))),
                      shape=(nrdof, nrdof)).tocsc()
    x = spla.spsolve(A, rhs) if nrdof > 0 else np.zeros(0)
    return x, lcon, lcon_off


def solve_and_error(mesh, elems, isol, zdofd=None):
    """Assemble the condensed interface system from per-element outputs
    (dicts with nextract/zbload/zastif/ndofm/aschur/bschur), solve it,
    back-substitute bubbles and return (H1 error, H1 norm, global solution,
    per-element full dof vectors)."""
    ne = mesh["nelem"]
    nnode = nnode_of(mesh)
    ndofm = np.stack([el["ndofm"] for el in elems]).astype(np.int32)
    nrdof, nfirst, lcon, lcon_off, elem_nnz = O.index_maps(nnode, mesh["nodes"], ndofm,
                                                           mesh["nnodes"])
    rows, cols, vals = [], [], []
    rhs = np.zeros(nrdof)
    for e in range(ne):
        lc = lcon[lcon_off[e]:lcon_off[e + 1]] - 1
        nc = len(lc)
        if nc == 0:
            continue
        rows.append(np.repeat(lc, nc)); cols.append(np.tile(lc, nc))
        vals.append(elems[e]["zastif"].ravel())
        np.add.at(rhs, lc, elems[e]["zbload"])
    A = sp.coo_matrix((np.concatenate(vals), (np.concatenate(rows), np.concatenate(cols))),
                      shape=(nrdof, nrdof)).tocsc()
    x = spla.spsolve(A, rhs) if nrdof > 0 else np.zeros(0)
    err2 = 0.0; nrm2 = 0.0
    dofs = []
    for e in range(ne):
        el = elems[e]
        ni = el["ni"]
        xi = np.zeros(ni) if zdofd is None else zdofd[e].copy()
        lc = lcon[lcon_off[e]:lcon_off[e + 1]] - 1
        xi[el["nextract"]] = x[lc]
        xb = O.stc_bwd(el["aschur"], el["bschur"], xi) if el["nb"] > 0 else np.zeros(0)
        dof = np.concatenate([xi, xb])
        dofs.append(dof)
        n = len(dof)
        et = int(mesh["etype"][e])
        nv = type_info(et)[0]
        xn = np.zeros((n, 3)); xn[:nv] = mesh["xvert"][e][:nv]
        e2 = np.zeros(1); r2 = np.zeros(1)
        L = O.lib()
        L.orc_element_error(et, O._p(O._i32(mesh["norder"][e]), O._i32p),
                            O._p(O._i32(mesh["nori_edge"][e]), O._i32p),
                            O._p(O._i32(mesh["nori_face"][e]), O._i32p),
                            O._p(O._f64(xn), O._f64p), O._p(O._f64(dof), O._f64p), isol,
                            O._p(e2, O._f64p), O._p(r2, O._f64p))
        err2 += e2[0]; nrm2 += r2[0]
    return np.sqrt(err2), np.sqrt(nrm2), x, dofs


def gpu_elements(ep, m):
    """Per-element outputs of the GPU library in the form the harness
    assembles (NEXTRACT rebuilt from the node dof counts: nodes in reverse
    order, Dirichlet nodes skipped)."""
    out = []
    for e in range(m["nelem"]):
        zb, zs = ep.condensed(e)
        a, b = ep.schur(e)
        et = int(m["etype"][e])
        nd = O.node_ndof(et, m["norder"][e])
        nn = len(nd)
        ndofm = np.zeros(26, dtype=np.int32)
        ndofm[:nn] = nd * (1 - m["bcflag"][e][:nn])
        first = np.concatenate([[0], np.cumsum(nd)])
        nx = [first[i] + q for i in range(nn - 1, -1, -1) for q in range(ndofm[i])]
        out.append(dict(nextract=np.array(nx, dtype=np.int64), zbload=zb, zastif=zs, ndofm=ndofm,
                        aschur=a, bschur=b, ni=int(nd.sum()), nb=a.shape[0]))
    return out
