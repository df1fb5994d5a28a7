"""Synthetic hexahedral meshes in the element-descriptor form of the C-ABI.

The reference builds its meshes through GMP + ``hp3gen`` + refinement; the
element pass only sees, per element, what ``find_order``/``find_orient``/
``nodcor``/``get_index`` return (problems/POISSON/GALERKIN/elem_opt.F90:66-74,
constrs/celem_systemI.F90:290-350).  These generators produce exactly that
descriptor for structured meshes of the unit cube:

* ``norder``  (19)  edge orders, face orders (MODORDER=10 packed), interior
  order (111*p style packing, set_initial_mesh.F90:56-62);
* ``nori_edge`` (12), ``nori_face`` (6) orientation codes;
* ``nodes`` (26)   global ids of vertex, edge and face nodes in element order
  (vertices v1..v8, edges e1..e12, faces f1..f6 as in
  src/modules/element_data.F90);
* ``bcflag`` (26)  1 when the node lies on a Dirichlet boundary (all its dof
  are known, get_index index=1);
* ``xvert`` (8,3)  vertex coordinates: trilinear geometry, higher-order
  geometry dof zero (EXGEOM=0, nodcor);
* ``kappa``        per-element coefficient.

Element node local numbering follows the hexahedron of the reference
(BlendProject.F90:197-439): v1=(0,0,0) v2=(1,0,0) v3=(1,1,0) v4=(0,1,0)
v5..v8 the same at z=1; edges e1=v1v2 e2=v2v3 e3=v4v3 e4=v1v4 e5=v5v6
e6=v6v7 e7=v8v7 e8=v5v8 e9=v1v5 e10=v2v6 e11=v3v7 e12=v4v8; faces
f1=z0 f2=z1 f3=y0 f4=x1 f5=y1 f6=x0.  On a lexicographically numbered grid
every local edge/face axis is aligned with the global one, so all
orientation codes are 0.
"""
from __future__ import annotations

import numpy as np

HEXA = 1

# vertex offsets (di,dj,dk)
_VOFF = np.array([[0, 0, 0], [1, 0, 0], [1, 1, 0], [0, 1, 0],
                  [0, 0, 1], [1, 0, 1], [1, 1, 1], [0, 1, 1]])
# edges: (axis, di, dj, dk) of the edge's start point
_EDEF = [(0, 0, 0, 0), (1, 1, 0, 0), (0, 0, 1, 0), (1, 0, 0, 0),
         (0, 0, 0, 1), (1, 1, 0, 1), (0, 0, 1, 1), (1, 0, 0, 1),
         (2, 0, 0, 0), (2, 1, 0, 0), (2, 1, 1, 0), (2, 0, 1, 0)]
# faces: (normal axis, di, dj, dk)
_FDEF = [(2, 0, 0, 0), (2, 0, 0, 1), (1, 0, 0, 0), (0, 1, 0, 0), (1, 0, 1, 0), (0, 0, 0, 0)]


def pack_order_hexa(p):
    """Norder(19) of an isotropic hexa of order p (find_order form)."""
    if np.isscalar(p):
        px = py = pz = int(p)
    else:
        px, py, pz = (int(v) for v in p)
    no = np.zeros(19, dtype=np.int32)
    for e, (ax, *_r) in enumerate(_EDEF):
        no[e] = (px, py, pz)[ax]
    face_axes = [(0, 1), (0, 1), (0, 2), (1, 2), (0, 2), (1, 2)]
    for f, (a, b) in enumerate(face_axes):
        pa, pb = (px, py, pz)[a], (px, py, pz)[b]
        no[12 + f] = 10 * pa + pb
    no[18] = 100 * px + 10 * py + pz
    return no


def structured_hexa(n, p, perturb=0.0, kappa_logrange=None, seed=12345,
                    dirichlet=True):
    """n x n x n hexahedra on [0,1]^3 of order p.

    perturb:  interior vertices moved by U(-perturb*h, +perturb*h) per
              coordinate (trilinear curvilinear geometry).
    kappa_logrange: (lo, hi) decades, kappa_e = 10**U(lo, hi); None -> 1.
    """
    rng = np.random.default_rng(seed)
    nv1 = n + 1
    h = 1.0 / n
    idx = np.arange(nv1)
    I, J, K = np.meshgrid(idx, idx, idx, indexing="ij")
    coords = np.stack([I.ravel(order="F"), J.ravel(order="F"), K.ravel(order="F")], axis=1)
    # vertex id = i + nv1*(j + nv1*k)
    vid = lambda i, j, k: i + nv1 * (j + nv1 * k)  # noqa: E731
    X = coords.astype(np.float64) * h
    if perturb > 0.0:
        interior = np.all((coords > 0) & (coords < n), axis=1)
        d = rng.uniform(-perturb * h, perturb * h, size=X.shape)
        X[interior] += d[interior]
    nverts = nv1 ** 3
    # edge ids per axis: axis a edges have n along a and nv1 along the others
    def eid(ax, i, j, k):
        if ax == 0:
            return nverts + i + n * (j + nv1 * k)
        if ax == 1:
            return nverts + n * nv1 * nv1 + i + nv1 * (j + n * k)
        return nverts + 2 * n * nv1 * nv1 + i + nv1 * (j + nv1 * k)
    nedges = 3 * n * nv1 * nv1
    def fid(ax, i, j, k):
        base = nverts + nedges
        if ax == 2:  # normal z: n x n x nv1
            return base + i + n * (j + n * k)
        if ax == 1:  # normal y: n x nv1 x n
            return base + n * n * nv1 + i + n * (j + nv1 * k)
        return base + 2 * n * n * nv1 + i + nv1 * (j + n * k)
    nfaces = 3 * n * n * nv1
    nnodes = nverts + nedges + nfaces
    ne = n ** 3
    nodes = np.zeros((ne, 26), dtype=np.int32)
    bcflag = np.zeros((ne, 26), dtype=np.int32)
    xvert = np.zeros((ne, 8, 3))
    e = 0
    for k in range(n):
        for j in range(n):
            for i in range(n):
                for v in range(8):
                    di, dj, dk = _VOFF[v]
                    nodes[e, v] = vid(i + di, j + dj, k + dk)
                    xvert[e, v] = X[nodes[e, v]]
                    bcflag[e, v] = int(i + di in (0, n) or j + dj in (0, n) or k + dk in (0, n))
                for q, (ax, di, dj, dk) in enumerate(_EDEF):
                    nodes[e, 8 + q] = eid(ax, i + di, j + dj, k + dk)
                    c = [i + di, j + dj, k + dk]
                    bcflag[e, 8 + q] = int(any(c[a] in (0, n) for a in range(3) if a != ax))
                for q, (ax, di, dj, dk) in enumerate(_FDEF):
                    nodes[e, 20 + q] = fid(ax, i + di, j + dj, k + dk)
                    c = [i + di, j + dj, k + dk]
                    bcflag[e, 20 + q] = int(c[ax] in (0, n))
                e += 1
    if not dirichlet:
        bcflag[:] = 0
    if kappa_logrange is None:
        kappa = np.ones(ne)
    else:
        lo, hi = kappa_logrange
        kappa = 10.0 ** rng.uniform(lo, hi, size=ne)
    no = pack_order_hexa(p)
    return dict(
        nelem=ne, n=n, h=h, p=p, nnodes=nnodes, nverts=nverts,
        etype=np.full(ne, HEXA, dtype=np.int32),
        norder=np.tile(no, (ne, 1)).astype(np.int32),
        nori_edge=np.zeros((ne, 12), dtype=np.int32),
        nori_face=np.zeros((ne, 6), dtype=np.int32),
        nodes=nodes, bcflag=bcflag, xvert=xvert, kappa=kappa,
        vertex_xyz=X,
    )


def random_orientations(mesh, seed=7):
    """Copy of ``mesh`` with random edge (0/1) and face (0..7) orientation
    codes: for element-level parity of orientation handling (the result is
    not a conforming global mesh)."""
    rng = np.random.default_rng(seed)
    m = dict(mesh)
    ne = mesh["nelem"]
    m["nori_edge"] = rng.integers(0, 2, size=(ne, 12)).astype(np.int32)
    m["nori_face"] = rng.integers(0, 8, size=(ne, 6)).astype(np.int32)
    return m


def hp_hexa(n, seed=2024, perturb=0.0, kappa_logrange=(-1, 1), pmax=6, dirichlet=True):
    """n^3 hexahedra of the unit cube with per-element anisotropic orders.

    Each (px, py, pz) is drawn in 1..pmax from a seeded geometric
    distribution whose mean grows with the distance of the element centre
    from the corner (0,0,0), so orders fall toward that corner.  Edge and face
    orders follow the minimum rule of the reference's adaptivity
    (adapt/enforce_min_rule.F90): an edge takes the minimum order of the
    elements sharing it along its direction, a face the minimum of its two
    elements along each of its axes.  Orientations are 0 (lexicographic
    grid), so local and global face frames coincide.
    """
    m = structured_hexa(n, 1, perturb=perturb, kappa_logrange=kappa_logrange, seed=seed,
                        dirichlet=dirichlet)
    rng = np.random.default_rng(seed + 1)
    ne = m["nelem"]
    orders = np.zeros((ne, 3), dtype=np.int32)
    e = 0
    centres = np.zeros((ne, 3))
    for k in range(n):
        for j in range(n):
            for i in range(n):
                centres[e] = (np.array([i, j, k]) + 0.5) / n
                e += 1
    r = np.linalg.norm(centres, axis=1) / np.sqrt(3.0)
    mean = 1.0 + (pmax - 1) * r  # mean order 1 at the corner, pmax far away
    for a in range(3):
        q = 1.0 / np.maximum(mean, 1.0)  # geometric with mean 1/q on {1,2,...}
        orders[:, a] = np.minimum(rng.geometric(q), pmax)
    # min rule over shared edges / faces
    edge_min = {}
    face_min = {}
    for e in range(ne):
        for q in range(12):
            g = int(m["nodes"][e, 8 + q])
            ax = _EDEF[q][0]
            edge_min[g] = min(edge_min.get(g, 99), int(orders[e, ax]))
        for q in range(6):
            g = int(m["nodes"][e, 20 + q])
            a1, a2 = [(0, 1), (0, 1), (0, 2), (1, 2), (0, 2), (1, 2)][q]
            cur = face_min.get(g, (99, 99))
            face_min[g] = (min(cur[0], int(orders[e, a1])), min(cur[1], int(orders[e, a2])))
    norder = np.zeros((ne, 19), dtype=np.int32)
    for e in range(ne):
        for q in range(12):
            norder[e, q] = edge_min[int(m["nodes"][e, 8 + q])]
        for q in range(6):
            o1, o2 = face_min[int(m["nodes"][e, 20 + q])]
            norder[e, 12 + q] = 10 * o1 + o2
        norder[e, 18] = 100 * orders[e, 0] + 10 * orders[e, 1] + orders[e, 2]
    m["norder"] = norder
    m["p"] = None
    m["orders"] = orders
    return m


TET = 3
# tetrahedron local edges / faces (shape_1/BlendProject.F90 ProjectTetE/F)
TET_EDGES = [(0, 1), (1, 2), (0, 2), (0, 3), (1, 3), (2, 3)]
TET_FACES = [(0, 1, 2), (0, 1, 3), (1, 2, 3), (0, 2, 3)]
# OrientTri: GS(k) = S(Or(nori, k)) (shape_1/Orient.F90:119-162)
ORIENT_TRI = [(0, 1, 2), (1, 2, 0), (2, 0, 1), (0, 2, 1), (1, 0, 2), (2, 1, 0)]


def tri_orientation(local, glob):
    """Orientation code o with local[ORIENT_TRI[o][k]] == glob[k]: the
    element's face functions then use the face node's own vertex order, so
    neighbours share their traces."""
    for o, perm in enumerate(ORIENT_TRI):
        if all(local[perm[k]] == glob[k] for k in range(3)):
            return o
    raise ValueError("face vertices do not match")


def _on_boundary(pts, n):
    """A straight edge or flat face lies on a face of the cube [0,n]^3 of
    grid indices when all its vertices share a coordinate equal to 0 or n."""
    pts = np.asarray(pts)
    for c in range(3):
        if np.all(pts[:, c] == 0) or np.all(pts[:, c] == n):
            return True
    return False


def _kappa(rng, ne, kappa_logrange):
    if kappa_logrange is None:
        return np.ones(ne)
    lo, hi = kappa_logrange
    return 10.0 ** rng.uniform(lo, hi, size=ne)


def structured_tet(n, p, perturb=0.0, kappa_logrange=None, seed=12345, dirichlet=True,
                   orders=None):
    """n^3 cubes of [0,1]^3, each split into the 6 tetrahedra of the Kuhn
    (Freudenthal) subdivision along its main diagonal, so neighbouring cubes
    share their face diagonals and the mesh is conforming.

    Element vertices follow the Kuhn path c, c+e_a, c+e_a+e_b, c+(1,1,1),
    with the last two swapped where that makes the Jacobian positive.  Edge
    nodes are oriented from the lower to the higher vertex id and face nodes
    list their vertices in increasing id; each element's codes follow from
    its local order (tri_orientation).  orders: optional per-element tet
    order (interior), edges and faces then take the minimum of their
    elements (min rule); otherwise all orders are p.
    """
    rng = np.random.default_rng(seed)
    nv1 = n + 1
    h = 1.0 / n
    idx = np.arange(nv1)
    I, J, K = np.meshgrid(idx, idx, idx, indexing="ij")
    coords = np.stack([I.ravel(order="F"), J.ravel(order="F"), K.ravel(order="F")], axis=1)
    X = coords.astype(np.float64) * h
    if perturb > 0.0:
        interior = np.all((coords > 0) & (coords < n), axis=1)
        d = rng.uniform(-perturb * h, perturb * h, size=X.shape)
        X[interior] += d[interior]
    vid = lambda i, j, k: i + nv1 * (j + nv1 * k)  # noqa: E731
    unit = np.eye(3, dtype=int)
    perms = [(0, 1, 2), (0, 2, 1), (1, 0, 2), (1, 2, 0), (2, 0, 1), (2, 1, 0)]
    tets = []
    for k in range(n):
        for j in range(n):
            for i in range(n):
                c = np.array([i, j, k])
                for pa in perms:
                    path = [c, c + unit[pa[0]], c + unit[pa[0]] + unit[pa[1]], c + 1]
                    v = [vid(*q) for q in path]
                    x = X[v]
                    vol = np.linalg.det(np.stack([x[1] - x[0], x[2] - x[0], x[3] - x[0]]))
                    if vol < 0:
                        v[2], v[3] = v[3], v[2]
                    tets.append(v)
    ne = len(tets)
    nverts = nv1 ** 3
    edge_id, face_id = {}, {}
    for v in tets:
        for a, b in TET_EDGES:
            key = tuple(sorted((v[a], v[b])))
            if key not in edge_id:
                edge_id[key] = nverts + len(edge_id)
    for v in tets:
        for f in TET_FACES:
            key = tuple(sorted(v[q] for q in f))
            if key not in face_id:
                face_id[key] = nverts + len(edge_id) + len(face_id)
    nnodes = nverts + len(edge_id) + len(face_id)
    if orders is None:
        orders = np.full(ne, p, dtype=np.int32)
    orders = np.asarray(orders, dtype=np.int32)
    emin, fmin = {}, {}
    for e, v in enumerate(tets):
        for a, b in TET_EDGES:
            key = tuple(sorted((v[a], v[b])))
            emin[key] = min(emin.get(key, 99), int(orders[e]))
        for f in TET_FACES:
            key = tuple(sorted(v[q] for q in f))
            fmin[key] = min(fmin.get(key, 99), int(orders[e]))
    nodes = np.zeros((ne, 26), dtype=np.int32)
    bcflag = np.zeros((ne, 26), dtype=np.int32)
    xvert = np.zeros((ne, 8, 3))
    norder = np.zeros((ne, 19), dtype=np.int32)
    nori_e = np.zeros((ne, 12), dtype=np.int32)
    nori_f = np.zeros((ne, 6), dtype=np.int32)
    for e, v in enumerate(tets):
        xvert[e, :4] = X[v]
        for q in range(4):
            nodes[e, q] = v[q]
            bcflag[e, q] = int(_on_boundary(coords[[v[q]]], n))
        for q, (a, b) in enumerate(TET_EDGES):
            key = tuple(sorted((v[a], v[b])))
            nodes[e, 4 + q] = edge_id[key]
            nori_e[e, q] = 0 if v[a] < v[b] else 1
            norder[e, q] = emin[key]
            bcflag[e, 4 + q] = int(_on_boundary(coords[list(key)], n))
        for q, f in enumerate(TET_FACES):
            loc = [v[r] for r in f]
            key = tuple(sorted(loc))
            nodes[e, 10 + q] = face_id[key]
            nori_f[e, q] = tri_orientation(loc, key)
            norder[e, 6 + q] = fmin[key]
            bcflag[e, 10 + q] = int(_on_boundary(coords[list(key)], n))
        norder[e, 10] = orders[e]
    if not dirichlet:
        bcflag[:] = 0
    return dict(
        nelem=ne, n=n, h=h, p=p, nnodes=nnodes, nverts=nverts,
        etype=np.full(ne, TET, dtype=np.int32), norder=norder, nori_edge=nori_e,
        nori_face=nori_f, nodes=nodes, bcflag=bcflag, xvert=xvert,
        kappa=_kappa(rng, ne, kappa_logrange), vertex_xyz=X, orders=orders,
    )


def hp_tet(n, seed=2024, perturb=0.0, kappa_logrange=(-1, 1), pmax=6, dirichlet=True):
    """Kuhn tetrahedral mesh with per-element orders drawn in 1..pmax from a
    seeded geometric distribution whose mean grows away from the corner
    (0,0,0), edge and face orders by the minimum rule."""
    base = structured_tet(n, 1, seed=seed)
    rng = np.random.default_rng(seed + 1)
    cen = base["xvert"][:, :4].mean(axis=1)
    r = np.linalg.norm(cen, axis=1) / np.sqrt(3.0)
    mean = 1.0 + (pmax - 1) * r
    orders = np.minimum(rng.geometric(1.0 / np.maximum(mean, 1.0)), pmax).astype(np.int32)
    return structured_tet(n, None, perturb=perturb, kappa_logrange=kappa_logrange, seed=seed,
                          dirichlet=dirichlet, orders=orders)


PRISM = 2
# local topology in each element's own frame (shape_1/BlendProject.F90):
#   edges: (from, to) in the local direction, and the element axis of the edge
#   faces: triangles (w0, w1, w2) in OrientTri order; quads (w0, w1, w2, w3)
#          with S along w0->w1 and T along w0->w3, and the element axes of S, T
# Hexa axes are x/y/z (orders px, py, pz); prism axes are 0 = horizontal
# (ph), 2 = vertical (pz); tet orders have one axis.
_HEXA_EDGES = [((0, 1), 0), ((1, 2), 1), ((3, 2), 0), ((0, 3), 1), ((4, 5), 0), ((5, 6), 1),
               ((7, 6), 0), ((4, 7), 1), ((0, 4), 2), ((1, 5), 2), ((2, 6), 2), ((3, 7), 2)]
_HEXA_FACES = [((0, 1, 2, 3), (0, 1)), ((4, 5, 6, 7), (0, 1)), ((0, 1, 5, 4), (0, 2)),
               ((1, 2, 6, 5), (1, 2)), ((3, 2, 6, 7), (0, 2)), ((0, 3, 7, 4), (1, 2))]
_PRISM_EDGES = [((0, 1), 0), ((1, 2), 0), ((0, 2), 0), ((3, 4), 0), ((4, 5), 0), ((3, 5), 0),
                ((0, 3), 2), ((1, 4), 2), ((2, 5), 2)]
_PRISM_FACES = [((0, 1, 2), (0, 0)), ((3, 4, 5), (0, 0)), ((0, 1, 4, 3), (0, 2)),
                ((1, 2, 5, 4), (0, 2)), ((0, 2, 5, 3), (0, 2))]
_TET_EDGES = [(e, 0) for e in TET_EDGES]
_TET_FACES = [(f, (0, 0)) for f in TET_FACES]
_TOPO = {HEXA: (8, _HEXA_EDGES, _HEXA_FACES), PRISM: (6, _PRISM_EDGES, _PRISM_FACES),
         TET: (4, _TET_EDGES, _TET_FACES)}

# OrientQuad (shape_1/Orient.F90:39-116): OrPa(1:2)-1, OrGS(0:1), OrGT(0:1)
ORIENT_QUAD = [(0, 1, 0, 1, 0, 1), (1, 0, 0, 1, 1, 0), (0, 1, 1, 0, 1, 0), (1, 0, 1, 0, 0, 1),
               (1, 0, 0, 1, 0, 1), (0, 1, 1, 0, 0, 1), (1, 0, 1, 0, 1, 0), (0, 1, 0, 1, 1, 0)]
_QUAD_ST = [(0, 0), (1, 0), (1, 1), (0, 1)]


def quad_orientation(local, glob):
    """Orientation code o under which the element's face functions use the
    face node's frame: with (s, t) the element's face coordinates, the
    OrientQuad map of o sends every local vertex to the global (S, T)
    coordinates of the same vertex."""
    for o, (pa1, pa2, _, gs1, _, gt1) in enumerate(ORIENT_QUAD):
        ok = True
        for k, w in enumerate(local):
            st = _QUAD_ST[k]
            S = st[pa1] if gs1 == 1 else 1 - st[pa1]
            T = st[pa2] if gt1 == 1 else 1 - st[pa2]
            if glob[_QUAD_ST.index((S, T))] != w:
                ok = False
                break
        if ok:
            return o
    raise ValueError("quad face vertices do not match")


def build_mesh(etypes, verts, X, grid, n, orders, kappa_logrange=None, seed=12345,
               dirichlet=True):
    """Conforming mesh from elements given by type and local vertex list.

    X: vertex coordinates; grid: integer grid coordinates on [0, n]^3 (for
    the Dirichlet boundary); orders: per element (px, py, pz) for a hexa,
    (ph, pz) for a prism, (p,) for a tet.  Edge nodes run from the lower to
    the higher vertex id, triangle faces list their vertices in increasing
    id, quad faces take the frame of the first element that reaches them;
    each element's NoriE / NoriF follow.  Edge and face orders follow the
    minimum rule of the element orders along each global direction
    (adapt/enforce_min_rule.F90); a face's (h, v) is in its own frame.
    """
    rng = np.random.default_rng(seed)
    ne = len(etypes)
    nverts = len(X)
    edge_id, face_id, face_frame = {}, {}, {}
    emin, fmin = {}, {}
    enode = [[] for _ in range(ne)]
    fnode = [[] for _ in range(ne)]
    nori_e = np.zeros((ne, 12), np.int32)
    nori_f = np.zeros((ne, 6), np.int32)
    ford = [[] for _ in range(ne)]

    def axis_order(t, o, ax):
        if t == HEXA:
            return int(o[ax])
        if t == PRISM:
            return int(o[0] if ax == 0 else o[1])
        return int(o[0])

    for e in range(ne):
        t, v, o = etypes[e], verts[e], orders[e]
        nv, edges, faces = _TOPO[t]
        for q, ((a, b), ax) in enumerate(edges):
            key = (min(v[a], v[b]), max(v[a], v[b]))
            if key not in edge_id:
                edge_id[key] = len(edge_id)
            enode[e].append(key)
            nori_e[e, q] = 0 if v[a] < v[b] else 1
            emin[key] = min(emin.get(key, 99), axis_order(t, o, ax))
        for q, (fv, (a1, a2)) in enumerate(faces):
            loc = tuple(v[r] for r in fv)
            key = tuple(sorted(loc))
            if key not in face_id:
                face_id[key] = len(face_id)
                face_frame[key] = key if len(loc) == 3 else loc
            fnode[e].append(key)
            if len(loc) == 3:
                nori_f[e, q] = tri_orientation(loc, face_frame[key])
                h = (axis_order(t, o, a1), 0)
            else:
                oq = quad_orientation(loc, face_frame[key])
                nori_f[e, q] = oq
                ps, pt = axis_order(t, o, a1), axis_order(t, o, a2)
                h = (pt, ps) if ORIENT_QUAD[oq][0] == 1 else (ps, pt)
            cur = fmin.get(key, (99, 99))
            fmin[key] = (min(cur[0], h[0]), min(cur[1], h[1]))
    nedges = len(edge_id)
    nnodes = nverts + nedges + len(face_id)
    nodes = np.full((ne, 26), 0, np.int32)
    bcflag = np.zeros((ne, 26), np.int32)
    xvert = np.zeros((ne, 8, 3))
    norder = np.zeros((ne, 19), np.int32)
    grid = np.asarray(grid)
    for e in range(ne):
        t, v, o = etypes[e], verts[e], orders[e]
        nv, edges, faces = _TOPO[t]
        xvert[e, :nv] = X[list(v)]
        k = 0
        for q in range(nv):
            nodes[e, k] = v[q]
            bcflag[e, k] = int(_on_boundary(grid[[v[q]]], n))
            k += 1
        for q, key in enumerate(enode[e]):
            nodes[e, k] = nverts + edge_id[key]
            bcflag[e, k] = int(_on_boundary(grid[list(key)], n))
            norder[e, q] = emin[key]
            k += 1
        for q, key in enumerate(fnode[e]):
            nodes[e, k] = nverts + nedges + face_id[key]
            bcflag[e, k] = int(_on_boundary(grid[list(key)], n))
            h, vv = fmin[key]
            norder[e, len(edges) + q] = h if len(key) == 3 else 10 * h + vv
            k += 1
        mid = len(edges) + len(faces)
        if t == HEXA:
            norder[e, mid] = 100 * o[0] + 10 * o[1] + o[2]
        elif t == PRISM:
            norder[e, mid] = 10 * o[0] + o[1]
        else:
            norder[e, mid] = o[0]
    if not dirichlet:
        bcflag[:] = 0
    return dict(
        nelem=ne, n=n, nnodes=nnodes, nverts=nverts, etype=np.asarray(etypes, np.int32),
        norder=norder, nori_edge=nori_e, nori_face=nori_f, nodes=nodes, bcflag=bcflag,
        xvert=xvert, kappa=_kappa(rng, ne, kappa_logrange), vertex_xyz=X,
        orders=[tuple(int(x) for x in o) for o in orders],
    )


def _grid(n, perturb, rng):
    nv1 = n + 1
    idx = np.arange(nv1)
    I, J, K = np.meshgrid(idx, idx, idx, indexing="ij")
    coords = np.stack([I.ravel(order="F"), J.ravel(order="F"), K.ravel(order="F")], axis=1)
    X = coords.astype(np.float64) / n
    if perturb > 0.0:
        interior = np.all((coords > 0) & (coords < n), axis=1)
        d = rng.uniform(-perturb / n, perturb / n, size=X.shape)
        X[interior] += d[interior]
    return coords, X


def _signed_volume(x, t):
    # a positive Jacobian at the reference origin for the type's first corner
    if t == TET:
        return np.linalg.det(np.stack([x[1] - x[0], x[2] - x[0], x[3] - x[0]]))
    return np.linalg.det(np.stack([x[1] - x[0], x[2] - x[0], x[3] - x[0]]))


def _prism_cells(vid, c, axis):
    """The two prisms of the unit cell at c extruded along `axis`, their
    cross-section squares split along the diagonal through the cell's low
    corner (matching the Kuhn split of the neighbouring tetrahedra)."""
    # (u, w, axis) right-handed, so every prism has a positive Jacobian
    u, w = {0: (1, 2), 1: (2, 0), 2: (0, 1)}[axis]
    e = np.eye(3, dtype=int)
    p00, p10, p11, p01 = c, c + e[u], c + e[u] + e[w], c + e[w]
    out = []
    for tri in ((p00, p10, p11), (p00, p11, p01)):
        bot = [vid(*q) for q in tri]
        top = [vid(*(q + e[axis])) for q in tri]
        out.append(bot + top)
    return out


def _hp_order(rng, centre, pmax, k):
    r = np.linalg.norm(centre) / np.sqrt(3.0)
    mean = 1.0 + (pmax - 1) * r
    return tuple(int(min(x, pmax)) for x in rng.geometric(1.0 / max(mean, 1.0), size=k))


def structured_prism(n, ph, pz, perturb=0.0, kappa_logrange=None, seed=12345, dirichlet=True):
    """n^3 cells of [0,1]^3, each split into two prisms extruded along z."""
    rng = np.random.default_rng(seed)
    coords, X = _grid(n, perturb, rng)
    nv1 = n + 1
    vid = lambda i, j, k: int(i + nv1 * (j + nv1 * k))  # noqa: E731
    verts = []
    for k in range(n):
        for j in range(n):
            for i in range(n):
                verts += _prism_cells(vid, np.array([i, j, k]), 2)
    et = [PRISM] * len(verts)
    return build_mesh(et, verts, X, coords, n, [(ph, pz)] * len(verts), kappa_logrange, seed,
                      dirichlet)


def mixed_mesh(n, a=0.875, b=0.875, p=None, pmax=6, perturb=0.0, kappa_logrange=(-1, 1),
               seed=2024, dirichlet=True, cy=None):
    """Mixed hexa / prism / tet mesh of [0,1]^3 on an n^3 grid of cells:

      x < a, z < b : hexahedra
      x > a, z < b : prisms extruded along z
      x > a, z > b : tetrahedra (Kuhn split of each cell)
      x < a, z > b : prisms extruded along x

    With cy given the tetrahedra fill only the corner block x > a, y > cy,
    z > b: prisms extruded along z below it, along x beside it in x and
    along y beside it in y (each column reaching the boundary), hexahedra
    everywhere else.

    Every interface is conforming: hexa faces meet prism quads, prism
    triangles meet tetrahedron faces split along the same diagonals.  With
    p=None the orders are drawn per element in 1..pmax from a seeded
    geometric distribution whose mean falls toward (0,0,0) -- (px,py,pz) for
    a hexa, (ph,pz) for a prism, p for a tet -- and edges/faces take the
    minimum rule; otherwise every order is p.
    """
    rng = np.random.default_rng(seed)
    coords, X = _grid(n, perturb, rng)
    nv1 = n + 1
    vid = lambda i, j, k: int(i + nv1 * (j + nv1 * k))  # noqa: E731
    ia, kb = int(round(a * n)), int(round(b * n))
    jc = 0 if cy is None else int(round(cy * n))
    et, verts, orders = [], [], []
    e3 = np.eye(3, dtype=int)
    perms = [(0, 1, 2), (0, 2, 1), (1, 0, 2), (1, 2, 0), (2, 0, 1), (2, 1, 0)]
    for k in range(n):
        for j in range(n):
            for i in range(n):
                c = np.array([i, j, k])
                centre = (c + 0.5) / n
                # inside the tetrahedron block along x, y, z: all three ->
                # tetrahedra, two -> prisms extruded along the third axis,
                # fewer -> hexahedra
                inside = (i >= ia, j >= jc, k >= kb)
                cnt = sum(inside)
                if cnt <= 1:
                    v = [vid(*(c + d)) for d in _VOFF]
                    et.append(HEXA); verts.append(v)
                    orders.append((p, p, p) if p else _hp_order(rng, centre, pmax, 3))
                elif cnt == 2:
                    for v in _prism_cells(vid, c, inside.index(False)):
                        et.append(PRISM); verts.append(v)
                        orders.append((p, p) if p else _hp_order(rng, centre, pmax, 2))
                else:
                    for pa in perms:
                        path = [c, c + e3[pa[0]], c + e3[pa[0]] + e3[pa[1]], c + 1]
                        v = [vid(*q) for q in path]
                        if _signed_volume(X[v], TET) < 0:
                            v[2], v[3] = v[3], v[2]
                        et.append(TET); verts.append(v)
                        orders.append((p,) if p else _hp_order(rng, centre, pmax, 1))
    return build_mesh(et, verts, X, coords, n, orders, kappa_logrange, seed, dirichlet)


def dpg_boundary_flags(mesh, imp_planes=(), tol=1e-12):
    """Node flags of the ultraweak DPG Maxwell pass on a hexa mesh of the unit
    cube: bit 0 (E trace known) on every edge and face node of a perfect
    conductor wall, bit 2 on the face nodes of impedance walls (ibc = 2).
    imp_planes: (axis, side) walls with the impedance condition; the other
    walls are perfect conductors.  An edge shared by both kinds of wall is a
    conductor edge.  Returns (n_elem, 26) int32."""
    ne = mesh["nelem"]
    out = np.zeros((ne, 26), np.int32)
    edges = [e for e, _ in _HEXA_EDGES]
    faces = [f for f, _ in _HEXA_FACES]

    def planes(x):
        return [(a, s) for a in range(3) for s in (0, 1) if abs(x[a] - s) < tol]

    for e in range(ne):
        xv = np.asarray(mesh["xvert"][e])[:8]
        pts = [xv[list(q)].mean(0) for q in edges] + [xv[list(q)].mean(0) for q in faces]
        for k, x in enumerate(pts):
            pl = planes(x)
            if any(q not in imp_planes for q in pl):
                out[e, 8 + k] |= 1
            elif pl and k >= 12:
                out[e, 8 + k] |= 4
    return out
