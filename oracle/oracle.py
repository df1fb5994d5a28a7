"""ctypes binding of the CPU oracle (liborc.so).

TEST INFRASTRUCTURE ONLY: imported by tests/, by ``__graft_entry__.smoke()``
and by the ``cpu_baseline`` / ``--impl reference`` legs of ``bench.py``.  The
product library never loads it.  The C sources restate Oden-EAG/hp3d routines
(citations in ``hp3d_oracle.h``).
"""
from __future__ import annotations

import ctypes
import os
import subprocess

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_LIB = os.path.join(_HERE, "liborc.so")
_lib = None

HEXA, PRISM, TET = 1, 2, 3

_i32p = ctypes.POINTER(ctypes.c_int32)
_i64p = ctypes.POINTER(ctypes.c_int64)
_f64p = ctypes.POINTER(ctypes.c_double)


def build(force: bool = False) -> str:
    """Compile liborc.so with the Makefile beside this file."""
    srcs = [os.path.join(_HERE, f) for f in ("hp3d_oracle.c", "hp3d_oracle_dpg.c",
                                             "hp3d_oracle.h", "hp3d_oracle_int.h")]
    newest = max(os.path.getmtime(f) for f in srcs)
    if force or not os.path.exists(_LIB) or os.path.getmtime(_LIB) < newest:
        subprocess.run(["make", "-C", _HERE, "-B", "liborc.so"], check=True,
                       stdout=subprocess.DEVNULL)
    return _LIB


def lib():
    global _lib
    if _lib is None:
        build()
        L = ctypes.CDLL(_LIB)
        L.orc_gauss1d.argtypes = [ctypes.c_int, _f64p, _f64p]
        L.orc_set_blas.argtypes = [ctypes.c_void_p] * 4
        L.orc_set_blas.restype = None
        L.orc_set_3D_int_hexa.argtypes = [_i32p, _i32p, ctypes.c_int, _f64p, _f64p]
        L.orc_set_3D_int_tet.argtypes = [_i32p, ctypes.c_int, _f64p, _f64p]
        L.orc_nrdofH_hexa.argtypes = [_i32p]
        L.orc_nrdofH_tet.argtypes = [_i32p]
        L.orc_nrdofH_prism.argtypes = [_i32p]
        L.orc_set_3D_int_prism.argtypes = [_i32p, _i32p, ctypes.c_int, _f64p, _f64p]
        L.orc_nrdofH_bubble.argtypes = [ctypes.c_int, _i32p]
        for f in (L.orc_shape3DH_hexa, L.orc_shape3DH_tet, L.orc_shape3DH_prism):
            f.argtypes = [_f64p, _i32p, _i32p, _i32p, _f64p, _f64p]
        L.orc_geom.argtypes = [_f64p, _f64p, _f64p]
        L.orc_getf.argtypes = [ctypes.c_int, _f64p]
        L.orc_getf.restype = ctypes.c_double
        L.orc_exact.argtypes = [ctypes.c_int, _f64p, _f64p, _f64p]
        L.orc_elem.argtypes = [ctypes.c_int, _i32p, _i32p, _i32p, _f64p, ctypes.c_double,
                               ctypes.c_int, ctypes.c_int, ctypes.c_int, _f64p, ctypes.c_int,
                               _f64p]
        L.orc_stc_fwd.argtypes = [ctypes.c_int, ctypes.c_int, _f64p, ctypes.c_int, _f64p,
                                  ctypes.c_int, _f64p, _f64p, _f64p, _f64p]
        L.orc_stc_bwd.argtypes = [ctypes.c_int, ctypes.c_int, _f64p, _f64p, _f64p, _f64p]
        L.orc_node_ndof.argtypes = [ctypes.c_int, _i32p, _i32p]
        L.orc_celem_compress.argtypes = [ctypes.c_int, _i32p, _i32p, _f64p, _f64p, _f64p,
                                         _i32p, _f64p, _f64p, _i32p]
        L.orc_index_maps.argtypes = [ctypes.c_int, ctypes.c_int, _i32p, _i32p, _i32p,
                                     ctypes.c_int, _i32p, _i32p, _i64p, _i64p]
        L.orc_index_maps.restype = ctypes.c_int64
        L.orc_element_pass.argtypes = [ctypes.c_int, _i32p, _i32p, _i32p, _i32p, _i32p,
                                       _f64p, _f64p, ctypes.c_int, ctypes.c_int,
                                       ctypes.c_int, ctypes.c_int, _i64p, _i64p, _i64p,
                                       _i64p, _f64p, _f64p, _f64p, _f64p]
        L.orc_celem_compress_nodes.argtypes = [ctypes.c_int, _i32p, _i32p, _f64p, _f64p, _f64p,
                                               _i32p, _f64p, _f64p, _i32p]
        L.orc_constrain.argtypes = [ctypes.c_int, _f64p, _f64p, ctypes.c_int, _i32p, _i32p,
                                    _f64p, ctypes.c_int, _f64p, _f64p]
        L.orc_dirichlet_hexa.argtypes = [_i32p, _i32p, _i32p, _f64p, _i32p, ctypes.c_int, _f64p]
        L.orc_gdof_hexa.argtypes = [_i32p, _i32p, _i32p, _f64p, ctypes.c_int, GMAP_FN,
                                    ctypes.c_void_p, ctypes.c_int, _f64p]
        L.orc_nrdofE_hexa.argtypes = [_i32p]
        L.orc_shape3DE_hexa.argtypes = [_f64p, _i32p, _i32p, _i32p, _f64p, _f64p]
        L.orc_shape3DQ_hexa.argtypes = [_f64p, _i32p, _f64p]
        L.orc_shape3EE_hexa.argtypes = [_f64p, ctypes.c_int, _f64p, _f64p]
        L.orc_set_2D_int_quad.argtypes = [_i32p, ctypes.c_int, ctypes.c_int, ctypes.c_int,
                                          _f64p, _f64p]
        L.orc_maxw_exact.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_double,
                                     ctypes.c_double, ctypes.c_double, ctypes.c_double, _f64p,
                                     _f64p, _f64p, _f64p]
        L.orc_maxw_exact.restype = None
        L.orc_dpg_sizes.argtypes = [_i32p, ctypes.c_int, _i32p]
        L.orc_dpg_maxwell_elem.argtypes = [_i32p, _i32p, _i32p, _f64p, ctypes.c_double,
                                           ctypes.c_double, ctypes.c_int32,
                                           ctypes.POINTER(MaxwParams), _f64p, _f64p]
        L.orc_stc_fwd_z.argtypes = [ctypes.c_int, ctypes.c_int, _f64p, ctypes.c_int, _f64p,
                                    _f64p, _f64p, _f64p, _f64p]
        L.orc_node_nshapeE.argtypes = [_i32p, _i32p]
        L.orc_celem_compress_z.argtypes = [_i32p, _i32p, _f64p, _f64p, _f64p, _i32p, _f64p,
                                           _f64p, _i32p]
        L.orc_dpg_pass.argtypes = [ctypes.c_int, _i32p, _i32p, _i32p, _i32p, _i32p, _f64p,
                                   _f64p, ctypes.POINTER(MaxwParams), ctypes.c_int, _i64p,
                                   _i64p, _i64p, _i64p, _f64p, _f64p, _f64p, _f64p]
        _lib = L
    return _lib


class MaxwParams(ctypes.Structure):
    """orc_maxw_params: OMEGA, MU, EPSILON, GAMMA, ALPHA_NORM, IBCFLAG,
    NORD_ADD, ISOL, ICOMP_EXACT (defaults of set_environment.F90)."""
    _fields_ = [("omega", ctypes.c_double), ("mu", ctypes.c_double),
                ("epsilon", ctypes.c_double), ("gamma", ctypes.c_double),
                ("alpha", ctypes.c_double), ("ibcflag", ctypes.c_int32),
                ("nord_add", ctypes.c_int32), ("isol", ctypes.c_int32),
                ("icomp", ctypes.c_int32)]


def maxw_params(omega=2 * np.pi, mu=1.0, epsilon=1.0, gamma=1.0, alpha=1.0, ibcflag=0,
                nord_add=1, isol=1, icomp=1):
    return MaxwParams(omega, mu, epsilon, gamma, alpha, ibcflag, nord_add, isol, icomp)


def _p(a, t):
    if a is None:
        return None
    return a.ctypes.data_as(t)


def _i32(a):
    return np.ascontiguousarray(a, dtype=np.int32)


def _f64(a):
    return np.ascontiguousarray(a, dtype=np.float64)


def _capsule_pointer(capsule):
    get_name = ctypes.pythonapi.PyCapsule_GetName
    get_name.restype = ctypes.c_char_p
    get_name.argtypes = [ctypes.py_object]
    get_ptr = ctypes.pythonapi.PyCapsule_GetPointer
    get_ptr.restype = ctypes.c_void_p
    get_ptr.argtypes = [ctypes.py_object, ctypes.c_char_p]
    return get_ptr(capsule, get_name(capsule))


def use_blas(on=True):
    """Route the oracle's DSYRK (elem_opt.F90:131) and DGETRF / DGETRS / DGEMM
    (stc.F90:462-507) through the optimised BLAS / LAPACK that SciPy bundles
    (its Cython-level routines, Fortran calling convention), as the reference
    does through its BLAS.  Returns a one-line description of the library, or
    None when SciPy is missing (the oracle's own loops stay in use).  Set
    OPENBLAS_NUM_THREADS=1 before SciPy loads when the oracle runs its own
    OpenMP threads."""
    if not on:
        lib().orc_set_blas(None, None, None, None)
        return None
    try:
        import scipy
        from scipy.linalg import cython_blas, cython_lapack
    except ImportError:
        return None
    b, la = cython_blas.__pyx_capi__, cython_lapack.__pyx_capi__
    lib().orc_set_blas(_capsule_pointer(b["dsyrk"]), _capsule_pointer(la["dgetrf"]),
                       _capsule_pointer(la["dgetrs"]), _capsule_pointer(b["dgemm"]))
    desc = f"scipy {scipy.__version__} BLAS/LAPACK"
    try:
        cfg = scipy.show_config(mode="dicts")
        bl = cfg.get("Build Dependencies", {}).get("blas", {})
        desc += f" ({bl.get('name', '?')} {bl.get('version', '')})".rstrip()
    except Exception:
        pass
    return desc


def gauss1d(n):
    x = np.zeros(n); w = np.zeros(n)
    assert lib().orc_gauss1d(n, _p(x, _f64p), _p(w, _f64p)) == 0
    return x, w


def quad_hexa(norder, nori_face=None, integration=0):
    norder = _i32(norder)
    nori_face = _i32(np.zeros(6) if nori_face is None else nori_face)
    xi = np.zeros((400, 3)); w = np.zeros(400)
    n = lib().orc_set_3D_int_hexa(_p(norder, _i32p), _p(nori_face, _i32p), integration,
                                  _p(xi, _f64p), _p(w, _f64p))
    return xi[:n].copy(), w[:n].copy()


def nrdofH(etype, norder):
    norder = _i32(norder)
    if etype == HEXA:
        return lib().orc_nrdofH_hexa(_p(norder, _i32p))
    if etype == PRISM:
        return lib().orc_nrdofH_prism(_p(norder, _i32p))
    return lib().orc_nrdofH_tet(_p(norder, _i32p))


def nrdof_bubble(etype, norder):
    return lib().orc_nrdofH_bubble(etype, _p(_i32(norder), _i32p))


def shape_hexa(xi, norder, nori_edge=None, nori_face=None):
    xi = _f64(xi)
    norder = _i32(norder)
    ne = _i32(np.zeros(12) if nori_edge is None else nori_edge)
    nf = _i32(np.zeros(6) if nori_face is None else nori_face)
    shap = np.zeros(343); grad = np.zeros((343, 3))
    n = lib().orc_shape3DH_hexa(_p(xi, _f64p), _p(norder, _i32p), _p(ne, _i32p),
                                _p(nf, _i32p), _p(shap, _f64p), _p(grad, _f64p))
    return shap[:n].copy(), grad[:n].copy()


def shape_tet(xi, norder, nori_edge=None, nori_face=None):
    xi = _f64(xi)
    norder = _i32(norder)
    ne = _i32(np.zeros(12) if nori_edge is None else nori_edge)
    nf = _i32(np.zeros(6) if nori_face is None else nori_face)
    shap = np.zeros(343); grad = np.zeros((343, 3))
    n = lib().orc_shape3DH_tet(_p(xi, _f64p), _p(norder, _i32p), _p(ne, _i32p),
                               _p(nf, _i32p), _p(shap, _f64p), _p(grad, _f64p))
    return shap[:n].copy(), grad[:n].copy()


def shape_prism(xi, norder, nori_edge=None, nori_face=None):
    xi = _f64(xi)
    norder = _i32(norder)
    ne = _i32(np.zeros(12) if nori_edge is None else nori_edge)
    nf = _i32(np.zeros(6) if nori_face is None else nori_face)
    shap = np.zeros(343); grad = np.zeros((343, 3))
    n = lib().orc_shape3DH_prism(_p(xi, _f64p), _p(norder, _i32p), _p(ne, _i32p),
                                 _p(nf, _i32p), _p(shap, _f64p), _p(grad, _f64p))
    return shap[:n].copy(), grad[:n].copy()


def quad_prism(norder, nori_face=None, integration=0):
    nf = _i32(np.zeros(6) if nori_face is None else nori_face)
    xi = np.zeros(3 * 400); w = np.zeros(400)
    n = lib().orc_set_3D_int_prism(_p(_i32(norder), _i32p), _p(nf, _i32p), integration,
                                   _p(xi, _f64p), _p(w, _f64p))
    return xi[: 3 * n].reshape(n, 3).copy(), w[:n].copy()


def shape(etype, xi, norder, nori_edge=None, nori_face=None):
    if etype == TET:
        return shape_tet(xi, norder, nori_edge, nori_face)
    if etype == PRISM:
        return shape_prism(xi, norder, nori_edge, nori_face)
    return shape_hexa(xi, norder, nori_edge, nori_face)


def quad_tet(norder, integration=0):
    xi = np.zeros(3 * 400); w = np.zeros(400)
    n = lib().orc_set_3D_int_tet(_p(_i32(norder), _i32p), integration, _p(xi, _f64p),
                                 _p(w, _f64p))
    return xi[: 3 * n].reshape(n, 3).copy(), w[:n].copy()


def getf(isol, x):
    return lib().orc_getf(isol, _p(_f64(x), _f64p))


def exact(isol, x):
    u = np.zeros(1); g = np.zeros(3)
    lib().orc_exact(isol, _p(_f64(x), _f64p), _p(u, _f64p), _p(g, _f64p))
    return u[0], g


def elem(etype, norder, nori_edge, nori_face, xnod, kappa=1.0, isol=10, integration=0,
         variant=0):
    """Element stiffness (n x n) and load (n); xnod is (nrdofH, 3) or the
    vertex coordinates (nvert, 3) padded with zeros."""
    norder = _i32(norder)
    n = nrdofH(etype, norder)
    xn = np.zeros((n, 3))
    xv = np.asarray(xnod, dtype=np.float64)
    xn[: xv.shape[0]] = xv
    xn = _f64(xn)
    K = np.zeros((n, n), order="F"); b = np.zeros(n)
    rc = lib().orc_elem(etype, _p(norder, _i32p), _p(_i32(nori_edge), _i32p),
                        _p(_i32(nori_face), _i32p), _p(xn, _f64p), float(kappa), isol,
                        integration, variant, K.ctypes.data_as(_f64p), n, _p(b, _f64p))
    return K, b, rc


def stc_fwd(K, b, nb, method=0):
    n = K.shape[0]
    ni = n - nb
    Kf = np.asfortranarray(K, dtype=np.float64)
    aii = np.zeros((ni, ni), order="F"); bi = np.zeros(ni)
    asch = np.zeros((nb, ni), order="F"); bsch = np.zeros(nb)
    rc = lib().orc_stc_fwd(ni, nb, Kf.ctypes.data_as(_f64p), n, _p(_f64(b), _f64p), method,
                           aii.ctypes.data_as(_f64p), _p(bi, _f64p), asch.ctypes.data_as(_f64p),
                           _p(bsch, _f64p))
    return aii, bi, asch, bsch, rc


def stc_bwd(asch, bsch, xi):
    nb, ni = asch.shape
    a = np.asfortranarray(asch)
    xb = np.zeros(nb)
    lib().orc_stc_bwd(ni, nb, a.ctypes.data_as(_f64p), _p(_f64(bsch), _f64p),
                      _p(_f64(xi), _f64p), _p(xb, _f64p))
    return xb


def node_ndof(etype, norder):
    nd = np.zeros(32, dtype=np.int32)
    nn = lib().orc_node_ndof(etype, _p(_i32(norder), _i32p), _p(nd, _i32p))
    return nd[:nn].copy()


def celem_compress(etype, norder, bcflag, aii, bi, zdofd=None):
    ni = aii.shape[0]
    a = np.asfortranarray(aii, dtype=np.float64)
    bc = _i32(np.zeros(26) if bcflag is None else np.pad(np.asarray(bcflag), (0, 26 - len(bcflag))))
    nextract = np.zeros(max(ni, 1), dtype=np.int32)
    zb = np.zeros(max(ni, 1)); zs = np.zeros(max(ni * ni, 1)); ndofm = np.zeros(32, dtype=np.int32)
    zd = None if zdofd is None else _f64(zdofd)
    nc = lib().orc_celem_compress(etype, _p(_i32(norder), _i32p), _p(bc, _i32p),
                                  a.ctypes.data_as(_f64p), _p(_f64(bi), _f64p),
                                  _p(zd, _f64p), _p(nextract, _i32p), _p(zb, _f64p),
                                  _p(zs, _f64p), _p(ndofm, _i32p))
    return nextract[:nc].copy(), zb[:nc].copy(), zs[: nc * nc].reshape(nc, nc).copy(), ndofm


def index_maps(nnode, nodes, ndofm, nnodes_global):
    nodes = _i32(nodes); ndofm = _i32(ndofm); nnode = _i32(nnode)
    nelem, nmax = nodes.shape
    nfirst = np.zeros(nnodes_global, dtype=np.int32)
    lcon_off = np.zeros(nelem + 1, dtype=np.int64)
    elem_nnz = np.zeros(nelem + 1, dtype=np.int64)
    lcon = np.zeros(int(ndofm.sum()) + 1, dtype=np.int32)
    nrdof = lib().orc_index_maps(nelem, nmax, _p(nnode, _i32p), _p(nodes, _i32p),
                                 _p(ndofm, _i32p), nnodes_global, _p(nfirst, _i32p),
                                 _p(lcon, _i32p), _p(lcon_off, _i64p), _p(elem_nnz, _i64p))
    return int(nrdof), nfirst, lcon[: lcon_off[-1]].copy(), lcon_off, elem_nnz


def element_pass(mesh, isol=10, integration=0, stc_method=0, nthreads=0,
                 elements=None):
    """Run elem -> stc_fwd -> compression over (a subset of) a mesh.

    ``mesh`` is a dict as produced by ``hp3d_gb300.mesh``; ``elements`` an
    optional index array restricting the pass (used for bounded CPU samples).
    Returns dict of concatenated outputs with their offsets."""
    idx = np.arange(mesh["nelem"]) if elements is None else np.asarray(elements)
    ne = len(idx)
    et = _i32(mesh["etype"][idx]); no = _i32(mesh["norder"][idx])
    ned = _i32(mesh["nori_edge"][idx]); nfc = _i32(mesh["nori_face"][idx])
    bc = _i32(mesh["bcflag"][idx]); xv = _f64(mesh["xvert"][idx]); ka = _f64(mesh["kappa"][idx])
    nrdofc = np.zeros(ne, dtype=np.int64); nb = np.zeros(ne, dtype=np.int64)
    ni = np.zeros(ne, dtype=np.int64)
    for j in range(ne):
        nd = node_ndof(int(et[j]), no[j])
        nn = len(nd)
        act = nd * (1 - bc[j][:nn])
        nrdofc[j] = act.sum()
        nb[j] = nrdof_bubble(int(et[j]), no[j])
        ni[j] = nd.sum()
    elem_nnz = np.concatenate([[0], np.cumsum(nrdofc * nrdofc)]).astype(np.int64)
    lcon_off = np.concatenate([[0], np.cumsum(nrdofc)]).astype(np.int64)
    schur_off = np.concatenate([[0], np.cumsum(nb * ni)]).astype(np.int64)
    bub_off = np.concatenate([[0], np.cumsum(nb)]).astype(np.int64)
    zastif = np.zeros(max(int(elem_nnz[-1]), 1)); zbload = np.zeros(max(int(lcon_off[-1]), 1))
    aschur = np.zeros(max(int(schur_off[-1]), 1)); bschur = np.zeros(max(int(bub_off[-1]), 1))
    rc = lib().orc_element_pass(ne, _p(et, _i32p), _p(no, _i32p), _p(ned, _i32p), _p(nfc, _i32p),
                                _p(bc, _i32p), _p(xv, _f64p), _p(ka, _f64p), isol, integration,
                                stc_method, nthreads, _p(elem_nnz, _i64p), _p(lcon_off, _i64p),
                                _p(schur_off, _i64p), _p(bub_off, _i64p), _p(zastif, _f64p),
                                _p(zbload, _f64p), _p(aschur, _f64p), _p(bschur, _f64p))
    return dict(rc=rc, zastif=zastif, zbload=zbload, aschur=aschur, bschur=bschur,
                elem_nnz=elem_nnz, lcon_off=lcon_off, schur_off=schur_off, bub_off=bub_off,
                nrdofc=nrdofc, nb=nb, ni=ni)


# --------------------------------------------------------------------------
# ultraweak DPG Maxwell (hexahedra)
# --------------------------------------------------------------------------
def _z(a):
    return np.ascontiguousarray(a, dtype=np.complex128)


def shapeE_hexa(xi, norder, nori_edge=None, nori_face=None):
    ne = _i32(np.zeros(12) if nori_edge is None else nori_edge)
    nf = _i32(np.zeros(6) if nori_face is None else nori_face)
    s = np.zeros((800, 3)); c = np.zeros((800, 3))
    n = lib().orc_shape3DE_hexa(_p(_f64(xi), _f64p), _p(_i32(norder), _i32p), _p(ne, _i32p),
                                _p(nf, _i32p), _p(s, _f64p), _p(c, _f64p))
    return s[:n].copy(), c[:n].copy()


def shapeQ_hexa(xi, norder):
    q = np.zeros(512)
    n = lib().orc_shape3DQ_hexa(_p(_f64(xi), _f64p), _p(_i32(norder), _i32p), _p(q, _f64p))
    return q[:n].copy()


def shapeEE_hexa(xi, nordP):
    s = np.zeros((800, 3)); c = np.zeros((800, 3))
    n = lib().orc_shape3EE_hexa(_p(_f64(xi), _f64p), int(nordP), _p(s, _f64p), _p(c, _f64p))
    return s[:n].copy(), c[:n].copy()


def quad_face(norderf, nori=0, integration=1, maxp=7):
    t = np.zeros((100, 2)); w = np.zeros(100)
    n = lib().orc_set_2D_int_quad(_p(_i32(norderf), _i32p), int(nori), integration, maxp,
                                  _p(t, _f64p), _p(w, _f64p))
    return t[:n].copy(), w[:n].copy()


def maxw_exact(x, prm, eps=1.0 + 0j):
    E = np.zeros(6); H = np.zeros(6); J = np.zeros(6)
    lib().orc_maxw_exact(prm.isol, prm.icomp, prm.omega, prm.mu, prm.epsilon * eps.real,
                         prm.epsilon * eps.imag, _p(_f64(x), _f64p), _p(E, _f64p),
                         _p(H, _f64p), _p(J, _f64p))
    return E.view(np.complex128), H.view(np.complex128), J.view(np.complex128)


def dpg_sizes(norder, nord_add=1):
    sz = np.zeros(5, dtype=np.int32)
    lib().orc_dpg_sizes(_p(_i32(norder), _i32p), nord_add, _p(sz, _i32p))
    return dict(nEi=int(sz[0]), nQ=int(sz[1]), nEE=int(sz[2]), ntest=int(sz[3]),
                ntrial=int(sz[4]))


def dpg_elem(norder, nori_edge, nori_face, xvert, eps=1.0 + 0j, imp_mask=0, prm=None):
    """DPG element matrix (NrTrial x NrTrial, complex) and load."""
    prm = maxw_params() if prm is None else prm
    n = dpg_sizes(norder, prm.nord_add)["ntrial"]
    A = np.zeros((n, n), dtype=np.complex128, order="F"); b = np.zeros(n, dtype=np.complex128)
    xv = _f64(np.asarray(xvert)[:8])
    rc = lib().orc_dpg_maxwell_elem(_p(_i32(norder), _i32p), _p(_i32(nori_edge), _i32p),
                                    _p(_i32(nori_face), _i32p), _p(xv, _f64p), eps.real,
                                    eps.imag, int(imp_mask), ctypes.byref(prm),
                                    A.ctypes.data_as(_f64p), b.ctypes.data_as(_f64p))
    return A, b, rc


def stc_fwd_z(A, b, nb):
    n = A.shape[0]
    ni = n - nb
    Af = np.asfortranarray(A, dtype=np.complex128)
    aii = np.zeros((ni, ni), dtype=np.complex128, order="F"); bi = np.zeros(ni, np.complex128)
    asch = np.zeros((nb, ni), dtype=np.complex128, order="F"); bsch = np.zeros(nb, np.complex128)
    rc = lib().orc_stc_fwd_z(ni, nb, Af.ctypes.data_as(_f64p), n, _z(b).ctypes.data_as(_f64p),
                             aii.ctypes.data_as(_f64p), bi.ctypes.data_as(_f64p),
                             asch.ctypes.data_as(_f64p), bsch.ctypes.data_as(_f64p))
    return aii, bi, asch, bsch, rc


def node_nshapeE(norder):
    ns = np.zeros(26, dtype=np.int32)
    lib().orc_node_nshapeE(_p(_i32(norder), _i32p), _p(ns, _i32p))
    return ns


def celem_compress_z(norder, bcflag, aii, bi, zdofd=None):
    ni = aii.shape[0]
    a = np.asfortranarray(aii, dtype=np.complex128)
    bc = _i32(np.pad(np.asarray(bcflag), (0, 26 - len(bcflag))))
    nx = np.zeros(max(ni, 1), dtype=np.int32)
    zb = np.zeros(max(ni, 1), np.complex128); zs = np.zeros(max(ni * ni, 1), np.complex128)
    ndofm = np.zeros(26, dtype=np.int32)
    zd = None if zdofd is None else _z(zdofd)
    nc = lib().orc_celem_compress_z(_p(_i32(norder), _i32p), _p(bc, _i32p),
                                    a.ctypes.data_as(_f64p), _z(bi).ctypes.data_as(_f64p),
                                    None if zd is None else zd.ctypes.data_as(_f64p),
                                    _p(nx, _i32p), zb.ctypes.data_as(_f64p),
                                    zs.ctypes.data_as(_f64p), _p(ndofm, _i32p))
    return nx[:nc].copy(), zb[:nc].copy(), zs[: nc * nc].reshape(nc, nc).copy(), ndofm


def dpg_pass(mesh, eps, bcflag, imp_mask, prm, elements=None, nthreads=0):
    """elem_maxwell -> stc_fwd_herm -> compression over (a subset of) a hexa
    mesh with OpenMP; returns the oracle's return code and the outputs."""
    idx = np.arange(mesh["nelem"]) if elements is None else np.asarray(elements)
    ne = len(idx)
    no = _i32(mesh["norder"][idx]); ned = _i32(mesh["nori_edge"][idx])
    nfc = _i32(mesh["nori_face"][idx]); bc = _i32(np.asarray(bcflag)[idx])
    im = _i32(np.asarray(imp_mask)[idx]); xv = _f64(np.asarray(mesh["xvert"])[idx, :8])
    ep = _z(np.asarray(eps)[idx])
    nc = np.zeros(ne, np.int64); s = dpg_sizes(no[0], prm.nord_add)
    ni, nb = 2 * s["nEi"], 6 * s["nQ"]
    for j in range(ne):
        nsh = node_nshapeE(no[j])
        nc[j] = sum(int(nsh[i]) * (2 - bin(int(bc[j][i]) & 3).count("1")) for i in range(26))
    elem_nnz = np.concatenate([[0], np.cumsum(nc * nc)]).astype(np.int64)
    lcon_off = np.concatenate([[0], np.cumsum(nc)]).astype(np.int64)
    schur_off = (np.arange(ne + 1) * nb * ni).astype(np.int64)
    bub_off = (np.arange(ne + 1) * nb).astype(np.int64)
    zs = np.zeros(max(int(elem_nnz[-1]), 1), np.complex128)
    zb = np.zeros(max(int(lcon_off[-1]), 1), np.complex128)
    asch = np.zeros(max(int(schur_off[-1]), 1), np.complex128)
    bsch = np.zeros(max(int(bub_off[-1]), 1), np.complex128)
    rc = lib().orc_dpg_pass(ne, _p(no, _i32p), _p(ned, _i32p), _p(nfc, _i32p), _p(bc, _i32p),
                            _p(im, _i32p), _p(xv, _f64p), ep.ctypes.data_as(_f64p),
                            ctypes.byref(prm), nthreads, _p(elem_nnz, _i64p),
                            _p(lcon_off, _i64p), _p(schur_off, _i64p), _p(bub_off, _i64p),
                            zs.ctypes.data_as(_f64p), zb.ctypes.data_as(_f64p),
                            asch.ctypes.data_as(_f64p), bsch.ctypes.data_as(_f64p))
    return dict(rc=rc, zastif=zs, zbload=zb, aschur=asch, bschur=bsch, elem_nnz=elem_nnz,
                lcon_off=lcon_off)


def constrain(aii, bi, ck, cl, cv, nmod):
    """amod = C^T aii C, bmod = C^T bi (celem_systemI.F90:541-760)."""
    ni = aii.shape[0]
    a = np.asfortranarray(aii, dtype=np.float64)
    am = np.zeros((nmod, nmod), order="F"); bm = np.zeros(nmod)
    rc = lib().orc_constrain(ni, a.ctypes.data_as(_f64p), _p(_f64(bi), _f64p), len(ck),
                             _p(_i32(ck), _i32p), _p(_i32(cl), _i32p), _p(_f64(cv), _f64p), nmod,
                             am.ctypes.data_as(_f64p), _p(bm, _f64p))
    assert rc == 0, rc
    return am, bm


def celem_compress_nodes(nd, bcflag, amod, bmod, zdofd=None):
    """Compression over a node list (modified element nodes)."""
    n = amod.shape[0]
    a = np.asfortranarray(amod, dtype=np.float64)
    nx = np.zeros(max(n, 1), dtype=np.int32)
    zb = np.zeros(max(n, 1)); zs = np.zeros(max(n * n, 1)); ndofm = np.zeros(len(nd), np.int32)
    zd = None if zdofd is None else _f64(zdofd)
    nc = lib().orc_celem_compress_nodes(len(nd), _p(_i32(nd), _i32p), _p(_i32(bcflag), _i32p),
                                        a.ctypes.data_as(_f64p), _p(_f64(bmod), _f64p),
                                        _p(zd, _f64p), _p(nx, _i32p), _p(zb, _f64p),
                                        _p(zs, _f64p), _p(ndofm, _i32p))
    return nx[:nc].copy(), zb[:nc].copy(), zs[: nc * nc].reshape(nc, nc).copy(), ndofm


GMAP_FN = ctypes.CFUNCTYPE(None, ctypes.POINTER(ctypes.c_double), ctypes.POINTER(ctypes.c_double),
                           ctypes.POINTER(ctypes.c_double), ctypes.c_void_p)


def gdof_hexa(norder, nori_edge, nori_face, etav, gmap, integration=1, linear=False):
    """update_gdof restated for one hexahedron: its geometry dof (nrdofH x 3,
    element dof order) from the block map gmap(eta) -> (x (3,), dxdeta (3, 3))
    and the element's vertices etav (8 x 3) in block coordinates."""
    def cb(eta, x, dx, _user):
        e = np.array([eta[0], eta[1], eta[2]])
        xv, J = gmap(e)
        for i in range(3):
            x[i] = float(xv[i])
            for j in range(3):
                dx[3 * i + j] = float(J[i, j])
    fn = GMAP_FN(cb)
    L = lib()
    n = L.orc_nrdofH_hexa(_p(_i32(norder), _i32p))
    out = np.zeros(3 * max(n, 1))
    rc = L.orc_gdof_hexa(_p(_i32(norder), _i32p), _p(_i32(nori_edge), _i32p),
                         _p(_i32(nori_face), _i32p), _p(_f64(np.asarray(etav)[:8]), _f64p),
                         integration, fn, None, int(linear), _p(out, _f64p))
    assert rc == n, rc
    return out[: 3 * n].reshape(n, 3).copy()


def dirichlet_hexa(norder, nori_edge, nori_face, xvert, bcflag, isol):
    """update_Ddof restated for one hexahedron: Dirichlet values per interface
    dof (element order)."""
    zd = np.zeros(400)
    n = lib().orc_dirichlet_hexa(_p(_i32(norder), _i32p), _p(_i32(nori_edge), _i32p),
                                 _p(_i32(nori_face), _i32p), _p(_f64(np.asarray(xvert)[:8]), _f64p),
                                 _p(_i32(np.asarray(bcflag)[:26]), _i32p), isol, _p(zd, _f64p))
    assert n >= 0
    return zd[:n].copy()
