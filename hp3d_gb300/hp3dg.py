"""Python mirror of the C ABI (include/hp3dg.h) over ctypes.

This is the host-side interface a Python caller (tests, benchmark, the torch
autograd harness) uses; the Fortran host binds the same entry points through
ISO_C_BINDING.  Loading fails loudly when libhp3dg.so is
missing: there is no CPU fallback.  Loading the library also loads the
package's tuning table (tune/gb300.json, written by hp3d_gb300.autotune) unless
the environment variable HP3DG_TUNE_FILE names another.
"""
from __future__ import annotations

import ctypes
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIBPATH = os.path.join(HERE, "libhp3dg.so")

HEXA, PRISM, TET = 1, 2, 3
FP64, MIXED = 0, 1

ERRORS = {0: "OK", -1: "NEG_JACOBIAN", -2: "NOT_SPD", -3: "BAD_ORDER", -4: "ALLOC", -5: "CUDA",
          -6: "TIMEOUT", -7: "ARG", -8: "STATE", -9: "UNSUPPORTED"}


class HP3DGError(RuntimeError):
    def __init__(self, code, msg, bad=-1):
        super().__init__(f"hp3dg error {code} ({ERRORS.get(code, '?')}): {msg}"
                         + (f" [element {bad}]" if bad >= 0 else ""))
        self.code = code
        self.bad = bad


class Opts(ctypes.Structure):
    _fields_ = [("precision", ctypes.c_int32), ("integration", ctypes.c_int32),
                ("isol", ctypes.c_int32), ("keep_elem", ctypes.c_int32),
                ("timing", ctypes.c_int32), ("device", ctypes.c_int32),
                ("ozaki_radix", ctypes.c_int32), ("ozaki_digits", ctypes.c_int32),
                ("stc_method", ctypes.c_int32), ("launch_mode", ctypes.c_int32),
                ("schur_fp64", ctypes.c_int32), ("download_chunks", ctypes.c_int32),
                ("fault_inject", ctypes.c_int32), ("tune", ctypes.c_int32),
                ("reserved", ctypes.c_int32 * 2)]


DESC_DTYPE = np.dtype([("etype", np.int32), ("mdle", np.int32), ("norder", np.int32, 19),
                       ("nori_edge", np.int32, 12), ("nori_face", np.int32, 6),
                       ("nodes", np.int32, 26), ("bcflag", np.int32, 26)])

_lib = None
_vp = ctypes.c_void_p
_i32p = ctypes.POINTER(ctypes.c_int32)
_i64p = ctypes.POINTER(ctypes.c_int64)
_f64p = ctypes.POINTER(ctypes.c_double)
_f32p = ctypes.POINTER(ctypes.c_float)

EXPORTS = ["hp3dg_batch_begin", "hp3dg_set_stream", "hp3dg_batch_submit",
           "hp3dg_batch_submit_constrained", "hp3dg_dirichlet_dofs", "hp3dg_batch_set_geometry",
           "hp3dg_batch_run",
           "hp3dg_batch_sync", "hp3dg_batch_download", "hp3dg_get_elem", "hp3dg_get_condensed",
           "hp3dg_get_schur", "hp3dg_index_map", "hp3dg_backsub", "hp3dg_get_dofs",
           "hp3dg_element_error", "hp3dg_adjoint", "hp3dg_condense_noalloc", "hp3dg_mixed_contract", "hp3dg_output_sizes", "hp3dg_device_outputs",
           "hp3dg_phase_times", "hp3dg_mixed_config", "hp3dg_pass_stats", "hp3dg_last_bad_element",
           "hp3dg_tune_load", "hp3dg_tune_lookup", "hp3dg_bin_info", "hp3dg_gdof_points",
           "hp3dg_update_gdof",
           "hp3dg_dpg_begin", "hp3dg_dpg_submit", "hp3dg_dpg_run", "hp3dg_dpg_sync",
           "hp3dg_dpg_download", "hp3dg_dpg_sizes", "hp3dg_dpg_get_elem",
           "hp3dg_dpg_get_condensed", "hp3dg_dpg_get_schur", "hp3dg_dpg_index_map",
           "hp3dg_dpg_phase_times", "hp3dg_dpg_pass_stats", "hp3dg_dpg_last_bad_element", "hp3dg_dpg_end", "hp3dg_batch_end", "hp3dg_strerror"]


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(LIBPATH):
            raise RuntimeError(f"{LIBPATH} is missing: build it with hp3d_gb300.build.build()")
        L = ctypes.CDLL(LIBPATH)
        L.hp3dg_batch_begin.argtypes = [ctypes.POINTER(Opts), ctypes.POINTER(_vp)]
        L.hp3dg_set_stream.argtypes = [_vp, _vp]
        L.hp3dg_batch_submit.argtypes = [_vp, ctypes.c_int32, _vp, _f64p, _f64p, _f64p,
                                         ctypes.c_int32]
        L.hp3dg_batch_submit_constrained.argtypes = [_vp, ctypes.c_int32, _vp, _f64p, _f64p,
                                                     _f64p, ctypes.c_int32,
                                                     ctypes.POINTER(Constraints)]
        L.hp3dg_dirichlet_dofs.argtypes = [_vp, ctypes.c_int32, _f64p, _i64p]
        L.hp3dg_batch_set_geometry.argtypes = [_vp, _f64p]
        L.hp3dg_gdof_points.argtypes = [_vp, _f64p, _f64p, _i64p]
        L.hp3dg_update_gdof.argtypes = [_vp, _f64p, _f64p, _f64p, _i32p, _f64p, ctypes.c_int32]
        L.hp3dg_batch_run.argtypes = [_vp]
        L.hp3dg_batch_sync.argtypes = [_vp]
        L.hp3dg_batch_download.argtypes = [_vp]
        L.hp3dg_get_elem.argtypes = [_vp, ctypes.c_int32, _f64p, ctypes.c_int32, _f64p]
        L.hp3dg_get_condensed.argtypes = [_vp, ctypes.c_int32, _f64p, _f64p, _i32p]
        L.hp3dg_get_schur.argtypes = [_vp, ctypes.c_int32, _f64p, _f64p, _i32p, _i32p]
        L.hp3dg_index_map.argtypes = [_vp, _i32p, _i64p, _i64p, _i32p, _i64p]
        L.hp3dg_output_sizes.argtypes = [_vp, _i64p, _i64p, _i64p, _i64p]
        L.hp3dg_backsub.argtypes = [_vp, _f64p]
        L.hp3dg_get_dofs.argtypes = [_vp, ctypes.c_int32, _f64p, _i32p]
        L.hp3dg_element_error.argtypes = [_vp, ctypes.c_int32, _f64p, _f64p]
        L.hp3dg_adjoint.argtypes = [_vp, _f64p, _f64p, _f64p]
        L.hp3dg_device_outputs.argtypes = [_vp] + [ctypes.POINTER(_vp)] * 5
        L.hp3dg_phase_times.argtypes = [_vp, _f32p, ctypes.c_int32]
        L.hp3dg_mixed_config.argtypes = [_vp, _i32p, _i32p, _i32p]
        L.hp3dg_pass_stats.argtypes = [_vp, _i64p, _f64p]
        L.hp3dg_tune_load.argtypes = [ctypes.c_char_p, _i32p]
        L.hp3dg_tune_lookup.argtypes = [ctypes.c_int32] * 5 + [_i32p] * 3
        L.hp3dg_bin_info.argtypes = [_vp, _i32p, ctypes.c_int32, _i32p, _i32p]
        L.hp3dg_last_bad_element.argtypes = [_vp]
        L.hp3dg_last_bad_element.restype = ctypes.c_int32
        L.hp3dg_batch_end.argtypes = [_vp]
        L.hp3dg_batch_end.restype = None
        L.hp3dg_mixed_contract.argtypes = [ctypes.c_int32] * 3 + [_vp] * 3 + \
            [ctypes.c_int32] * 2 + [_vp]
        L.hp3dg_strerror.argtypes = [ctypes.c_int]
        L.hp3dg_strerror.restype = ctypes.c_char_p
        L.hp3dg_dpg_begin.argtypes = [ctypes.POINTER(DpgOpts), ctypes.POINTER(_vp)]
        L.hp3dg_dpg_submit.argtypes = [_vp, ctypes.c_int32, _vp, _f64p, _f64p, ctypes.c_int32]
        for f in (L.hp3dg_dpg_run, L.hp3dg_dpg_sync, L.hp3dg_dpg_download):
            f.argtypes = [_vp]
        L.hp3dg_dpg_sizes.argtypes = [_vp, _i32p, _i32p, _i32p]
        L.hp3dg_dpg_get_elem.argtypes = [_vp, ctypes.c_int32, _f64p, ctypes.c_int32, _f64p]
        L.hp3dg_dpg_get_condensed.argtypes = [_vp, ctypes.c_int32, _f64p, _f64p, _i32p]
        L.hp3dg_dpg_get_schur.argtypes = [_vp, ctypes.c_int32, _f64p, _f64p, _i32p, _i32p]
        L.hp3dg_dpg_index_map.argtypes = [_vp, _i32p, _i64p, _i64p, _i32p, _i64p]
        L.hp3dg_dpg_phase_times.argtypes = [_vp, _f32p, ctypes.c_int32]
        L.hp3dg_dpg_pass_stats.argtypes = [_vp, _i64p]
        L.hp3dg_dpg_last_bad_element.argtypes = [_vp]
        L.hp3dg_dpg_last_bad_element.restype = ctypes.c_int32
        L.hp3dg_dpg_end.argtypes = [_vp]
        L.hp3dg_dpg_end.restype = None
        _lib = L
        # the tuning table shipped with the package, unless the environment
        # names one (the library reads that itself at the first submit)
        if not os.environ.get("HP3DG_TUNE_FILE") and os.path.exists(DEFAULT_TUNE_FILE):
            L.hp3dg_tune_load(os.fsencode(DEFAULT_TUNE_FILE), None)
    return _lib


class Constraints(ctypes.Structure):
    """hp3dg_constraints: logic's data of the constrained elements."""
    _fields_ = [("n", ctypes.c_int32), ("iel", _i32p), ("node_off", _i64p), ("nodm", _i32p),
                ("ndof", _i32p), ("bcflag", _i32p), ("coef_off", _i64p), ("coef_k", _i32p),
                ("coef_l", _i32p), ("coef_v", _f64p), ("zdofd", _f64p)]


def pack_constraints(cons):
    """Constraints struct (and the arrays it points to) from a list with, per
    element, None or a dict with nodm, ndof, bc, ck, cl, cv (and optionally
    zd, the Dirichlet values of the modified dof)."""
    iel = [e for e, c in enumerate(cons) if c is not None]
    arrs = {}
    arrs["iel"] = np.array(iel, np.int32)
    arrs["node_off"] = np.concatenate([[0], np.cumsum([len(cons[e]["nodm"]) for e in iel])]).astype(np.int64)
    arrs["nodm"] = np.concatenate([cons[e]["nodm"] for e in iel]).astype(np.int32)
    arrs["ndof"] = np.concatenate([cons[e]["ndof"] for e in iel]).astype(np.int32)
    arrs["bcflag"] = np.concatenate([cons[e]["bc"] for e in iel]).astype(np.int32)
    arrs["coef_off"] = np.concatenate([[0], np.cumsum([len(cons[e]["ck"]) for e in iel])]).astype(np.int64)
    arrs["coef_k"] = np.concatenate([cons[e]["ck"] for e in iel]).astype(np.int32)
    arrs["coef_l"] = np.concatenate([cons[e]["cl"] for e in iel]).astype(np.int32)
    arrs["coef_v"] = np.concatenate([cons[e]["cv"] for e in iel]).astype(np.float64)
    zd = None
    if any("zd" in cons[e] for e in iel):
        zd = np.concatenate([cons[e].get("zd", np.zeros(int(np.sum(cons[e]["ndof"]))))
                             for e in iel]).astype(np.float64)
    arrs["zdofd"] = zd
    st = Constraints(len(iel), *[_p(arrs[k], t) for k, t in
                                 (("iel", _i32p), ("node_off", _i64p), ("nodm", _i32p),
                                  ("ndof", _i32p), ("bcflag", _i32p), ("coef_off", _i64p),
                                  ("coef_k", _i32p), ("coef_l", _i32p), ("coef_v", _f64p),
                                  ("zdofd", _f64p))])
    return st, arrs


def mesh_descriptors(mesh):
    """Element descriptors (hp3dg_elem_desc array) of a mesh dict."""
    ne = mesh["nelem"]
    d = np.zeros(ne, dtype=DESC_DTYPE)
    d["etype"] = mesh["etype"]
    d["mdle"] = np.arange(ne, dtype=np.int32)
    d["norder"] = mesh["norder"]
    d["nori_edge"] = mesh["nori_edge"]
    d["nori_face"] = mesh["nori_face"]
    d["nodes"] = mesh["nodes"]
    d["bcflag"] = mesh["bcflag"]
    return d


def _p(a, t):
    return None if a is None else a.ctypes.data_as(t)


class ElementPass:
    """One batched element pass (a context of the C ABI)."""

    def __init__(self, precision=FP64, integration=0, isol=10, keep_elem=False, timing=False,
                 device=0, ozaki_radix=0, ozaki_digits=0, graph=True, schur_tc=True,
                 download_chunks=0, fault_inject=0, tune=True):
        self.L = lib()
        o = Opts()
        o.precision = precision
        o.integration = integration
        o.isol = isol
        o.keep_elem = int(keep_elem)
        o.timing = int(timing)
        o.device = device
        o.ozaki_radix = ozaki_radix
        o.ozaki_digits = ozaki_digits
        o.launch_mode = 0 if graph else 1
        o.schur_fp64 = 0 if schur_tc else 1
        o.download_chunks = download_chunks
        o.fault_inject = fault_inject
        o.tune = 0 if tune else 1
        self.ctx = _vp()
        self._check(self.L.hp3dg_batch_begin(ctypes.byref(o), ctypes.byref(self.ctx)), "begin")
        self.nel = 0

    def _check(self, rc, what):
        if rc != 0:
            bad = self.L.hp3dg_last_bad_element(self.ctx) if self.ctx else -1
            raise HP3DGError(rc, f"{what}: {self.L.hp3dg_strerror(rc).decode()}", bad)

    def set_stream(self, stream_ptr):
        self._check(self.L.hp3dg_set_stream(self.ctx, _vp(stream_ptr)), "set_stream")

    def submit(self, mesh, zdofd=None, desc=None, constraints=None):
        """constraints: None, or per element None / dict (see pack_constraints)."""
        self.mesh = mesh
        self.desc = mesh_descriptors(mesh) if desc is None else desc
        self.xvert = np.ascontiguousarray(mesh["xvert"], dtype=np.float64)
        self.kappa = np.ascontiguousarray(mesh["kappa"], dtype=np.float64)
        self.zd = None if zdofd is None else np.ascontiguousarray(np.concatenate(zdofd), np.float64)
        self.nel = mesh["nelem"]
        if constraints is None:
            self._check(self.L.hp3dg_batch_submit(self.ctx, self.nel,
                                                  self.desc.ctypes.data_as(_vp),
                                                  _p(self.xvert, _f64p), _p(self.kappa, _f64p),
                                                  _p(self.zd, _f64p), int(mesh["nnodes"])),
                        "submit")
        else:
            self._cons, self._cons_arrs = pack_constraints(constraints)
            self._check(self.L.hp3dg_batch_submit_constrained(
                self.ctx, self.nel, self.desc.ctypes.data_as(_vp), _p(self.xvert, _f64p),
                _p(self.kappa, _f64p), _p(self.zd, _f64p), int(mesh["nnodes"]),
                ctypes.byref(self._cons)), "submit")

    def run(self):
        self._check(self.L.hp3dg_batch_run(self.ctx), "run")

    def set_geometry(self, xnod):
        """Isoparametric geometry: a list of per-element (nrdofH, 3) arrays of
        geometry dof in element dof order (None: back to the vertices)."""
        if xnod is None:
            self._check(self.L.hp3dg_batch_set_geometry(self.ctx, None), "set_geometry")
            return
        self._xnod = np.ascontiguousarray(np.concatenate([np.asarray(x, np.float64).reshape(-1, 3)
                                                          for x in xnod]).ravel())
        self._check(self.L.hp3dg_batch_set_geometry(self.ctx, _p(self._xnod, _f64p)),
                    "set_geometry")

    def gdof_points(self, etav):
        """Block coordinates (npts x 3) at which the caller evaluates its
        geometry-block maps for update_gdof; etav: n_elem x 8 x 3 element
        vertices in block coordinates."""
        etav = np.ascontiguousarray(etav, np.float64)
        n = ctypes.c_int64()
        self._check(self.L.hp3dg_gdof_points(self.ctx, _p(etav, _f64p), None, ctypes.byref(n)),
                    "gdof_points")
        eta = np.zeros((max(n.value, 1), 3))
        self._check(self.L.hp3dg_gdof_points(self.ctx, _p(etav, _f64p), _p(eta, _f64p),
                                             ctypes.byref(n)), "gdof_points")
        return eta[: n.value]

    def update_gdof(self, etav, x, dxdeta, linear=None, apply=False):
        """Geometry dof of every element (list of (nrdofH, 3) arrays, element
        dof order) from the maps' values x (npts x 3) and Jacobians dxdeta
        (npts x 3 x 3) at gdof_points(etav); apply=True makes them the pass's
        geometry."""
        etav = np.ascontiguousarray(etav, np.float64)
        x = np.ascontiguousarray(x, np.float64)
        j = np.ascontiguousarray(dxdeta, np.float64)
        lin = None if linear is None else np.ascontiguousarray(linear, np.int32)
        sizes = self.nrdof_h()
        out = np.zeros(max(3 * int(sizes.sum()), 1))
        self._check(self.L.hp3dg_update_gdof(self.ctx, _p(etav, _f64p), _p(x, _f64p), _p(j, _f64p),
                                             None if lin is None else _p(lin, _i32p),
                                             _p(out, _f64p), int(apply)), "update_gdof")
        off = np.concatenate([[0], np.cumsum(sizes)])
        return [out[3 * off[e]: 3 * off[e + 1]].reshape(-1, 3).copy() for e in range(self.nel)]

    def dirichlet_dofs(self, isol):
        """Per element Dirichlet values of the interface dof (update_Ddof on
        the GPU), split per element (the zdofd layout of submit)."""
        n = ctypes.c_int64()
        self._check(self.L.hp3dg_dirichlet_dofs(self.ctx, isol, None, ctypes.byref(n)), "dirichlet")
        z = np.zeros(max(n.value, 1))
        self._check(self.L.hp3dg_dirichlet_dofs(self.ctx, isol, _p(z, _f64p), ctypes.byref(n)),
                    "dirichlet")
        ni = [int(sum(self._node_ndof(e))) for e in range(self.nel)]
        return np.split(z[: n.value], np.cumsum(ni)[:-1])

    def nrdof_h(self):
        """Every element's H1 dof count (hexahedra: the 26 nodes and the
        interior)."""
        out = np.zeros(self.nel, np.int64)
        for e in range(self.nel):
            o = int(self.mesh["norder"][e][18])
            x, y, z = o // 100, (o // 10) % 10, o % 10
            out[e] = sum(self._node_ndof(e)) + max(x - 1, 0) * max(y - 1, 0) * max(z - 1, 0)
        return out

    def _node_ndof(self, e):
        no = self.mesh["norder"][e]
        nd = [1] * 8 + [max(int(no[i]) - 1, 0) for i in range(12)]
        for f in range(6):
            a, b = int(no[12 + f]) // 10, int(no[12 + f]) % 10
            nd.append(max(a - 1, 0) * max(b - 1, 0))
        return nd

    def sync(self):
        self._check(self.L.hp3dg_batch_sync(self.ctx), "sync")

    def download(self):
        self._check(self.L.hp3dg_batch_download(self.ctx), "download")

    def sizes(self):
        v = [ctypes.c_int64() for _ in range(4)]
        self._check(self.L.hp3dg_output_sizes(self.ctx, *[ctypes.byref(x) for x in v]), "sizes")
        return [x.value for x in v]

    def condensed(self, e):
        nnz, nl, _, _ = self.sizes()
        nc = ctypes.c_int32()
        self._check(self.L.hp3dg_get_condensed(self.ctx, e, None, None, ctypes.byref(nc)), "cond")
        zb = np.zeros(max(nc.value, 1)); zs = np.zeros(max(nc.value ** 2, 1))
        self._check(self.L.hp3dg_get_condensed(self.ctx, e, _p(zb, _f64p), _p(zs, _f64p),
                                               ctypes.byref(nc)), "cond")
        n = nc.value
        return zb[:n], zs[: n * n].reshape(n, n)

    def schur(self, e):
        nb = ctypes.c_int32(); ni = ctypes.c_int32()
        self._check(self.L.hp3dg_get_schur(self.ctx, e, None, None, ctypes.byref(nb),
                                           ctypes.byref(ni)), "schur")
        a = np.zeros(max(nb.value * ni.value, 1)); b = np.zeros(max(nb.value, 1))
        self._check(self.L.hp3dg_get_schur(self.ctx, e, _p(a, _f64p), _p(b, _f64p),
                                           ctypes.byref(nb), ctypes.byref(ni)), "schur")
        return (a[: nb.value * ni.value].reshape(ni.value, nb.value).T.copy(), b[: nb.value])

    def outputs(self):
        """Every element's condensed outputs after download, concatenated in
        element order: dict of zastif (row-major nrdofc^2 blocks), zbload,
        aschur (column-major nb x ni blocks), bschur and the offsets of each
        (elem_nnz, lcon_off, schur_off, bub_off; n_elem + 1 entries)."""
        nnz, nl, ns, nbub = self.sizes()
        _, _, _, lo, en = self.index_map()
        nb = np.zeros(self.nel, np.int64); ni = np.zeros(self.nel, np.int64)
        b_, i_ = ctypes.c_int32(), ctypes.c_int32()
        for e in range(self.nel):
            self._check(self.L.hp3dg_get_schur(self.ctx, e, None, None, ctypes.byref(b_),
                                               ctypes.byref(i_)), "schur")
            nb[e], ni[e] = b_.value, i_.value
        so = np.concatenate([[0], np.cumsum(nb * ni)]).astype(np.int64)
        bo = np.concatenate([[0], np.cumsum(nb)]).astype(np.int64)
        za = np.zeros(max(nnz, 1)); zb = np.zeros(max(nl, 1))
        sa = np.zeros(max(ns, 1)); sb = np.zeros(max(nbub, 1))
        nc = ctypes.c_int32()
        for e in range(self.nel):
            self._check(self.L.hp3dg_get_condensed(self.ctx, e, zb[lo[e]:].ctypes.data_as(_f64p),
                                                   za[en[e]:].ctypes.data_as(_f64p),
                                                   ctypes.byref(nc)), "cond")
            self._check(self.L.hp3dg_get_schur(self.ctx, e, sa[so[e]:].ctypes.data_as(_f64p),
                                               sb[bo[e]:].ctypes.data_as(_f64p),
                                               ctypes.byref(b_), ctypes.byref(i_)), "schur")
        return dict(zastif=za, zbload=zb, aschur=sa, bschur=sb, elem_nnz=en, lcon_off=lo,
                    schur_off=so, bub_off=bo)

    def elem(self, e, n):
        a = np.zeros((n, n), order="F"); b = np.zeros(n)
        self._check(self.L.hp3dg_get_elem(self.ctx, e, a.ctypes.data_as(_f64p), n,
                                          _p(b, _f64p)), "elem")
        return a, b

    def index_map(self):
        nnz, nl, _, _ = self.sizes()
        nf = np.zeros(self.mesh["nnodes"], dtype=np.int32)
        en = np.zeros(self.nel + 1, dtype=np.int64)
        lo = np.zeros(self.nel + 1, dtype=np.int64)
        lc = np.zeros(max(nl, 1), dtype=np.int32)
        nr = ctypes.c_int64()
        self._check(self.L.hp3dg_index_map(self.ctx, _p(nf, _i32p), _p(en, _i64p), _p(lo, _i64p),
                                           _p(lc, _i32p), ctypes.byref(nr)), "index_map")
        return nr.value, nf, lc[:nl], lo, en

    def backsub(self, x_global):
        self._xg = np.ascontiguousarray(x_global, dtype=np.float64)
        self._check(self.L.hp3dg_backsub(self.ctx, _p(self._xg, _f64p)), "backsub")

    def dofs(self, e):
        n = ctypes.c_int32()
        self._check(self.L.hp3dg_get_dofs(self.ctx, e, None, ctypes.byref(n)), "dofs")
        d = np.zeros(n.value)
        self._check(self.L.hp3dg_get_dofs(self.ctx, e, _p(d, _f64p), ctypes.byref(n)), "dofs")
        return d

    def element_error(self, isol):
        e2 = np.zeros(self.nel); n2 = np.zeros(self.nel)
        self._check(self.L.hp3dg_element_error(self.ctx, isol, _p(e2, _f64p), _p(n2, _f64p)),
                    "element_error")
        return e2, n2

    def adjoint(self, dofs=None):
        """dJ/dkappa (n_elem) and per-element vertex contributions (n_elem, 8, 3)
        of the compliance J = f^T u; dofs: list of full element dof vectors or
        None (those of backsub)."""
        d = None if dofs is None else np.ascontiguousarray(np.concatenate(dofs), np.float64)
        dk = np.zeros(self.nel); dx = np.zeros((self.nel, 8, 3))
        self._check(self.L.hp3dg_adjoint(self.ctx, _p(d, _f64p), _p(dk, _f64p), _p(dx, _f64p)),
                    "adjoint")
        return dk, dx

    def phase_times(self):
        t = (ctypes.c_float * 6)()
        self._check(self.L.hp3dg_phase_times(self.ctx, t, 6), "times")
        return list(t)

    def mixed_config(self):
        r, d, p = ctypes.c_int32(), ctypes.c_int32(), ctypes.c_int32()
        self._check(self.L.hp3dg_mixed_config(self.ctx, ctypes.byref(r), ctypes.byref(d),
                                              ctypes.byref(p)), "mixed_config")
        return r.value, d.value, p.value

    def pass_stats(self):
        """(kernel launches per run from the captured graph, or -1; algorithmic
        contraction FLOPs per run)."""
        k, f = ctypes.c_int64(), ctypes.c_double()
        self._check(self.L.hp3dg_pass_stats(self.ctx, ctypes.byref(k), ctypes.byref(f)), "stats")
        return k.value, f.value

    def bin_info(self):
        """Per bin of the last submit: dicts of etype, n, nb, nint, nel, cond
        (condensation variant in use: 1 fused tensor-core, 2 FP64 factor +
        tensor-core Schur update, 3 FP64), grp (contraction raster group
        requested, 0 = built-in), tuned (the table supplied the variant); and
        each element's bin."""
        nb = ctypes.c_int32()
        self._check(self.L.hp3dg_bin_info(self.ctx, ctypes.byref(nb), 0, None, None), "bin_info")
        bins = []
        info = np.zeros(8, np.int32)
        for b in range(nb.value):
            self._check(self.L.hp3dg_bin_info(self.ctx, None, b, _p(info, _i32p), None), "bin_info")
            bins.append(dict(zip(("etype", "n", "nb", "nint", "nel", "cond", "grp", "tuned"),
                                 (int(x) for x in info))))
        bin_of = np.zeros(max(self.nel, 1), np.int32)
        self._check(self.L.hp3dg_bin_info(self.ctx, None, -1, None, _p(bin_of, _i32p)), "bin_info")
        return bins, bin_of[: self.nel]

    def ozaki_pairs(self):
        return self.mixed_config()[2]

    def close(self):
        if self.ctx:
            self.L.hp3dg_batch_end(self.ctx)
            self.ctx = _vp()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


# --------------------------------------------------------------------------
# tuning table (hp3dg_tune_*)
DEFAULT_TUNE_FILE = os.path.join(HERE, "tune", "gb300.json")


def tune_load(path=DEFAULT_TUNE_FILE):
    """Load a tuning table (JSON written by hp3d_gb300.autotune) for every
    later submit of this process; None clears it.  Returns the number of bin
    entries."""
    n = ctypes.c_int32()
    rc = lib().hp3dg_tune_load(None if path is None else os.fsencode(path), ctypes.byref(n))
    if rc != 0:
        raise HP3DGError(rc, f"tune_load {path}")
    return n.value


def tune_lookup(etype, n, nb, nint, precision=MIXED):
    """(cond, grp, nstage) of the loaded table for a bin, or None when the
    table has no entry for it."""
    c, g, s = ctypes.c_int32(), ctypes.c_int32(), ctypes.c_int32()
    rc = lib().hp3dg_tune_lookup(etype, n, nb, nint, precision, ctypes.byref(c), ctypes.byref(g),
                                 ctypes.byref(s))
    return (c.value, g.value, s.value) if rc == 0 else None


# --------------------------------------------------------------------------
# ultraweak DPG Maxwell (hexahedra), hp3dg_dpg_*
# --------------------------------------------------------------------------
class DpgOpts(ctypes.Structure):
    _fields_ = [("omega", ctypes.c_double), ("mu", ctypes.c_double),
                ("epsilon", ctypes.c_double), ("gamma", ctypes.c_double),
                ("alpha", ctypes.c_double), ("ibcflag", ctypes.c_int32),
                ("nord_add", ctypes.c_int32), ("isol", ctypes.c_int32),
                ("icomp", ctypes.c_int32), ("device", ctypes.c_int32),
                ("timing", ctypes.c_int32), ("keep_elem", ctypes.c_int32),
                ("precision", ctypes.c_int32), ("reserved", ctypes.c_int32 * 4)]


class DPGPass:
    """One batch of the DPG Maxwell element pass (a context of the C ABI)."""

    def __init__(self, omega=2 * np.pi, mu=1.0, epsilon=1.0, gamma=1.0, alpha=1.0, ibcflag=0,
                 nord_add=1, isol=1, icomp=1, device=0, timing=False, keep_elem=False,
                 precision=FP64):
        self.L = lib()
        o = DpgOpts(omega, mu, epsilon, gamma, alpha, ibcflag, nord_add, isol, icomp, device,
                    int(timing), int(keep_elem), precision)
        self.ctx = _vp()
        self._check(self.L.hp3dg_dpg_begin(ctypes.byref(o), ctypes.byref(self.ctx)), "begin")
        self.nel = 0

    def _check(self, rc, what):
        if rc != 0:
            bad = self.L.hp3dg_dpg_last_bad_element(self.ctx) if self.ctx else -1
            raise HP3DGError(rc, f"{what}: {self.L.hp3dg_strerror(rc).decode()}", bad)

    def submit(self, mesh, eps, bcflag):
        """mesh: a hexa mesh dict; eps: complex relative permittivity per
        element; bcflag: (n_elem, 26) DPG node flags (bit 0 E known, bit 1 H
        known, bit 2 impedance face)."""
        self.mesh = mesh
        d = mesh_descriptors(mesh)
        d["bcflag"] = np.asarray(bcflag, dtype=np.int32)
        self.desc = d
        self.xvert = np.ascontiguousarray(np.asarray(mesh["xvert"])[:, :8], dtype=np.float64)
        self.eps = np.ascontiguousarray(np.asarray(eps, dtype=np.complex128))
        self.nel = mesh["nelem"]
        self._check(self.L.hp3dg_dpg_submit(self.ctx, self.nel, self.desc.ctypes.data_as(_vp),
                                            _p(self.xvert, _f64p),
                                            self.eps.ctypes.data_as(_f64p),
                                            int(mesh["nnodes"])), "submit")

    def run(self):
        self._check(self.L.hp3dg_dpg_run(self.ctx), "run")

    def sync(self):
        self._check(self.L.hp3dg_dpg_sync(self.ctx), "sync")

    def download(self):
        self._check(self.L.hp3dg_dpg_download(self.ctx), "download")

    def sizes(self):
        v = [ctypes.c_int32() for _ in range(3)]
        self._check(self.L.hp3dg_dpg_sizes(self.ctx, *[ctypes.byref(x) for x in v]), "sizes")
        return [x.value for x in v]

    def elem(self, e):
        n = self.sizes()[0]
        a = np.zeros((n, n), dtype=np.complex128, order="F"); b = np.zeros(n, np.complex128)
        self._check(self.L.hp3dg_dpg_get_elem(self.ctx, e, a.ctypes.data_as(_f64p), n,
                                              b.ctypes.data_as(_f64p)), "elem")
        return a, b

    def condensed(self, e):
        nc = ctypes.c_int32()
        self._check(self.L.hp3dg_dpg_get_condensed(self.ctx, e, None, None, ctypes.byref(nc)),
                    "cond")
        n = nc.value
        zb = np.zeros(max(n, 1), np.complex128); zs = np.zeros(max(n * n, 1), np.complex128)
        self._check(self.L.hp3dg_dpg_get_condensed(self.ctx, e, zb.ctypes.data_as(_f64p),
                                                   zs.ctypes.data_as(_f64p),
                                                   ctypes.byref(nc)), "cond")
        return zb[:n], zs[: n * n].reshape(n, n)

    def schur(self, e):
        _, ni, nb = self.sizes()
        a = np.zeros(nb * ni, np.complex128); b = np.zeros(nb, np.complex128)
        self._check(self.L.hp3dg_dpg_get_schur(self.ctx, e, a.ctypes.data_as(_f64p),
                                               b.ctypes.data_as(_f64p), None, None), "schur")
        return a.reshape(ni, nb).T.copy(), b

    def index_map(self):
        lo = np.zeros(self.nel + 1, dtype=np.int64)
        en = np.zeros(self.nel + 1, dtype=np.int64)
        nr = ctypes.c_int64()
        self._check(self.L.hp3dg_dpg_index_map(self.ctx, None, None, _p(lo, _i64p), None,
                                               ctypes.byref(nr)), "index_map")
        nf = np.zeros(self.mesh["nnodes"], dtype=np.int32)
        lc = np.zeros(max(int(lo[-1]), 1), dtype=np.int32)
        self._check(self.L.hp3dg_dpg_index_map(self.ctx, _p(nf, _i32p), _p(en, _i64p),
                                               _p(lo, _i64p), _p(lc, _i32p), ctypes.byref(nr)),
                    "index_map")
        return nr.value, nf, lc[: lo[-1]], lo, en

    def phase_times(self):
        t = (ctypes.c_float * 5)()
        self._check(self.L.hp3dg_dpg_phase_times(self.ctx, t, 5), "times")
        return list(t)

    def pass_stats(self):
        """Kernels launched on the device by the last run()."""
        k = ctypes.c_int64()
        self._check(self.L.hp3dg_dpg_pass_stats(self.ctx, ctypes.byref(k)), "stats")
        return k.value

    def close(self):
        if self.ctx:
            self.L.hp3dg_dpg_end(self.ctx)
            self.ctx = _vp()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
