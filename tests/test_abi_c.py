"""The C ABI from C: tests/abi_client.c, compiled by gcc against
include/hp3dg.h and linked with libhp3dg.so, is the kind of caller the
Fortran host's ISO_C_BINDING interface is.

- Without a GPU: the offset and size of every field of the public structs,
  as the C compiler lays them out from the header, equal what the ctypes
  binding (hp3d_gb300/hp3dg.py) assumes.
- On the GPU: the C client fills hp3dg_opts and the descriptors itself, runs
  begin / submit / run / sync / download / get_condensed / get_schur /
  index_map, and its outputs equal the Python binding's bit for bit and the
  oracle's (elem_opt + stc_fwd + celem_systemI compression) within 1e-12.
"""
import ctypes
import os
import shutil
import struct
import subprocess

import numpy as np
import pytest

from hp3d_gb300 import build as B
from hp3d_gb300 import hp3dg as H
from hp3d_gb300 import mesh as M
from oracle import oracle as O

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


@pytest.fixture(scope="module")
def client(tmp_path_factory):
    gcc = shutil.which("gcc") or shutil.which("cc")
    if gcc is None:
        pytest.skip("no C compiler")
    lib = B.build()
    exe = str(tmp_path_factory.mktemp("abi") / "abi_client")
    libdir = os.path.dirname(lib)
    cmd = [gcc, "-std=c99", "-O1", "-Wall", "-Werror", "-I", os.path.join(ROOT, "include"),
           os.path.join(ROOT, "tests", "abi_client.c"), "-o", exe, "-L", libdir, "-lhp3dg",
           f"-Wl,-rpath,{libdir}"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    return exe


def _layout(exe):
    out = subprocess.run([exe, "layout"], capture_output=True, text=True, check=True).stdout
    fields, sizes = {}, {}
    for ln in out.splitlines():
        s, f, off, sz = ln.split()
        if f == "-":
            sizes[s] = int(off)
        else:
            fields[(s, f)] = (int(off), int(sz))
    return fields, sizes


def _ctypes_fields(cls):
    return {name: (getattr(cls, name).offset, getattr(cls, name).size) for name, *_ in cls._fields_}


def test_struct_field_offsets_match_the_c_compiler(client):
    fields, sizes = _layout(client)
    for sname, cls in (("hp3dg_opts", H.Opts), ("hp3dg_constraints", H.Constraints),
                       ("hp3dg_dpg_opts", H.DpgOpts)):
        got = _ctypes_fields(cls)
        want = {f: v for (s, f), v in fields.items() if s == sname}
        assert got == want, (sname, got, want)
        assert ctypes.sizeof(cls) == sizes[sname], sname
    want = {f: v for (s, f), v in fields.items() if s == "hp3dg_elem_desc"}
    got = {f: (H.DESC_DTYPE.fields[f][1], H.DESC_DTYPE.fields[f][0].itemsize)
           for f in H.DESC_DTYPE.names}
    assert got == want
    assert H.DESC_DTYPE.itemsize == sizes["hp3dg_elem_desc"]


def _write_input(path, mesh):
    desc = H.mesh_descriptors(mesh)
    with open(path, "wb") as f:
        f.write(struct.pack("<ii", mesh["nelem"], mesh["nnodes"]))
        f.write(desc.tobytes())
        f.write(np.ascontiguousarray(mesh["xvert"], np.float64).tobytes())
        f.write(np.ascontiguousarray(mesh["kappa"], np.float64).tobytes())


def _read_output(path, nel):
    buf = open(path, "rb").read()
    off = 0

    def take(dt, n):
        nonlocal off
        a = np.frombuffer(buf, dtype=dt, count=n, offset=off)
        off += a.nbytes
        return a

    nrdof, nl = take(np.int64, 2)
    lcon = take(np.int32, int(nl))
    els = []
    for _ in range(nel):
        nc, nb, ni = take(np.int32, 3)
        zb = take(np.float64, nc)
        zs = take(np.float64, nc * nc).reshape(nc, nc)
        asch = take(np.float64, nb * ni).reshape(ni, nb).T
        bsch = take(np.float64, nb)
        els.append((zb, zs, asch, bsch))
    assert off == len(buf)
    return int(nrdof), lcon, els


@pytest.mark.gpu
@pytest.mark.parametrize("precision", [H.FP64, H.MIXED])
def test_c_client_runs_the_pass(client, tmp_path, precision):
    mesh = M.random_orientations(M.structured_hexa(2, 3, perturb=0.15, kappa_logrange=(-2, 2),
                                                   seed=23), seed=4)
    fin, fout = str(tmp_path / "in.bin"), str(tmp_path / "out.bin")
    _write_input(fin, mesh)
    r = subprocess.run([client, "run", fin, fout, str(precision)], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    nrdof, lcon, els = _read_output(fout, mesh["nelem"])

    ep = H.ElementPass(precision, integration=1, isol=10, download_chunks=1)
    ep.submit(mesh)
    ep.run()
    ep.download()
    nr, _, plcon, _, _ = ep.index_map()
    assert nrdof == nr
    assert np.array_equal(lcon, plcon)
    for e in range(mesh["nelem"]):
        zb, zs = ep.condensed(e)
        a, b = ep.schur(e)
        czb, czs, ca, cb = els[e]
        assert np.array_equal(czb, zb) and np.array_equal(czs, zs)
        assert np.array_equal(ca, a) and np.array_equal(cb, b)
        # the oracle: elem_opt -> stc_fwd -> celem_systemI compression
        K, bl, rc = O.elem(1, mesh["norder"][e], mesh["nori_edge"][e], mesh["nori_face"][e],
                           mesh["xvert"][e], mesh["kappa"][e], isol=10, integration=1)
        nb = O.nrdof_bubble(1, mesh["norder"][e])
        aii, bi, _, _, _ = O.stc_fwd(K, bl, nb, 0)
        _, ozb, ozs, _ = O.celem_compress(1, mesh["norder"][e], mesh["bcflag"][e], aii, bi)
        if ozs.size:
            tol = 1e-12 if precision == H.FP64 else 1e-10
            assert np.abs(czs - ozs).max() <= tol * np.abs(ozs).max()
            assert np.abs(czb - ozb).max() <= tol * max(np.abs(ozb).max(), 1e-300)
    ep.close()
