#!/usr/bin/env python
"""Benchmark of the hp3D element pass on GB300 (one JSON line on rank 0).

Workload (the metric's configuration): Galerkin Poisson on 24^3 = 13,824
hexahedra of the unit cube, isotropic p = 5 (216 H1 dof per element,
64 bubbles, 152 interface dof), INTEGRATION = 1 (7^3 Gauss points),
interior vertices perturbed by U(-0.15h, 0.15h) (trilinear geometry),
kappa_e = 10**U(-2, 2), f = 3 pi^2 sin(pi x) sin(pi y) sin(pi z),
homogeneous Dirichlet BC on the whole boundary.  Seeded synthetic mesh.

A step = one element pass over the whole mesh: geometry + load, B^T D B
contraction, static condensation, compression and index maps (everything the
reference's mumps_sc STEP 2 element loop computes before MUMPS).
``value`` times ``hp3dg_batch_run`` with the inputs already in HBM;
``e2e`` times submit (host -> device) + run + download (device -> host of
the condensed matrices, loads, Schur blocks and LCON) through the C ABI.

--impl reference times the CPU oracle (a restatement of the reference's
Fortran element loop; the Fortran reference cannot be compiled here) with
OpenMP over the host cores on a bounded sample of the same workload.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time

# the CPU legs run the oracle on OpenMP threads, each calling a single-threaded
# BLAS; set before numpy / scipy load their BLAS
os.environ.setdefault("OPENBLAS_NUM_THREADS", "1")

import numpy as np  # noqa: E402

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "condensed elements/s at p=5: mixed-precision vs plain FP64 GPU at 1e-10 rel err"


def mixed_cells(args):
    """Grid of the hp batching workload: 25^3 cells by default."""
    return 25 if args.n == 24 else args.n


def make_mesh(args, seed=12345):
    """hexa: the metric's uniform mesh.  mixed: the hp-adaptive mesh of
    hexahedra, prisms and tetrahedra of the unit cube (orders 1..6 drawn per
    element, minimum rule on shared edges and faces, kappa = 10**U(-1, 1)):
    n^3 cells with the tetrahedra in a 6 x 6 x 7 corner block and prism
    columns along x, y and z beside it -- at n = 25, 19,129 elements,
    68.6 / 23.5 / 7.9 % hexa / prism / tet."""
    from hp3d_gb300 import mesh as M
    if args.workload == "mixed":
        n = mixed_cells(args)
        return M.mixed_mesh(n, a=(n - 6) / n, b=(n - 7) / n, cy=(n - 6) / n, pmax=6,
                            perturb=0.0, kappa_logrange=(-1, 1), seed=seed)
    return M.structured_hexa(args.n, args.p, perturb=0.15, kappa_logrange=(-2, 2), seed=seed)


class ClockSampler:
    """nvidia-smi clocks/throttle sampling during the timed region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index=0):
        self.index = index
        self.proc = None
        self.lines = []

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--id={self.index}", f"--query-gpu={self.FIELDS}",
                 "--format=csv,noheader,nounits", "-lms", "100"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
        except Exception:
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            parts = [x.strip() for x in ln.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1])); smax.append(float(parts[2]))
            except ValueError:
                continue
            for nm, v in zip(names, parts[5:9]):
                if v.lower() == "active":
                    reasons.add(nm)
        return {"sm_mhz": statistics.median(sm) if sm else None,
                "sm_max_mhz": max(smax) if smax else None, "reasons": sorted(reasons),
                "samples": len(sm)}


def measured_peaks():
    """(HBM GB/s, BF16 TFLOP/s burst, BF16 TFLOP/s sustained, kind)."""
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        d = json.load(open(p))
        return (d.get("hbm_gbs", 6800.0), d.get("bf16_tflops", 1900.0),
                d.get("bf16_tflops_sustained", d.get("bf16_tflops", 1700.0)), "measured")
    return 6800.0, 1900.0, 1700.0, "fallback"


def measured_fp64_tflops(device):
    """FP64 rate of this GPU: cuBLAS DGEMM 4096^3 through torch, best of 5."""
    import torch
    a = torch.randn(4096, 4096, dtype=torch.float64, device=device)
    b = torch.randn(4096, 4096, dtype=torch.float64, device=device)
    for _ in range(2):
        a @ b
    torch.cuda.synchronize()
    best = float("inf")
    e0 = torch.cuda.Event(enable_timing=True); e1 = torch.cuda.Event(enable_timing=True)
    for _ in range(5):
        e0.record(); a @ b; e1.record(); torch.cuda.synchronize()
        best = min(best, e0.elapsed_time(e1) / 1000.0)
    return 2.0 * 4096 ** 3 / best / 1e12


def cpu_model():
    try:
        out = subprocess.run(["lscpu"], capture_output=True, text=True, timeout=10).stdout
        for ln in out.splitlines():
            if ln.startswith("Model name:"):
                return ln.split(":", 1)[1].strip()
    except Exception:
        pass
    import platform
    return platform.processor() or platform.machine()


def seg_rel(x, y, off):
    """Largest per-segment relative difference max|x - y| / max|y| over the
    segments [off[k], off[k+1]) of two concatenated arrays."""
    off = np.asarray(off, np.int64)
    keep = np.diff(off) > 0
    if not keep.any():
        return 0.0
    idx = off[:-1][keep]
    end = int(off[-1])
    d = np.maximum.reduceat(np.abs(x[:end] - y[:end]), idx)
    m = np.maximum.reduceat(np.abs(y[:end]), idx)
    return float((d / np.maximum(m, 1e-300)).max())


OUT_KEYS = (("zastif", "elem_nnz"), ("zbload", "lcon_off"), ("aschur", "schur_off"),
            ("bschur", "bub_off"))


def cpu_baseline(mesh, isol, integration, seconds=15.0, nthreads=0, gpu_out=None,
                 min_sample=0):
    """Time the oracle (OpenMP over the host cores, BLAS-3 DSYRK and
    DGETRF / DGETRS / DGEMM from SciPy's bundled OpenBLAS, as the reference
    calls them) on a bounded sample of the mesh; with gpu_out (the mixed GPU
    pass's outputs) also the largest per-element relative difference of the
    GPU's condensed blocks from the oracle's on that sample."""
    from oracle import oracle as O
    blas = O.use_blas() or "oracle loops (no BLAS library found)"
    cores = nthreads if nthreads > 0 else (os.cpu_count() or 1)
    # size the sample: one probe round of `cores` elements, spread evenly over
    # the mesh (an hp mesh's orders vary with position)
    nel = mesh["nelem"]
    spread = lambda k: np.unique(np.round(np.linspace(0, nel - 1, k)).astype(np.int64))  # noqa: E731
    probe = spread(min(cores, nel))
    t0 = time.perf_counter()
    O.element_pass(mesh, isol=isol, integration=integration, stc_method=0, nthreads=cores,
                   elements=probe)
    dt = time.perf_counter() - t0
    per_round = max(dt, 1e-3)
    rounds = max(1, int(seconds / per_round))
    sample = spread(min(nel, max(rounds * len(probe), min_sample)))
    ns = len(sample)
    t0 = time.perf_counter()
    r = O.element_pass(mesh, isol=isol, integration=integration, stc_method=0, nthreads=cores,
                       elements=sample)
    dt = time.perf_counter() - t0
    assert r["rc"] == 0
    out = {"value": ns / dt, "unit": "elements/s", "cores": cores, "cpu": cpu_model(),
           "kind": "port",
           "sample": f"{ns} of {nel} elements (evenly spread over ELEM_ORDER), one pass, "
                     f"{dt:.1f} s, oracle C restatement (elem_opt with DSYRK, stc_fwd_gen with "
                     f"DGETRF/DGETRS/DGEMM, compression), OpenMP, {blas}"}
    if gpu_out is not None:
        worst = {}
        for key, okey in OUT_KEYS:
            w = 0.0
            for j, e in enumerate(sample):
                a0, a1 = r[okey][j], r[okey][j + 1]
                g0 = gpu_out[okey][e]
                ref = r[key][a0:a1]
                if ref.size == 0:
                    continue
                got = gpu_out[key][g0:g0 + (a1 - a0)]
                w = max(w, float(np.abs(got - ref).max() / max(np.abs(ref).max(), 1e-300)))
            worst[key] = w
        out["gpu_vs_oracle_on_sample"] = worst
    return out


def final_solution_check(args, local, n=6):
    """The condensed interface system (what MUMPS solves) on n^3 hexahedra of
    the metric's kind (p, INTEGRATION, perturbation, kappa range as the
    workload), assembled from the mixed GPU pass, the FP64 GPU pass and the
    FP64 oracle; each solved to the working accuracy by iterative refinement
    on one sparse LU of the oracle's matrix.  Returns the relative 2-norm
    differences mixed vs FP64 GPU and FP64 GPU vs oracle (the FP64 floor)."""
    import scipy.sparse as sp
    import scipy.sparse.linalg as spla
    sys.path.insert(0, os.path.join(ROOT, "tests"))
    import fem_harness as FH
    from hp3d_gb300 import hp3dg as H
    from hp3d_gb300 import mesh as M
    from oracle import oracle as O
    O.use_blas()
    m = M.structured_hexa(n, args.p, perturb=0.15, kappa_logrange=(-2, 2), seed=7)
    systems = {}
    for name, prec in (("mixed", H.MIXED), ("fp64", H.FP64)):
        ep = H.ElementPass(prec, integration=args.integration, isol=args.isol, device=local)
        ep.submit(m); ep.run(); ep.download()
        systems[name] = FH.gpu_elements(ep, m)
        ep.close()
    systems["oracle"] = FH.oracle_element_outputs(m, args.isol, integration=args.integration,
                                                  stc_method=0)
    ndofm = np.stack([el["ndofm"] for el in systems["oracle"]]).astype(np.int32)
    nrdof, _, lcon, lcon_off, _ = O.index_maps(FH.nnode_of(m), m["nodes"], ndofm, m["nnodes"])
    mats = {}
    for name, els in systems.items():
        rows, cols, vals = [], [], []
        rhs = np.zeros(nrdof)
        for e in range(m["nelem"]):
            lc = lcon[lcon_off[e]:lcon_off[e + 1]] - 1
            nc = len(lc)
            if nc == 0:
                continue
            rows.append(np.repeat(lc, nc)); cols.append(np.tile(lc, nc))
            vals.append(els[e]["zastif"].ravel())
            np.add.at(rhs, lc, els[e]["zbload"])
        A = sp.coo_matrix((np.concatenate(vals), (np.concatenate(rows), np.concatenate(cols))),
                          shape=(nrdof, nrdof)).tocsc()
        mats[name] = (A, rhs)
    lu = spla.splu(mats["oracle"][0])
    sol = {}
    for name, (A, rhs) in mats.items():
        x = lu.solve(rhs)
        for _ in range(8):
            dx = lu.solve(rhs - A @ x)
            x = x + dx
            if np.linalg.norm(dx) <= 1e-16 * np.linalg.norm(x):
                break
        sol[name] = x
    rel = lambda a, b: float(np.linalg.norm(a - b) / np.linalg.norm(b))  # noqa: E731
    return {"mesh": f"{n}^3 hexahedra, p={args.p}, INTEGRATION={args.integration}, "
                    f"U(-0.15h,0.15h), kappa 10**U(-2,2)",
            "unknowns": int(nrdof),
            "mixed_vs_fp64_gpu": rel(sol["mixed"], sol["fp64"]),
            "fp64_gpu_vs_fp64_oracle": rel(sol["fp64"], sol["oracle"]),
            "note": "interface solution of the condensed system (the MUMPS solve), relative "
                    "2-norm; the FP64-vs-FP64 figure is the floor set by the global "
                    "conditioning"}


def gpu_accuracy(mesh, args, local, stream):
    """Mixed vs plain FP64 GPU pass on every element of the workload (untimed
    contexts keeping the element matrices): the largest per-element relative
    difference of the element matrices, condensed matrices and loads, ASchur
    and BSchur.  Returns (figures, the mixed pass's outputs)."""
    from hp3d_gb300 import hp3dg as H
    eps = {}
    for prec in (H.FP64, H.MIXED):
        ep = H.ElementPass(prec, integration=args.integration, isol=args.isol, keep_elem=True,
                           device=local)
        ep.set_stream(stream.cuda_stream)
        ep.submit(mesh); ep.run(); ep.download()
        eps[prec] = ep
    om, of = eps[H.MIXED].outputs(), eps[H.FP64].outputs()
    res = {"elements": int(mesh["nelem"])}
    for key, okey in OUT_KEYS:
        res[key] = seg_rel(om[key], of[key], of[okey])
    n = (args.p + 1) ** 3
    w = 0.0
    for e in range(mesh["nelem"]):
        km, _ = eps[H.MIXED].elem(e, n)
        kf, _ = eps[H.FP64].elem(e, n)
        w = max(w, float(np.abs(km - kf).max() / np.abs(kf).max()))
    res["element_matrix"] = w
    for ep in eps.values():
        ep.close()
    return res, om


def run_reference(args, rank, world):
    """The reference's element pass on the host cores: the oracle restatement
    (per-element shape functions at every point, DSYRK, DGETRF / DGETRS /
    DGEMM from SciPy's OpenBLAS, compression) with OpenMP over all cores, the
    whole mesh every step (warm-up steps included)."""
    if rank != 0:
        return
    from oracle import oracle as O
    blas = O.use_blas() or "oracle loops (no BLAS library found)"
    mesh = make_mesh(args)
    cores = os.cpu_count() or 1
    nel = mesh["nelem"]
    times = []
    for i in range(args.warmup + args.steps):
        t0 = time.perf_counter()
        r = O.element_pass(mesh, isol=args.isol, integration=args.integration, stc_method=0,
                           nthreads=cores)
        dt = time.perf_counter() - t0
        assert r["rc"] == 0
        if i >= args.warmup:
            times.append(dt)
    ms = 1000.0 * statistics.median(times)
    v = nel / (ms / 1000.0)
    cb = {"value": v, "unit": "elements/s", "cores": cores, "cpu": cpu_model(), "kind": "port",
          "sample": f"the whole mesh ({nel} elements) every step, oracle C restatement "
                    f"(elem_opt with DSYRK, stc_fwd_gen with DGETRF/DGETRS/DGEMM, "
                    f"compression), OpenMP, {blas}"}
    line = {"impl": "reference", "metric": METRIC, "value": v, "unit": "elements/s",
            "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": ms, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": config_dict(args, world, mesh),
            "cpu_baseline": cb,
            "e2e": {"value": v, "unit": "elements/s", "h2d_bytes_per_step": 0,
                    "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def tuning_info():
    """The tuning table the pass reads at submit (loaded with the library)."""
    from hp3d_gb300 import hp3dg as H
    path = os.environ.get("HP3DG_TUNE_FILE") or H.DEFAULT_TUNE_FILE
    if not os.path.exists(path):
        return None
    try:
        with open(path) as f:
            tab = json.load(f)
        return {"file": os.path.relpath(path, os.path.dirname(os.path.abspath(__file__))),
                "bin_entries": len(tab.get("bins", [])), "device": tab.get("device")}
    except (OSError, ValueError):
        return None


def config_dict(args, world, mesh):
    cfg = _config_dict(args, world, mesh)
    cfg["tuning"] = tuning_info()
    return cfg


def _config_dict(args, world, mesh):
    if args.workload == "mixed":
        cnt = np.bincount(mesh["etype"], minlength=4)[1:]
        return {"workload": f"galerkin_poisson_hp_mixed_{mixed_cells(args)}^3_cells_pmax6_integration{args.integration}",
                "elements_per_gpu": int(mesh["nelem"]),
                "hexa_prism_tet": [int(x) for x in cnt], "orders": "1..6 per element, min rule",
                "layout": "tetrahedra in a 6x6x7 corner block, prism columns along x, y, z",
                "perturbation": "none (unit-cube geometry)", "kappa": "10**U(-1,1)",
                "precision": args.precision,
                "parallelism": f"replicas{world}" if world > 1 else "single",
                "l2": "working set per step > L2, no flush needed"}
    return {"workload": f"galerkin_poisson_hexa_{args.n}^3_p{args.p}_integration{args.integration}",
            "elements_per_gpu": args.n ** 3, "p": args.p, "quadrature_points": (min(args.p + args.integration, 6) + 1) ** 3,
            "perturbation": "U(-0.15h,0.15h) interior vertices", "kappa": "10**U(-2,2)",
            "precision": args.precision, "parallelism": f"replicas{world}" if world > 1 else "single",
            "l2": "working set per step > L2 (condensed outputs 3.7 GB), no flush needed"}


DPG_METRIC = "DPG Maxwell elements/s (complex FP64, trial p=3, test p=4, condensed)"


def job_max(x, world):
    """The job's figure for a per-rank time: the maximum over the ranks
    (all_reduce MAX on the process group's device: CUDA under NCCL, the host
    under gloo).  One rank: x itself."""
    if world <= 1:
        return float(x)
    import torch
    import torch.distributed as dist
    dev = "cuda" if dist.get_backend() == "nccl" else "cpu"
    t = torch.tensor([float(x)], dtype=torch.float64, device=dev)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def job_value(world, units_per_rank, ms_job):
    """Whole-job throughput of weak scaling: every rank processes
    units_per_rank (its own replica), the job takes ms_job."""
    return world * units_per_rank / (ms_job / 1000.0)


def measured_traffic(workload, kernel):
    """DRAM bytes of `kernel` on `workload` from the committed figures of an
    ncu capture (profiles/dram_traffic.txt), or None."""
    path = os.path.join(os.path.dirname(os.path.abspath(__file__)), "profiles", "dram_traffic.txt")
    try:
        with open(path) as f:
            for line in f:
                t = line.split()
                if len(t) == 5 and t[0] == "traffic" and t[1] == workload and t[2] == kernel:
                    return int(t[4]), t[3]
    except OSError:
        pass
    return None


def dpg_flops(ntest, ntrial, ni, nb):
    """Dense algebra of the DPG element per element (real FLOPs): Cholesky of
    the Gram matrix (ZPPTRF), the triangular solve of [B|l] (ZTPTRS), X^H X
    (ZHERK), then the condensation of the L2 fields (Cholesky, two solves,
    Schur update)."""
    n1 = ntrial + 1
    f = 4.0 / 3.0 * ntest ** 3 + 4.0 * ntest ** 2 * n1 + 4.0 * n1 * (n1 + 1) * ntest
    f += 4.0 / 3.0 * nb ** 3 + 8.0 * nb ** 2 * (ni + 1) + 4.0 * ni * ni * nb
    return f


def run_dpg(args, rank, world):
    """Ultraweak DPG Maxwell on 10^3 hexahedra of the unit cube: trial p = 3,
    test p + 1, omega = 2 pi, eps_r = U[1,4] (1 - i tan d), tan d = U[0, 0.1]
    per element, impedance on the wall x = 1 (IBCFLAG = 2), perfect conductor
    elsewhere, sin source (mfd_solutions case 1); interior vertices perturbed
    by U(-0.1h, 0.1h).  Seeded synthetic mesh."""
    from hp3d_gb300 import mesh as M
    from oracle import oracle as O
    n = 10 if args.n == 24 else args.n
    mesh = M.structured_hexa(n, 3, perturb=0.1, seed=4321 + rank)
    rng = np.random.default_rng(99 + rank)
    ne = mesh["nelem"]
    eps = rng.uniform(1, 4, ne) * (1 - 1j * rng.uniform(0, 0.1, ne))
    flags = M.dpg_boundary_flags(mesh, ((0, 1),))
    imp = np.zeros(ne, np.int32)
    for f in range(6):
        imp |= ((flags[:, 20 + f] >> 2) & 1) << f
    prm = O.maxw_params(isol=1, ibcflag=2)
    cfg = {"workload": f"ultraweak_dpg_maxwell_hexa_{n}^3_p3_impedance", "elements_per_gpu": ne,
           "p": 3, "test_order": 4, "quadrature_points": 125, "omega": "2 pi",
           "eps_r": "U[1,4](1 - i U[0,0.1])", "precision": args.precision,
           "parallelism": f"replicas{world}" if world > 1 else "single",
           "l2": "working set per step > L2 (Gram matrices 5.8 GB), no flush needed"}
    s = O.dpg_sizes([3] * 12 + [33] * 6 + [333])
    fl_el = dpg_flops(s["ntest"], s["ntrial"], 2 * s["nEi"], 6 * s["nQ"])

    def cpu(seconds):
        cores = os.cpu_count() or 1
        probe = np.arange(min(cores, ne))
        t0 = time.perf_counter()
        O.dpg_pass(mesh, eps, flags & 3, imp, prm, elements=probe, nthreads=cores)
        dt = max(time.perf_counter() - t0, 1e-3)
        k = max(1, int(seconds / dt)) * len(probe)
        sample = np.unique(np.round(np.linspace(0, ne - 1, min(ne, k))).astype(np.int64))
        t0 = time.perf_counter()
        r = O.dpg_pass(mesh, eps, flags & 3, imp, prm, elements=sample, nthreads=cores)
        dt = time.perf_counter() - t0
        assert r["rc"] == 0
        return {"value": len(sample) / dt, "unit": "elements/s", "cores": cores, "kind": "port",
                "sample": f"{len(sample)} of {ne} elements (evenly spread), one pass, {dt:.1f} s, "
                          f"oracle C restatement of elem_maxwell (ZPPTRF/ZTPTRS/ZHERK) + "
                          f"stc_fwd_herm + compression, OpenMP"}

    if args.impl == "reference":
        if rank != 0:
            return
        vals, cb = [], None
        sec = min(args.cpu_seconds, 120.0 / max(1, args.warmup + args.steps))
        for i in range(args.warmup + args.steps):
            c = cpu(sec)
            if i >= args.warmup:
                vals.append(c["value"])
                cb = c
        v = statistics.median(vals)
        print(json.dumps({"impl": "reference", "metric": DPG_METRIC, "value": v,
                          "unit": "elements/s", "n_gpus": world, "steps": args.steps,
                          "warmup": args.warmup, "ms_per_step": 1000.0 * ne / v,
                          "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
                          "dtype": "c128", "data": "synthetic", "config": cfg, "cpu_baseline": cb,
                          "e2e": {"value": v, "unit": "elements/s", "h2d_bytes_per_step": 0,
                                  "d2h_bytes_per_step": 0}}), flush=True)
        return

    import torch
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
    local = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(local)
    from hp3d_gb300 import build as B
    B.build()
    from hp3d_gb300 import hp3dg as H
    dprec = H.MIXED if args.precision == "mixed" else H.FP64
    ep = H.DPGPass(omega=prm.omega, ibcflag=2, isol=1, timing=True, device=local, precision=dprec)
    ep.submit(mesh, eps, flags)
    for _ in range(args.warmup):
        ep.run(); ep.sync()
    if world > 1:
        torch.distributed.barrier()
    clk = ClockSampler(local)
    clk.start()
    ph = []
    for _ in range(args.steps):
        ep.run(); ep.sync()
        ph.append(ep.phase_times())
    clocks = clk.stop()
    launches = ep.pass_stats()
    ph = np.array(ph)
    ms = job_max(float(np.median(ph[:, 4])), world)
    value = job_value(world, ne, ms)
    # end to end: submit (descriptors, vertices, permittivities), run, download
    ep.download()
    ntrial, ni, nb = ep.sizes()
    nr, _, _, lo, en = ep.index_map()
    d2h = int(16 * (en[-1] + lo[-1] + ne * (ni * nb + nb)) + 4 * lo[-1])
    h2d = int(ep.desc.nbytes + ep.xvert.nbytes + ep.eps.nbytes)
    t0 = time.perf_counter()
    for _ in range(max(1, args.e2e_steps)):
        ep.submit(mesh, eps, flags); ep.run(); ep.download()
    e2e_s = (time.perf_counter() - t0) / max(1, args.e2e_steps)
    med = np.median(ph, axis=0)
    t_la = (med[1] + med[2]) / 1000.0
    hbm, bf16, bf16s, peak_kind = measured_peaks()
    achieved = ne * fl_el / t_la / 1e12 if t_la > 0 else None
    if dprec == H.FP64:
        fp64 = measured_fp64_tflops(f"cuda:{local}")
        roof = {"bound": "fp64", "achieved": achieved, "peak": fp64, "unit": "TFLOP/s",
                "frac": achieved / fp64 if achieved else None, "traffic": None,
                "kernel": "k_dpg_dpg + k_dpg_condense",
                "note": "dense DPG algebra (Gram Cholesky, forward solve of [B|l], X^H X, L2-field "
                        "condensation) per element over the two kernels' time; peak = cuBLAS "
                        "DGEMM 4096^3 measured in this run (the measured-peaks file has no FP64 "
                        "figure)"}
    else:
        # tensor work: 28 digit pairs x 2 real products of K = 128 per complex update
        # (4 real MACs per complex MAC); the algorithmic count is the complex FLOPs
        tens = fl_el * 28 / 2.0 * 2.0
        ach = ne * tens / t_la / 1e12 if t_la > 0 else None
        roof = {"bound": "tensor", "achieved": ach, "peak": bf16, "unit": "TFLOP/s",
                "frac": ach / bf16 if ach else None,
                "kernel": "k_zupd + k_zdiag + digit slices (augmented partial Cholesky)",
                "traffic": (measured_traffic(cfg["workload"], "k_zupd") or (None,))[0],
                "note": f"BF16 digit-pair MMA work of the dense DPG algebra (28 pairs of the "
                        f"complex FLOP count) over the stage's time; peak {peak_kind}; the "
                        f"complex-FP64-equivalent rate is {ne * fl_el / t_la / 1e12:.3f} TFLOP/s"}
    cb = cpu(args.cpu_seconds) if (rank == 0 and not args.no_cpu_baseline) else None
    line = {"metric": DPG_METRIC, "value": value, "unit": "elements/s", "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "c128",
            "data": "synthetic", "config": cfg,
            "e2e": {"value": job_value(world, ne, 1000 * e2e_s), "unit": "elements/s",
                    "h2d_bytes_per_step": h2d,
                    "d2h_bytes_per_step": d2h, "ms_per_step": 1000 * e2e_s,
                    "note": "submit (descriptors, vertices, permittivities), run, download of "
                            "the condensed systems, Schur blocks and LCON"},
            "roofline": roof, "cpu_baseline": cb, "clocks": clocks,
            "gpu_launches": launches * args.steps, "launches_per_pass": launches,
            "phase_ms": {"geometry_contractions_assembly": float(med[0]),
                         "gram_cholesky_solve_herk_impedance": float(med[1]),
                         "condensation_compression": float(med[2]),
                         "index_maps": float(med[3]), "pass": float(med[4])}}
    ep.close()
    if rank == 0:
        print(json.dumps(line), flush=True)
    if world > 1:
        torch.distributed.destroy_process_group()


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--precision", default="mixed", choices=["mixed", "fp64"])
    ap.add_argument("--workload", default="hexa", choices=["hexa", "mixed", "dpg"],
                    help="hexa: uniform p hexahedra (the metric's mesh); mixed: hp-adaptive "
                         "hexa/prism/tet mesh; dpg: ultraweak DPG Maxwell, 10^3 hexahedra p=3")
    ap.add_argument("--n", type=int, default=24)
    ap.add_argument("--p", type=int, default=5)
    ap.add_argument("--integration", type=int, default=1)
    ap.add_argument("--isol", type=int, default=10)
    ap.add_argument("--cpu-seconds", type=float, default=15.0)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-fp64-compare", action="store_true")
    ap.add_argument("--no-accuracy", action="store_true",
                    help="skip the per-element mixed-vs-FP64 and oracle comparisons and the "
                         "final-solution check")
    ap.add_argument("--e2e-steps", type=int, default=10)
    ap.add_argument("--download-chunks", type=int, default=4,
                    help="e2e: pass in this many element chunks, each copied to the host "
                         "as soon as it is done (1 = one piece)")
    args = ap.parse_args()

    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if args.workload == "dpg":
        return run_dpg(args, rank, world)
    if args.impl == "reference":
        return run_reference(args, rank, world)

    import torch
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
    torch.cuda.set_device(local)
    from hp3d_gb300 import build as B
    B.build()
    from hp3d_gb300 import hp3dg as H

    mesh = make_mesh(args, seed=12345 + rank)
    prec = H.MIXED if args.precision == "mixed" else H.FP64
    stream = torch.cuda.current_stream()

    def timed(precision, steps, warmup):
        ep = H.ElementPass(precision, integration=args.integration, isol=args.isol, timing=True,
                           device=local)
        ep.set_stream(stream.cuda_stream)
        ep.submit(mesh)
        for _ in range(warmup):
            ep.run()
        ep.sync()
        if world > 1:
            torch.distributed.barrier()
        torch.cuda.synchronize()
        phases = []
        e0 = torch.cuda.Event(enable_timing=True); e1 = torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        for _ in range(steps):
            ep.run()
            ep.sync()
            phases.append(ep.phase_times())
        e1.record(stream)
        torch.cuda.synchronize()
        ms = job_max(e0.elapsed_time(e1), world)
        return ep, ms, phases

    clk = ClockSampler(local)
    clk.start()
    ep, ms, phases = timed(prec, args.steps, args.warmup)
    clocks = clk.stop()
    ms_step = ms / args.steps
    nel = mesh["nelem"]
    value = job_value(world, nel, ms_step)

    # end to end through the C ABI with host buffers (submit + run + download).
    # Each step resubmits the mesh with this step's geometry and coefficient:
    # the descriptors equal the batch's, so submit uploads xvert and kappa
    # (the per-step inputs) and keeps the device state; download copies the
    # condensed matrices, loads, Schur blocks and LCON into pinned buffers.
    nnz, nl, ns, nbub = ep.sizes()
    d2h = int(8 * (nnz + nl + ns + nbub) + 4 * nl)
    epe = H.ElementPass(prec, integration=args.integration, isol=args.isol, device=local,
                        download_chunks=args.download_chunks)
    epe.set_stream(stream.cuda_stream)
    rng = np.random.default_rng(7 + rank)
    steps_in = []
    for _ in range(args.e2e_steps):
        mk = dict(mesh)
        mk["kappa"] = mesh["kappa"] * (1.0 + 0.01 * rng.random(mesh["nelem"]))
        steps_in.append(mk)
    h2d = int(mesh["xvert"].nbytes + mesh["kappa"].nbytes)
    # the element descriptors (orders, orientations, nodes) of a fixed mesh are
    # built once, as a host that resubmits new geometry and coefficients would
    desc = H.mesh_descriptors(mesh)
    epe.submit(mesh, desc=desc); epe.run(); epe.download()  # pinned result buffers exist from here on
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    step_ms = []
    for mk in steps_in:
        ts = time.perf_counter()
        epe.submit(mk, desc=desc)
        epe.run()
        epe.download()
        step_ms.append(1000 * (time.perf_counter() - ts))
    torch.cuda.synchronize()
    e2e_s = job_max((time.perf_counter() - t0) / args.e2e_steps, world)
    epe.close()
    # one cold step: a new context (descriptor processing, allocations, bin
    # tables, operand digits, graph capture, pinned buffers) for reference
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    epc = H.ElementPass(prec, integration=args.integration, isol=args.isol, device=local)
    epc.set_stream(stream.cuda_stream)
    epc.submit(mesh); epc.run(); epc.download()
    torch.cuda.synchronize()
    cold_ms = 1000 * (time.perf_counter() - t0)
    epc.close()
    e2e = {"value": job_value(world, nel, 1000 * e2e_s), "unit": "elements/s",
           "h2d_bytes_per_step": h2d,
           "d2h_bytes_per_step": d2h, "ms_per_step": 1000 * e2e_s,
           "cold_step_ms": cold_ms,
           # the chunked pass applies to a batch of one bin (the uniform mesh)
           "download_chunks": args.download_chunks if args.workload == "hexa" else 1,
           "step_ms": [round(x, 3) for x in step_ms],
           "note": "resubmit of the mesh with new kappa each step (upload xvert+kappa, "
                   "run, download all condensed outputs, each element chunk copied as "
                   "soon as it is done); cold_step_ms = new context"}

    # the plain FP64 GPU form on the same mesh (the comparison the metric names)
    fp64 = None
    if prec == H.MIXED and not args.no_fp64_compare:
        ep64, ms64, ph64 = timed(H.FP64, max(2, min(3, args.steps)), 1)
        fp64 = {"value": world * nel / (ms64 / max(2, min(3, args.steps)) / 1000.0),
                "unit": "elements/s", "phase_ms": [round(x, 3) for x in ph64[-1]]}
        ep64.close()

    ph = np.median(np.array(phases), axis=0)
    hbm, bf16, bf16s, peak_kind = measured_peaks()
    # dominant kernel = the contraction (one launch per bin; one bin for the
    # uniform mesh); its FLOPs per run come from the library
    kernels, flops = ep.pass_stats()
    t_con = ph[2] / 1000.0
    con_note = ""
    if args.workload == "mixed":
        # bins run on parallel branches: the contraction's own time is not
        # separable, so the whole pass bounds it from above
        t_con = ph[5] / 1000.0
        con_note = "; time = whole pass (bins run concurrently), a lower bound on the rate"
    if prec == H.MIXED:
        pairs = ep.ozaki_pairs()
        # algorithmic work: the DSYRK count n(n+1) 3 nint per element
        # (elem_opt.F90:131) times the digit-pair products; the library counts
        # the executed MMA FLOPs, pairs x 2 (6 nint) n(n+1)/2, twice that (the
        # shared-operand form D.M expands the symmetric 3x3 D into 6 terms)
        alg = flops / 2.0
        roof = {"bound": "tensor", "achieved": alg / t_con / 1e12 if t_con > 0 else None,
                "peak": bf16, "unit": "TFLOP/s", "kernel": "k_ozaki_gemm",
                "algorithmic_flop_per_launch": alg,
                "executed_mma_tflops": flops / t_con / 1e12 if t_con > 0 else None,
                "note": f"achieved = (n(n+1) 3 nint per element, the DSYRK count) x {pairs} "
                        f"digit-pair passes x elements / contraction time; peak = {peak_kind} "
                        f"BF16 burst: the SM clock stayed at its maximum with no power-cap "
                        f"reason during the timed region (clocks field){con_note}"}
        if roof["achieved"]:
            roof["executed_frac"] = roof["executed_mma_tflops"] / bf16
            roof["frac_of_sustained_peak"] = roof["achieved"] / bf16s
    else:
        roof = {"bound": "fp64", "achieved": flops / t_con / 1e12 if t_con > 0 else None,
                "peak": measured_fp64_tflops(f"cuda:{local}"), "unit": "TFLOP/s",
                "kernel": "k_contract_fp64",
                "note": "FP64 CUDA-core contraction (DSYRK count) against cuBLAS DGEMM measured "
                        "in this run"}
    if roof["achieved"] is not None:
        roof["frac"] = roof["achieved"] / roof["peak"]
    tr = (measured_traffic(config_dict(args, world, mesh)["workload"], roof["kernel"])
          if args.workload == "hexa" else None)
    roof["traffic"] = tr[0] if tr else None
    if tr:
        roof["note"] += "; traffic: DRAM bytes per launch from an ncu capture of this size"
    elif prec == H.MIXED and args.workload == "hexa":
        # captures of smaller meshes of the same kind; traffic per element is not
        # constant across sizes, so nothing is scaled to this one
        small = {}
        for nn in (12, 16):
            t = measured_traffic(f"galerkin_poisson_hexa_{nn}^3_p{args.p}_integration{args.integration}",
                                 roof["kernel"])
            if t:
                small[f"{nn}^3"] = t[0]
        if small:
            roof["traffic_small_cases"] = small
            roof["note"] += ("; traffic null: DRAM bytes per launch were captured on 12^3 and "
                             "16^3 (traffic_small_cases) and do not grow in proportion to the "
                             "elements, so they are not scaled to this size")

    accuracy, mixed_out = None, None
    if prec == H.MIXED and args.workload == "hexa" and not args.no_accuracy:
        accuracy, mixed_out = gpu_accuracy(mesh, args, local, stream)
        accuracy = {"mixed_vs_fp64_gpu_per_element_max_rel": accuracy}

    cb = None
    if rank == 0 and not args.no_cpu_baseline:
        cb = cpu_baseline(mesh, args.isol, args.integration, seconds=args.cpu_seconds,
                          gpu_out=mixed_out, min_sample=256 if mixed_out is not None else 0)
        if accuracy is not None:
            accuracy["mixed_vs_oracle_per_element_max_rel"] = cb.pop("gpu_vs_oracle_on_sample")
            accuracy["oracle_sample"] = cb["sample"].split(",")[0]
            accuracy["final_solution"] = final_solution_check(args, local)
    mixed_out = None

    # kernel launches per pass: the kernel nodes of the captured graph
    launches_per_step = kernels
    line = {"metric": METRIC, "value": value, "unit": "elements/s", "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms_step,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "f64" if prec == H.FP64 else "bf16-digits->f64", "data": "synthetic",
            "config": config_dict(args, world, mesh), "e2e": e2e, "roofline": roof,
            "cpu_baseline": cb, "clocks": clocks,
            "gpu_launches": launches_per_step * args.steps if launches_per_step > 0 else None,
            "launches_per_pass": launches_per_step,
            "phase_ms": {"tables": float(ph[0]), "geometry_load": float(ph[1]),
                         "contraction": float(ph[2]), "condensation": float(ph[3]),
                         "index_maps": float(ph[4]), "pass": float(ph[5])},
            "fp64_gpu": fp64,
            "speedup_vs_fp64_gpu": (value / fp64["value"]) if fp64 else None,
            "accuracy": accuracy}
    ep.close()
    if rank == 0:
        print(json.dumps(line), flush=True)
    if world > 1:
        torch.distributed.destroy_process_group()


if __name__ == "__main__":
    main()
