"""Tuned variants of the mixed-precision pass on the GPU.

- The contraction's raster group and ring depth change only the order of the
  work: outputs are bit-identical to the built-in choice.
- Each condensation variant a bin can use (fused tensor-core, FP64 factor +
  tensor-core Schur update, FP64) is the one that runs when the table asks
  for it, and meets the pass's bar against the oracle (1e-10 relative for
  the condensed matrices and loads); a variant the bin cannot use falls back
  to the built-in rule.
- opts.tune = 1 ignores the table."""
import json

import numpy as np
import pytest

from hp3d_gb300 import hp3dg as H
from hp3d_gb300 import mesh as M
import fem_harness as FH

pytestmark = pytest.mark.gpu


@pytest.fixture(autouse=True)
def _clear():
    H.tune_load(None)
    yield
    H.tune_load(None)


def _run(m, tune=True):
    ep = H.ElementPass(H.MIXED, integration=1, isol=10, tune=tune)
    ep.submit(m)
    ep.run()
    ep.download()
    out = [(ep.condensed(e), ep.schur(e)) for e in range(m["nelem"])]
    bins, _ = ep.bin_info()
    ep.close()
    return out, bins


def _table(tmp_path, recs, nstage=0):
    p = tmp_path / "tab.json"
    p.write_text(json.dumps({"version": 1, "launch": {"nstage": nstage}, "bins": recs}))
    return H.tune_load(str(p))


def _sig(b):
    return {"etype": b["etype"], "n": b["n"], "nb": b["nb"], "nint": b["nint"], "precision": 1}


def _same(a, b):
    for ((zb1, zs1), (a1, b1)), ((zb0, zs0), (a0, b0)) in zip(a, b):
        assert np.array_equal(zb1, zb0) and np.array_equal(zs1, zs0)
        assert np.array_equal(a1, a0) and np.array_equal(b1, b0)


def test_raster_group_and_ring_depth_are_bit_identical(tmp_path):
    m = M.structured_hexa(3, 5, perturb=0.15, kappa_logrange=(-2, 2), seed=5)
    ref, bins = _run(m)
    assert len(bins) == 1 and bins[0]["tuned"] == 0
    for grp, nstage in ((1, 0), (2, 3), (7, 4)):
        _table(tmp_path, [dict(_sig(bins[0]), cond=0, grp=grp)], nstage)
        out, b2 = _run(m)
        assert b2[0]["tuned"] == 1 and b2[0]["grp"] == grp
        _same(out, ref)


def test_condensation_variants_meet_the_oracle_bar(tmp_path):
    m = M.structured_hexa(2, 5, perturb=0.15, kappa_logrange=(-2, 2), seed=6)
    ref = FH.oracle_element_outputs(m, 10, integration=1)
    _, bins = _run(m)
    for cond in (1, 2, 3):
        _table(tmp_path, [dict(_sig(bins[0]), cond=cond, grp=0)])
        out, b2 = _run(m)
        assert b2[0]["cond"] == cond
        for e, ((zb, zs), _) in enumerate(out):
            r = ref[e]
            assert np.abs(zs - r["zastif"]).max() <= 1e-10 * np.abs(r["zastif"]).max(), (cond, e)
            assert np.abs(zb - r["zbload"]).max() <= 1e-10 * np.abs(r["zbload"]).max(), (cond, e)


def test_unusable_variant_falls_back_and_tune_off_ignores_the_table(tmp_path):
    # p = 6 hexahedra: 125 bubbles, neither tensor-core condensation fits
    m = M.structured_hexa(1, 6, perturb=0.1, kappa_logrange=None, seed=7)
    ref, bins = _run(m)
    assert bins[0]["cond"] == 3
    _table(tmp_path, [dict(_sig(bins[0]), cond=1, grp=3)])
    out, b2 = _run(m)
    assert b2[0]["cond"] == 3 and b2[0]["tuned"] == 1
    _same(out, ref)
    _, b3 = _run(m, tune=False)
    assert b3[0]["tuned"] == 0 and b3[0]["grp"] == 0


def test_committed_table_applies_to_the_hp_mesh():
    import os
    if not os.path.exists(H.DEFAULT_TUNE_FILE):
        pytest.skip("no tuning table committed")
    H.tune_load(H.DEFAULT_TUNE_FILE)
    m = M.mixed_mesh(4, a=0.5, b=0.5, cy=0.5, perturb=0.1, seed=21, kappa_logrange=(-1, 1))
    out, bins = _run(m)
    ref, bref = _run(m, tune=False)
    tab = json.load(open(H.DEFAULT_TUNE_FILE))
    keys = {(r["etype"], r["n"], r["nb"], r["nint"]): r for r in tab["bins"]}
    for b in bins:
        r = keys.get((b["etype"], b["n"], b["nb"], b["nint"]))
        assert b["tuned"] == (1 if r else 0)
    # where the table keeps each bin's built-in condensation, the bits too
    if all(b["cond"] == b0["cond"] for b, b0 in zip(bins, bref)):
        _same(out, ref)
