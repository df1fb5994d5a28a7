"""The tuning table of the element pass through the C ABI, without a GPU:
hp3dg_tune_load parses the JSON the autotuner writes, hp3dg_tune_lookup
returns a bin's variant, a malformed file is refused and leaves the loaded
table as it was, NULL clears it, and the file named by HP3DG_TUNE_FILE is
read when nothing was loaded.  The committed table parses."""
import json
import os
import subprocess
import sys

import numpy as np
import pytest

from hp3d_gb300 import hp3dg as H

REC = {"etype": 1, "n": 216, "nb": 64, "nint": 343, "precision": 1, "cond": 2, "grp": 9,
       "ms_cond": {"1": 1.0, "2": 0.9}, "nel": 512}


@pytest.fixture(autouse=True)
def _clear():
    yield
    H.tune_load(None)


def _write(tmp_path, obj, name="t.json"):
    p = tmp_path / name
    p.write_text(obj if isinstance(obj, str) else json.dumps(obj))
    return str(p)


def test_load_and_lookup(tmp_path):
    p = _write(tmp_path, {"version": 1, "launch": {"nstage": 4}, "bins": [REC]})
    assert H.tune_load(p) == 1
    assert H.tune_lookup(1, 216, 64, 343, H.MIXED) == (2, 9, 4)
    assert H.tune_lookup(1, 216, 64, 343, H.FP64) is None
    assert H.tune_lookup(2, 216, 64, 343, H.MIXED) is None


@pytest.mark.parametrize("bad", [
    "{", '{"bins": [1, 2]}', '{"bins": [{"etype": 9, "n": 1, "nb": 0, "nint": 1, "precision": 1}]}',
    '{"bins": [{"etype": 1, "n": 8, "nb": 0, "nint": 8, "precision": 1, "cond": 7}]}',
    '{"launch": {"nstage": -1}}', '[]', '{"bins": []} trailing'])
def test_malformed_tables_are_refused_and_keep_the_loaded_one(tmp_path, bad):
    good = _write(tmp_path, {"bins": [REC]})
    H.tune_load(good)
    with pytest.raises(H.HP3DGError) as ei:
        H.tune_load(_write(tmp_path, bad, "bad.json"))
    assert ei.value.code == -7
    assert H.tune_lookup(1, 216, 64, 343) == (2, 9, 0)


def test_missing_file_and_clear(tmp_path):
    with pytest.raises(H.HP3DGError):
        H.tune_load(str(tmp_path / "none.json"))
    H.tune_load(_write(tmp_path, {"bins": [REC]}))
    assert H.tune_load(None) == 0
    assert H.tune_lookup(1, 216, 64, 343) is None


def test_environment_variable_is_read_when_nothing_was_loaded(tmp_path):
    p = _write(tmp_path, {"launch": {"nstage": 3}, "bins": [REC]})
    code = ("from hp3d_gb300 import hp3dg as H; "
            "print(H.tune_lookup(1, 216, 64, 343))")
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    env = dict(os.environ, HP3DG_TUNE_FILE=p, PYTHONPATH=root)
    out = subprocess.run([sys.executable, "-c", code], env=env, capture_output=True, text=True,
                         timeout=120, cwd=root)
    assert out.returncode == 0, out.stderr
    assert out.stdout.strip() == "(2, 9, 3)"


def test_committed_table_parses():
    if not os.path.exists(H.DEFAULT_TUNE_FILE):
        pytest.skip("no tuning table committed")
    n = H.tune_load(H.DEFAULT_TUNE_FILE)
    tab = json.load(open(H.DEFAULT_TUNE_FILE))
    assert n == len(tab["bins"]) > 0
    for r in tab["bins"]:
        assert H.tune_lookup(r["etype"], r["n"], r["nb"], r["nint"], r["precision"])[:2] == \
            (r["cond"], r["grp"])


def test_autotune_sweep_logic_with_a_model_of_the_timings(tmp_path, monkeypatch):
    """The sweep's decisions on CPU, with the GPU replaced by a timing model:
    keys in order of contraction work, each condensation variant timed as the
    whole workload's pass and kept only when it beats the current pass by
    0.3 %, a key tuned on the first workload kept on the second, unusable
    variants skipped, raster group and ring depth kept at their defaults when
    no candidate is clearly faster; the table written is one the library
    loads."""
    from hp3d_gb300 import autotune as AT
    bins_by_wl = {
        "hexa": [dict(etype=1, n=216, nb=64, nint=343, nel=1000)],
        "mixed": [dict(etype=1, n=216, nb=64, nint=343, nel=50),
                  dict(etype=2, n=140, nb=30, nint=198, nel=400),
                  dict(etype=3, n=84, nb=10, nint=392, nel=300),
                  dict(etype=1, n=343, nb=125, nint=343, nel=100)],
    }
    # per key: time of each usable variant (variant 0 = the built-in rule = 1
    # where usable, else 3)
    cost = {(1, 216, 64, 343): {1: 10.0, 2: 12.0, 3: 14.0},
            (2, 140, 30, 198): {1: 2.0, 2: 1.5, 3: 1.99},
            (3, 84, 10, 392): {1: 1.0, 2: 1.001, 3: 0.999},
            (1, 343, 125, 343): {3: 3.0}}
    state = {"wl": None}

    class FakePass:
        def __init__(self, *a, **k):
            pass

        def submit(self, m):
            state["wl"] = m["wl"]

        def bin_info(self):
            bins = [dict(b, cond=0, grp=0, tuned=0) for b in bins_by_wl[state["wl"]]]
            return bins, np.arange(len(bins), dtype=np.int32)

        def close(self):
            pass

    def fake_time_pass(m, reps=5, warm=2, tune=True):
        total, got = 0.0, []
        for b in bins_by_wl[m["wl"]]:
            key = (b["etype"], b["n"], b["nb"], b["nint"])
            r = H.tune_lookup(*key, H.MIXED)
            c = r[0] if r else 0
            usable = cost[key]
            if c not in usable:
                c = 1 if 1 in usable else 3
            total += usable[c]
            got.append(dict(b, cond=c, grp=r[1] if r else 0, tuned=int(r is not None)))
        if r is not None and r[2] == 3:
            total += 1.0  # a shallow ring is slower
        return total, got

    monkeypatch.setattr(AT.H, "ElementPass", FakePass)
    monkeypatch.setattr(AT, "time_pass", fake_time_pass)
    monkeypatch.setattr(AT, "workload_mesh", lambda wl, seed=12345: {"wl": wl, "nelem": 10})
    monkeypatch.setattr(AT, "sub_mesh", lambda m, idx: m)
    import types
    monkeypatch.setitem(sys.modules, "torch", types.SimpleNamespace(
        cuda=types.SimpleNamespace(get_device_name=lambda i: "model")))
    out = str(tmp_path / "tab.json")
    tab = AT.sweep(("hexa", "mixed"), out, reps=1, log=lambda *a: None)
    recs = {(r["etype"], r["n"], r["nb"], r["nint"]): r for r in tab["bins"]}
    assert recs[(1, 216, 64, 343)]["cond"] == 0       # the built-in rule is fastest
    assert recs[(2, 140, 30, 198)]["cond"] == 2       # 25 % better pass
    assert recs[(3, 84, 10, 392)]["cond"] == 0        # 0.001 ms is within 0.3 %
    assert recs[(1, 343, 125, 343)]["cond"] == 0      # one usable variant
    assert set(recs[(1, 343, 125, 343)]["ms_cond"]) == {"3"}
    assert recs[(1, 216, 64, 343)]["grp"] == 0 and tab["launch"]["nstage"] == 0
    assert H.tune_load(out) == len(tab["bins"])
    assert H.tune_lookup(2, 140, 30, 198) == (2, 0, 0)
