"""The tuning table of the element pass through the C ABI, without a GPU:
hp3dg_tune_load parses the JSON the autotuner writes, hp3dg_tune_lookup
returns a bin's variant, a malformed file is refused and leaves the loaded
table as it was, NULL clears it, and the file named by HP3DG_TUNE_FILE is
read when nothing was loaded.  The committed table parses."""
import json
import os
import subprocess
import sys

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
