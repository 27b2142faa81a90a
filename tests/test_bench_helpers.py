"""Host-side helpers of bench.py on the CPU: the error measures every bench line
and config test states, the per-kernel table, and the detail records (strict
JSON, non-finite values written as null)."""
import json
import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)
import bench  # noqa: E402


def test_field_error_is_worst_substrate_max_and_l2():
    rng = np.random.default_rng(3)
    ref = rng.random((4, 5, 6, 3)) + 0.5
    got = ref.copy()
    got[1, 2, 3, 0] += 1e-3           # substrate 0: one point off
    got[..., 2] *= 1.0 + 2e-4         # substrate 2: uniformly scaled
    max_rel, l2_rel = bench.field_error(got, ref)
    r = ref.reshape(-1, 3)
    d = np.abs(got.reshape(-1, 3) - r)
    want_max = max(d[:, s].max() / np.abs(r[:, s]).max() for s in range(3))
    want_l2 = max(np.linalg.norm(d[:, s]) / np.linalg.norm(r[:, s]) for s in range(3))
    assert max_rel == pytest.approx(want_max)
    assert l2_rel == pytest.approx(want_l2)
    assert bench.field_error(ref, ref) == (0.0, 0.0)


def test_kernel_table_shares_and_bandwidth():
    stats = {"sweep_x": {"launches": 4, "ms": 2.0, "bytes": 8e9},
             "cells_apply": {"launches": 4, "ms": 0.5, "bytes": 1e9},
             "idle": {"launches": 0, "ms": 0.0, "bytes": 0.0}}
    t = bench.kernel_table(stats)
    assert set(t) == {"sweep_x", "cells_apply"}  # kernels that did not run are left out
    assert t["sweep_x"]["us_per_launch"] == 500.0
    assert t["sweep_x"]["share"] + t["cells_apply"]["share"] == pytest.approx(1.0)
    assert t["sweep_x"]["gbps"] == pytest.approx(8e9 / 2e-3 / 1e9)


def test_details_are_strict_json(tmp_path, capsys):
    det = bench.Details(str(tmp_path / "d.json"))
    det.add("leg", {"value": 1.5, "bad": float("nan"), "nested": {"inf": float("inf"), "ok": 2}})
    det.write()
    line = capsys.readouterr().err.strip().splitlines()[-1]
    rec = json.loads(line)
    assert rec["detail"] == "leg" and rec["value"] == 1.5 and rec["nested"]["ok"] == 2
    whole = json.load(open(tmp_path / "d.json"))
    assert whole["leg"]["value"] == 1.5
    # non-finite values are written as null
    assert rec["bad"] is None and rec["nested"]["inf"] is None
    assert "NaN" not in line and "Infinity" not in line
