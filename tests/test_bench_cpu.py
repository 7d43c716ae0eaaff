"""The bench's reference arm on the host: the JSON line it prints and its
time budget (the oracle's REF22 restatement of four_strucf_omp, no GPU)."""
import argparse
import json
import os
import subprocess
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)


def _line(text):
    return json.loads([r for r in text.strip().splitlines() if r.startswith("{")][-1])


def test_reference_arm_json_line():
    out = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference", "--workload",
                          "perovskite-201^2", "--steps", "2", "--warmup", "1"],
                         capture_output=True, text=True, timeout=600, cwd=ROOT)
    assert out.returncode == 0, out.stderr[-2000:]
    d = _line(out.stdout)
    assert d["impl"] == "reference" and d["n_gpus"] == 1 and d["steps"] == 2 and d["warmup"] == 1
    assert d["metric"] == "G atom.hkl pairs/s for |F|^2" and d["unit"] == "G pairs/s"
    assert d["higher_is_better"] is True and d["value"] > 0 and d["ms_per_step"] > 0
    assert d["config"]["workload"] == "perovskite-201^2"
    cb = d["cpu_baseline"]
    assert cb["kind"] == "port" and cb["cores"] >= 1 and cb["value"] == d["value"] and "rows" in cb["sample"]
    assert d["e2e"] == {"value": d["value"], "unit": "G pairs/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}


def test_reference_arm_budget_takes_part_of_the_atoms(capsys, monkeypatch):
    import bench
    monkeypatch.setattr(bench, "REF_BUDGET_S", 0.0)
    args = argparse.Namespace(workload="perovskite-201^2", steps=3, warmup=1, gpus=1)
    bench.run_reference(args, 1, 0)
    d = _line(capsys.readouterr().out)
    assert d["steps"] == 3 and d["value"] > 0
    assert "the first 1% of the atoms per step" in d["cpu_baseline"]["sample"]


def test_reference_arm_other_ranks_print_nothing(capsys):
    import bench
    args = argparse.Namespace(workload="perovskite-201^2", steps=1, warmup=0, gpus=2)
    bench.run_reference(args, 2, 1)
    assert capsys.readouterr().out == ""
