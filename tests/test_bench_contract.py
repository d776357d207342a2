"""bench.py's output line: the keys and types every run must print.

The GPU arm runs a small grid on the GPU; the reference arm runs on the CPU
(the CPU implementation of the path on a tiny grid).
"""
import json
import os
import subprocess
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

BASE_KEYS = {"metric": str, "value": float, "unit": str, "n_gpus": int, "steps": int, "warmup": int,
             "ms_per_step": float, "higher_is_better": bool, "scaling": str, "dtype": str,
             "data": str, "config": dict, "e2e": dict}


def _run(args, tmp_path):
    p = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py")] + args, cwd=str(tmp_path),
                       stdout=subprocess.PIPE, stderr=subprocess.PIPE, text=True, timeout=900)
    assert p.returncode == 0, p.stderr[-3000:]
    lines = [l for l in p.stdout.splitlines() if l.startswith("{")]
    assert len(lines) == 1, p.stdout
    return json.loads(lines[0])


def _check_base(d, steps, warmup):
    for k, t in BASE_KEYS.items():
        assert k in d, k
        assert isinstance(d[k], t) or (t is float and isinstance(d[k], int)), (k, d[k])
    assert "vs_baseline" in d and d["vs_baseline"] is None
    assert d["steps"] == steps and d["warmup"] >= 3 and warmup >= 0
    assert d["value"] > 0 and d["ms_per_step"] > 0
    assert "workload" in d["config"]
    e = d["e2e"]
    for k in ("value", "unit", "h2d_bytes_per_step", "d2h_bytes_per_step"):
        assert k in e, k


def test_reference_arm_line(tmp_path):
    d = _run(["--impl", "reference", "--size", "64", "--steps", "2", "--warmup", "1"], tmp_path)
    _check_base(d, 2, 1)
    assert d["impl"] == "reference"
    cb = d["cpu_baseline"]
    assert cb["kind"] in ("reference", "port") and cb["cores"] >= 1 and cb["value"] == d["value"]
    assert d["e2e"]["h2d_bytes_per_step"] == 0 and d["e2e"]["d2h_bytes_per_step"] == 0


@pytest.mark.gpu
def test_gpu_arm_line(gpu_available, tmp_path):
    d = _run(["--size", "256", "--steps", "5", "--warmup", "3"], tmp_path)
    _check_base(d, 5, 3)
    r = d["roofline"]
    for k in ("bound", "achieved", "peak", "unit", "frac", "traffic"):
        assert k in r, k
    assert r["bound"] in ("hbm", "tensor") and r["frac"] == pytest.approx(r["achieved"] / r["peak"])
    assert d["gpu_launches"] > 0
    c = d["clocks"]
    assert {"sm_mhz", "sm_max_mhz", "reasons"} <= set(c)
    cb = d["cpu_baseline"]
    for k in ("value", "unit", "cores", "kind", "sample"):
        assert k in cb, k
    assert d["e2e"]["h2d_bytes_per_step"] > 0 and d["e2e"]["d2h_bytes_per_step"] > 0
    # both forms carry their arithmetic and HBM roofs; the precision study's
    # 8192^2 point blast rides along on the default workload
    forms = d["forms"]
    assert forms["fp32"]["roofline"]["bound"] == "hbm"
    # the binding roofs beyond HBM: the FP64 pipe, and instruction issue for the
    # FP32 form; their figures come with the committed counts (2048^2 only)
    fr64, fr32 = d["fp_roofline"], forms["fp32"]["fp_roofline"]
    assert fr64["bound"] == "fp64_pipe" and fr32["bound"] == "issue"
    if "achieved" in fr64:
        assert fr64["frac"] == pytest.approx(fr64["achieved"] / fr64["peak"]) and "issue" in fr64
    if "fp32_pipe" in fr32 and "achieved" in fr32:
        assert fr32["frac"] == pytest.approx(fr32["achieved"] / fr32["peak"])
    blast = forms["point_blast_8192"]
    assert blast["fp64"]["value"] > 0 and blast["fp32"]["value"] > 0
    assert set(blast["fp32"]["rel_l1_vs_fp64"]) == {"density", "velocity_x", "velocity_y", "pressure"}
    assert blast["fp32"]["rel_l1_vs_fp64"]["density"] < 1e-4
    ens = forms["ensemble_256"]
    assert ens["fp64"]["value"] > 0 and ens["fp32"]["speedup_vs_fp64"] > 1.7
    assert ens["fp32"]["rel_l1_vs_fp64"]["density"] < 1e-4
    adj = forms["adjoint_1024"]
    assert adj["backward_vs_forward"] <= 3.0 and adj["recompute_mismatches"] == 0
    assert adj["dot_product_rel"] < 1e-11 and adj["fd_frozen_rel"] < 1e-6
    # the reference arm reports the same workload under the same config
    r = _run(["--impl", "reference", "--size", "256", "--steps", "5", "--warmup", "3"], tmp_path)
    assert r["config"] == d["config"] and r["warmup"] == d["warmup"] and r["steps"] == d["steps"]
