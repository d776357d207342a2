"""HYDRO_GPU_TRACE: a 2D drop-in launch prints the host wall time of each of
its phases to stderr (GPU; a child process, since the variable is read once
per process)."""
import os
import re
import subprocess
import sys

import pytest

pytestmark = pytest.mark.gpu

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

CHILD = r"""
import sys
sys.path.insert(0, sys.argv[1])
import hydrofv_gb300 as H
from hydrofv_gb300.problems import shear_layer
p = shear_layer(64, steps=5)
r = H.run_2d(p.nx, p.ny, p.g, (0, 1, 0, 1), p.gamma, p.W, p.U, bc=p.bc,
             slope_limiter=p.slope_limiter, cfl=p.cfl, tf=p.tf, max_steps=5)
assert r.code == 0, r.message
"""


@pytest.mark.parametrize("value,traced", [("1", True), ("0", False)])
def test_launch_phases_on_stderr(gpu_available, value, traced):
    env = dict(os.environ, HYDRO_GPU_TRACE=value)
    p = subprocess.run([sys.executable, "-c", CHILD, ROOT], env=env, stdout=subprocess.PIPE,
                       stderr=subprocess.PIPE, text=True, timeout=300)
    assert p.returncode == 0, p.stderr[-2000:]
    phases = re.findall(r"hydro_gpu: (\S+)\s+([0-9.]+) ms", p.stderr)
    if traced:
        assert [name for name, _ in phases] == ["set-up", "upload", "begin", "stepping", "download",
                                                "teardown"]
        assert all(float(ms) >= 0.0 for _, ms in phases)
    else:
        assert phases == []
