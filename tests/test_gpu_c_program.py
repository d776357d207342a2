"""A C program written against hydro.h, built with gcc and run on the GPU.

tests/c_programs/sod_tube.c sets up the 1000-cell Sod tube through the
reference's API (system_init, convert_primitive_to_conserved, the parameter
structs) and calls launch_simulation, as the reference's example programs do.
It is compiled against include/ and linked to libhydro_gb300.so, like a
hydroFV program moved to this library.  Its final state is compared with
the reference's own result for the same problem (golden fixture).
"""
import os
import shutil
import subprocess

import numpy as np
import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)

pytestmark = pytest.mark.gpu


@pytest.mark.skipif(shutil.which("gcc") is None, reason="gcc not available")
def test_c_program_runs_sod_on_the_gpu(gpu_available, tmp_path):
    import hydrofv_gb300 as H
    libdir = os.path.dirname(H.LIB_PATH)
    exe = str(tmp_path / "sod_tube")
    build = subprocess.run(["gcc", "-std=gnu99", "-O2", "-I", os.path.join(ROOT, "include"), "-o", exe,
                            os.path.join(HERE, "c_programs", "sod_tube.c"), "-L", libdir,
                            "-l:" + os.path.basename(H.LIB_PATH), "-lm", "-Wl,-rpath," + libdir],
                           stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
    assert build.returncode == 0, build.stdout
    out = str(tmp_path / "state.bin")
    run = subprocess.run([exe, out], stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True,
                         timeout=300)
    assert run.returncode == 0, run.stdout[-3000:]

    g = np.load(os.path.join(HERE, "golden", "sod_1000_godunov_exact.npz"))
    total = g["W"].shape[1]
    raw = np.fromfile(out, dtype=np.uint8)
    assert raw.size == 24 + 6 * total * 8
    steps = int(raw[:8].view(np.int64)[0])
    t = float(raw[8:16].view(np.float64)[0])
    state = raw[24:].view(np.float64).reshape(6, total)
    assert steps == int(g["num_steps"])
    assert t == pytest.approx(float(g["t"]), rel=1e-14)
    for got, want in ((state[:3], g["W"]), (state[3:], g["U"])):
        scale = np.max(np.abs(want), axis=1, keepdims=True)
        assert np.all(np.abs(got - want) <= 1e-12 * scale)
