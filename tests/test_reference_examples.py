"""The reference's example programs build unchanged against this library.

Each examples/<name>/<name>.c of hydroFV is compiled, as it is, against
include/ and linked to libhydro_gb300.so (the reference links the same
sources to its `hydro` target, examples/*/CMakeLists.txt:14-23).  On a
machine without a GPU the program must fail loudly inside launch_simulation
with the CUDA error, in the reference's traceback format: there is no CPU
fallback.  The programs are read from the staged copy of the reference tree
(oracle/_ref/examples, made by `make -C oracle stage`), so the test skips
where there is none.
"""
import glob
import os
import shutil
import subprocess
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, os.path.join(ROOT, "oracle"))
import oracle as O  # noqa: E402

EXAMPLES = O.REF_EXAMPLES
SOURCES = sorted(glob.glob(os.path.join(EXAMPLES, "*", "*.c")))

pytestmark = pytest.mark.skipif(not SOURCES or shutil.which("gcc") is None,
                                reason="reference examples or gcc not available")


def _build(src, out_dir, hydro_lib):
    import hydrofv_gb300 as H
    libdir = os.path.dirname(H.LIB_PATH)
    exe = os.path.join(out_dir, os.path.splitext(os.path.basename(src))[0])
    cmd = ["gcc", "-std=gnu99", "-O1", "-Wno-format", "-I", os.path.join(ROOT, "include"), "-o", exe, src,
           "-L", libdir, "-l:" + os.path.basename(H.LIB_PATH), "-lm", "-Wl,-rpath," + libdir]
    p = subprocess.run(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
    assert p.returncode == 0, p.stdout
    return exe


@pytest.mark.parametrize("src", SOURCES, ids=[os.path.basename(s) for s in SOURCES])
def test_example_compiles_and_links_unchanged(src, tmp_path, hydro_lib):
    assert os.path.exists(_build(src, str(tmp_path), hydro_lib))


def test_example_fails_loudly_without_a_gpu(tmp_path, hydro_lib):
    import hydrofv_gb300 as H
    if H.device_count() > 0:
        pytest.skip("a GPU is visible: the program would run")
    src = [s for s in SOURCES if s.endswith("sod_shock_1d.c")]
    if not src:
        pytest.skip("sod_shock_1d.c not in the reference examples")
    exe = _build(src[0], str(tmp_path), hydro_lib)
    p = subprocess.run([exe], cwd=str(tmp_path), stdout=subprocess.PIPE, stderr=subprocess.STDOUT,
                       text=True, timeout=120)
    assert p.returncode != 0
    assert "launch_simulation" in p.stdout and "CUDA error" in p.stdout, p.stdout[-2000:]


@pytest.mark.skipif(shutil.which("cmake") is None, reason="cmake not available")
def test_example_builds_with_its_own_cmake(tmp_path, hydro_lib):
    """The route of the examples' own CMakeLists.txt (add_subdirectory of
    ../../src, target_link_libraries(... hydro)) with ../../src reaching
    include/ through a symbolic link: the unmodified file configures, builds
    and links libhydro_gb300.so."""
    import hydrofv_gb300 as H
    src = [s for s in SOURCES if s.endswith("sod_shock_1d.c")]
    if not src:
        pytest.skip("sod_shock_1d not in the reference examples")
    ex = tmp_path / "examples" / "sod_shock_1d"
    shutil.copytree(os.path.dirname(src[0]), ex)
    os.symlink(os.path.join(ROOT, "include"), tmp_path / "src")
    build = tmp_path / "build"
    for cmd in (["cmake", "-S", str(ex), "-B", str(build)], ["cmake", "--build", str(build)]):
        p = subprocess.run(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True, timeout=600)
        assert p.returncode == 0, p.stdout[-3000:]
    exe = build / "sod_shock_1d"
    assert exe.exists()
    ldd = subprocess.run(["ldd", str(exe)], stdout=subprocess.PIPE, text=True).stdout
    assert os.path.basename(H.LIB_PATH) in ldd
