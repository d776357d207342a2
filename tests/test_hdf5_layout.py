"""The HDF5 snapshot layout, checked without an HDF5 library (CPU only).

Neither build machine has libhdf5, so the library itself writes snapshots
as raw .bin files; its HDF5 writer (csrc/host/storing.c, the
HYDRO_WITH_HDF5 branch) is what a build on a machine with HDF5 uses.  That
branch is compiled here against a recording stand-in for the HDF5 API
(tests/hdf5_fake/), and so is the reference's own writer
(src/storing.c:230-765, from the staged copy of its tree).  Both are called
through store_snapshot on the same System, and the listings of what they
wrote -- groups, dataset paths, element types, shapes and values -- must be
identical, for 1D (Cartesian and spherical) and 2D snapshots.  The
reference's plotting scripts read these paths (e.g. fields/velocity_x,
examples/sod_shock_1d/plot_comparison.py:27).
"""
import ctypes as C
import os
import shutil
import subprocess
import sys

import numpy as np
import pytest

import hydrofv_gb300 as H

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
FAKE = os.path.join(HERE, "hdf5_fake")
sys.path.insert(0, os.path.join(ROOT, "oracle"))
import oracle as O  # noqa: E402

pytestmark = pytest.mark.skipif(shutil.which("gcc") is None, reason="gcc not available")


def _build(tmp, name, sources, includes, defines=()):
    out = os.path.join(tmp, f"lib{name}.so")
    cmd = ["gcc", "-std=gnu99", "-O1", "-shared", "-fPIC", "-include", "time.h", *defines,
           *[f"-I{d}" for d in includes], *sources, os.path.join(FAKE, "fake_hdf5.c"), "-o", out]
    p = subprocess.run(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
    assert p.returncode == 0, p.stdout
    lib = C.CDLL(out)
    lib.store_snapshot.restype = H.ErrorStatus
    lib.store_snapshot.argtypes = [C.POINTER(H.BoundaryConditionParam), C.POINTER(H.System),
                                   C.c_void_p, C.POINTER(H.SimulationStatus), C.POINTER(H.StoringParam)]
    return lib


@pytest.fixture(scope="module")
def writers(tmp_path_factory):
    tmp = str(tmp_path_factory.mktemp("h5writers"))
    host = os.path.join(ROOT, "hydrofv_gb300", "csrc", "host")
    ours = _build(tmp, "ours", [os.path.join(host, "storing.c"), os.path.join(host, "error.c")],
                  [FAKE, os.path.join(ROOT, "include"), host], ["-DHYDRO_WITH_HDF5"])
    ref = None
    if os.path.exists(os.path.join(O.REF_SRC, "storing.c")):
        ref = _build(tmp, "ref", [os.path.join(O.REF_SRC, "storing.c"), os.path.join(O.REF_SRC, "error.c")],
                     [FAKE, O.REF_SRC])
    return ours, ref


def _snapshot(lib, out_dir, coord, coord_flag, nx, ny, g, bc, rng):
    """store_snapshot on a System whose arrays hold seeded values; returns
    the listing the stand-in wrote."""
    s = H.System()
    ctypes_keep = []
    s.coord_sys = coord.encode()
    s.coord_sys_flag_ = coord_flag
    s.gamma = 1.4
    s.x_min, s.x_max = -0.5, 1.25
    s.num_cells_x = nx
    s.num_ghost_cells_side = g
    tot = (nx + 2 * g) * ((ny + 2 * g) if ny else 1)
    s.dx_ = 1.75 / (nx + 2 * g)
    if ny:
        s.y_min, s.y_max = 0.0, 2.0
        s.num_cells_y = ny
        s.dy_ = 2.0 / (ny + 2 * g)
    names = ["density_", "velocity_x_", "velocity_y_", "pressure_"] if ny else ["density_", "velocity_x_",
                                                                               "pressure_"]
    for n in names:
        a = rng.normal(size=tot)
        ctypes_keep.append(a)
        setattr(s, n, a.ctypes.data_as(C.POINTER(C.c_double)))
    bcp = H.BoundaryConditionParam()
    enc = [b.encode() for b in bc]
    ctypes_keep.append(enc)
    bcp.boundary_condition_x_min, bcp.boundary_condition_x_max = enc[0], enc[1]
    if ny:
        bcp.boundary_condition_y_min, bcp.boundary_condition_y_max = enc[2], enc[3]
    st = H.SimulationStatus(123, 0.625, 1.5e-3)
    sp = H.StoringParam()
    d = (out_dir + "/").encode()
    ctypes_keep.append(d)
    sp.is_storing = True
    sp.output_dir = d
    sp.store_count_ = 7
    e = lib.store_snapshot(C.byref(bcp), C.byref(s), None, C.byref(st), C.byref(sp))
    assert e.return_code == 0
    assert sp.store_count_ == 8
    with open(os.path.join(out_dir, "snapshot_7.h5")) as f:
        return f.read().splitlines()


CASES = [
    ("cartesian_1d", 1, 20, 0, 2, ("transmissive", "reflective")),
    ("spherical_1d", 5, 17, 0, 3, ("reflective", "transmissive")),
    ("cartesian_2d", 2, 9, 6, 2, ("periodic", "periodic", "reflective", "transmissive")),
]


@pytest.mark.parametrize("coord,flag,nx,ny,g,bc", CASES, ids=[c[0] for c in CASES])
def test_hdf5_layout_matches_the_reference_writer(writers, tmp_path, coord, flag, nx, ny, g, bc):
    ours, ref = writers
    rng = np.random.default_rng(5)
    d1 = tmp_path / "ours"
    d1.mkdir()
    got = _snapshot(ours, str(d1), coord, flag, nx, ny, g, bc, rng)
    # the layout the reference's plotting scripts read
    paths = {line.split("\t")[0]: line.split("\t")[1] for line in got}
    for p in ("/fields/density", "/fields/velocity_x", "/fields/pressure", "/simulation_status/num_steps",
              "/simulation_status/simulation_time", "/simulation_status/dt", "/parameters/coordinate_system"):
        assert p in paths, p
    assert ("/fields/velocity_y" in paths) == (ny > 0)
    assert paths["/parameters/coordinate_system"] == "vlen_str"
    if ref is None:
        pytest.skip("reference sources not staged (make -C oracle stage)")
    d2 = tmp_path / "ref"
    d2.mkdir()
    want = _snapshot(ref, str(d2), coord, flag, nx, ny, g, bc, np.random.default_rng(5))
    assert got == want
