"""Snapshots of the 2D GPU path (src/storing.c:768-844 semantics).

A snapshot is due when t >= interval * (count - offset + 1).  The default
path copies the materialized state to the host on a side stream and writes
it from a host thread while the steps go on; `sync_snapshots` makes stepping
wait for each write.  Both must produce the same files, and every snapshot
must hold the state the oracle reaches after the same number of steps.
"""
import os

import numpy as np
import pytest

import hydrofv_gb300 as H

pytestmark = pytest.mark.gpu


def read_bin(path):
    with open(path, "rb") as f:
        raw = f.read()
    assert raw[:8] == b"HYDROFV\0"
    dim, nx, ny, g = np.frombuffer(raw, np.int32, 4, 8)
    steps = int(np.frombuffer(raw, np.int64, 1, 24)[0])
    t, dt = np.frombuffer(raw, np.float64, 2, 32)
    n = (nx + 2 * g) * (ny + 2 * g)
    W = np.frombuffer(raw, np.float64, 4 * n, 48).reshape(4, ny + 2 * g, nx + 2 * g)
    return steps, t, dt, W


def run(p, out_dir, sync, interval, tf):
    os.makedirs(out_dir, exist_ok=True)
    return H.run_2d(p.nx, p.ny, p.g, (p.x_min, p.x_max, p.y_min, p.y_max), p.gamma, p.W, p.U,
                    bc=p.bc, slope_limiter=p.slope_limiter, cfl=p.cfl, tf=tf, max_steps=-1,
                    options=H.default_options(sync_snapshots=sync),
                    storing={"interval": interval, "output_dir": out_dir + "/", "store_initial": True})


def test_async_and_sync_snapshots_match_oracle(gpu_available, oracle_mod, tmp_path):
    O = oracle_mod
    p = O.shear_layer(64, steps=-1)
    tf, interval = 0.05, 0.01
    ra = run(p, str(tmp_path / "async"), 0, interval, tf)
    rs = run(p, str(tmp_path / "sync"), 1, interval, tf)
    assert ra.code == 0 and rs.code == 0, (ra.message, rs.message)
    files = sorted(os.listdir(tmp_path / "async"))
    assert files == sorted(os.listdir(tmp_path / "sync"))
    assert len(files) == 6          # initial + one per interval up to tf
    orc = O.load("oracle")
    for f in files:
        a = open(tmp_path / "async" / f, "rb").read()
        assert a == open(tmp_path / "sync" / f, "rb").read(), f
        steps, t, dt, W = read_bin(str(tmp_path / "async" / f))
        if steps == 0:
            assert np.array_equal(W, p.W)
            continue
        q = p.copy()
        if steps == ra.num_steps:       # the last snapshot: the run to tf (clipped last step)
            q.max_steps, q.tf = -1, tf
        else:                           # earlier ones: no clipping happened yet
            q.max_steps, q.tf = steps, 1e300
        ref = orc.run_2d(q)
        assert ref.num_steps == steps and ref.t == t
        assert np.all(O.rel_l1(W, ref.W, p.g) <= 1e-12)
    assert np.all(O.rel_l1(ra.U, rs.U, p.g) == 0.0)


def test_snapshot_write_error_is_reported(gpu_available, oracle_mod, tmp_path):
    """The second snapshot's file name is taken by a directory, so its write
    fails mid-run: the failure comes back as the writer's OS error, in both
    modes (after the run in the asynchronous one)."""
    O = oracle_mod
    p = O.shear_layer(32, steps=-1)
    for sync in (0, 1):
        d = tmp_path / f"blocked{sync}"
        os.makedirs(d / "snapshot_1.bin")
        r = H.run_2d(p.nx, p.ny, p.g, (p.x_min, p.x_max, p.y_min, p.y_max), p.gamma, p.W, p.U,
                     bc=p.bc, slope_limiter=p.slope_limiter, cfl=p.cfl, tf=0.02, max_steps=-1,
                     options=H.default_options(sync_snapshots=sync),
                     storing={"interval": 0.005, "output_dir": str(d) + "/", "store_initial": False})
        assert r.code != 0 and "snapshot" in r.message.lower()


def read_bin_1d(path):
    with open(path, "rb") as f:
        raw = f.read()
    assert raw[:8] == b"HYDROFV\0"
    dim, nx, ny, g = np.frombuffer(raw, np.int32, 4, 8)
    assert dim == 1
    steps = int(np.frombuffer(raw, np.int64, 1, 24)[0])
    t, dt = np.frombuffer(raw, np.float64, 2, 32)
    W = np.frombuffer(raw, np.float64, 3 * (nx + 2 * g), 48).reshape(3, nx + 2 * g)
    return steps, t, dt, W


@pytest.mark.parametrize("integ,solver", [("godunov_first_order_1d", "riemann_solver_exact"),
                                          ("muscl_hancock_1d", "riemann_solver_hllc")])
def test_1d_snapshots_match_oracle(gpu_available, oracle_mod, tmp_path, integ, solver):
    """1D runs stop the cluster kernel when a snapshot is due and relaunch it
    after the host has stored it: every snapshot holds the oracle's state
    after the same number of steps, and storing does not change the run."""
    O = oracle_mod
    p = O.sod_1d(200)
    p.integrator, p.riemann_solver = integ, solver
    tf, interval = 0.2, 0.05
    out = str(tmp_path / "snaps")
    os.makedirs(out)
    args = dict(bc=p.bc, integrator=p.integrator, riemann_solver=p.riemann_solver,
                slope_limiter=p.slope_limiter, cfl=p.cfl, tf=tf, max_steps=-1)
    r = H.run_1d(p.nx, p.g, (p.x_min, p.x_max), p.gamma, p.W, p.U,
                 storing={"interval": interval, "output_dir": out + "/", "store_initial": True}, **args)
    plain = H.run_1d(p.nx, p.g, (p.x_min, p.x_max), p.gamma, p.W, p.U, **args)
    assert r.code == 0 and plain.code == 0, (r.message, plain.message)
    assert r.num_steps == plain.num_steps
    assert np.array_equal(r.U, plain.U) and np.array_equal(r.W, plain.W)
    files = sorted(os.listdir(out))
    assert len(files) == 5          # initial + one per interval up to tf
    orc = O.load("oracle")
    seen = []
    for f in files:
        steps, t, dt, W = read_bin_1d(os.path.join(out, f))
        seen.append(steps)
        if steps == 0:
            assert np.array_equal(W, p.W)
            continue
        q = p.copy()
        if steps == r.num_steps:
            q.max_steps, q.tf = -1, tf
        else:
            q.max_steps, q.tf = steps, 1e300
        ref = orc.run_1d(q)
        assert ref.num_steps == steps and ref.t == t
        scale = np.max(np.abs(ref.W), axis=1, keepdims=True)
        assert np.all(np.abs(W - ref.W) <= 1e-12 * scale)
    assert seen == sorted(seen) and seen[-1] == r.num_steps
