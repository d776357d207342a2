"""Benchmark: 2D MUSCL-Hancock + HLLC cell-updates/s on one GB300.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl gpu|reference]

Workload (one "step" = one time step of the whole grid): the shear layer on
[0,1]^2, 2048 x 2048 interior cells, G = 2, periodic, gamma = 5/3, rho = 2 /
vx = +0.5 for |y-0.5| < 0.25 else rho = 1 / vx = -0.5, p = 2.5,
vy = 0.01 sin(4 pi x), seeded U[-1e-3, 1e-3] noise on vx and vy;
MUSCL-Hancock + HLLC + monotonized-central limiter, CFL 0.8, FP64 (the
drop-in arithmetic).  Default K = 200 steps, W = 5.

value: device-resident cell-updates/s (state already in HBM; the timed K
  steps start from the initial condition after W warm-up steps and a rewind;
  CUDA-event time of the stepping; the 0.74 GB state exceeds the 129 MB L2).
e2e:   the same K steps through hydro_gpu_launch_simulation with the
  caller's host arrays, host->device upload and device->host download of the
  full state inside the timed region (host wall clock).
roofline: the step kernel against measured HBM bandwidth (64 algorithmic
  bytes per cell-update: 4 conserved fields read + 4 written), plus the FP64
  pipe roof measured by hydro_gpu_calibrate, which is the binding one.
cpu_baseline: the CPU implementation of the same step on this host's cores,
  on a bounded sample (the first few steps of the same grid).
forms: the FP32 form of the same steps (L1 error against FP64, its own
  rooflines), and the other configurations, each at its own size and step
  count: the 8192^2 point blast (K steps, FP64 and FP32), the 256-instance
  four-quadrant ensemble (500 steps, FP64 and FP32) and the 1024^2 adjoint
  (400 steps, backward cost, one dot-product and finite-difference check).

Other workloads (--workload): point_blast (8192^2 with --size 8192), ensemble
(256 four-quadrant grids), adjoint (1024^2 shear layer), snapshots, and sod:
the 1000-cell Sod tube, Godunov + exact solver, one "step" = one whole run to
t = 0.2, timed on the device and through the drop-in call, with the serial
CPU implementation timed beside it.

--impl reference times the reference's CPU implementation of the path: the
unmodified reference build (oracle/_ref) where it exists, else this
project's C restatement (oracle/), OpenMP over all host cores.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

N_SIDE = 2048
BYTES_PER_CELL_FP64 = 64
METRIC = "2D MUSCL-HLLC cell-updates/s: FP64 plain vs FP32/batched at stated L1 error"
WORKLOAD = "shear_layer_2048x2048_muscl_hancock_hllc_mc_fp64"


def peaks() -> dict:
    path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(path):
        with open(path) as f:
            d = json.load(f)
        return {"hbm_gbs": d["hbm_gbs"], "source": "measured"}
    return {"hbm_gbs": 6800.0, "source": "fallback"}


def profile_traffic(precision: str = "fp64") -> float | None:
    """DRAM bytes per step launch at 2048^2 from the committed ncu capture
    (profiles/mh2d_fp64_traffic.json; the FP32 form's in mh2d_fp32_counts.json)."""
    if precision == "fp64":
        path = os.path.join(ROOT, "profiles", "mh2d_fp64_traffic.json")
        key = "dram_bytes_per_launch_2048"
    else:
        path = os.path.join(ROOT, "profiles", "mh2d_fp32_counts.json")
        key = "dram_bytes_per_launch"
    if not os.path.exists(path):
        return None
    with open(path) as f:
        d = json.load(f)
    return float(d[key]) if key in d else None


def hbm_roofline(value: float, bytes_per_cell: int, pk: dict, traffic: float | None) -> dict:
    """The step against measured HBM bandwidth: algorithmic bytes (4 conserved
    fields read and written per cell-update) per second."""
    achieved = bytes_per_cell * value / 1e9
    return {"bound": "hbm", "achieved": achieved, "peak": pk["hbm_gbs"], "unit": "GB/s",
            "frac": achieved / pk["hbm_gbs"], "traffic": traffic, "peak_source": pk["source"],
            "bytes_per_cell_update": bytes_per_cell}


def profile_counts(precision: str) -> dict | None:
    """FP-pipe instructions per cell-update of the step kernel (committed ncu
    counts of one launch: profiles/mh2d_fp64_counts.json, mh2d_fp32_counts.json)."""
    path = os.path.join(ROOT, "profiles", f"mh2d_{precision}_counts.json")
    if not os.path.exists(path):
        return None
    with open(path) as f:
        return json.load(f)


class ClockSampler:
    """nvidia-smi sampling of SM clocks and throttle reasons during the timed region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device: int):
        self.device = device
        self.proc = None
        self.fh = None
        self.path = os.path.join(tempfile.gettempdir(), f"hydro_bench_clocks_{os.getpid()}_{id(self)}.csv")

    def __enter__(self):
        try:
            self.fh = open(self.path, "w")
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.device), f"--query-gpu={self.FIELDS}",
                 "--format=csv,noheader,nounits", "-lms", "100"],
                stdout=self.fh, stderr=subprocess.DEVNULL)
            time.sleep(0.3)
        except (OSError, FileNotFoundError):
            self.proc = None
        return self

    def __exit__(self, *exc):
        if self.proc is not None:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()
            self.fh.close()

    def summary(self) -> dict:
        try:
            return self._summary()
        finally:
            if os.path.exists(self.path):
                os.remove(self.path)

    def _summary(self) -> dict:
        if self.proc is None or not os.path.exists(self.path):
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        with open(self.path) as f:
            for line in f:
                parts = [p.strip() for p in line.split(",")]
                if len(parts) < 9:
                    continue
                try:
                    sm.append(float(parts[1]))
                    smax.append(float(parts[2]))
                except ValueError:
                    continue
                for name, val in zip(names, parts[5:9]):
                    if val.lower() == "active":
                        reasons.add(name)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(smax),
                "reasons": sorted(reasons), "samples": len(sm)}


def dist_env():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


def max_over_ranks(x: float, ws: int) -> float:
    if ws <= 1:
        return x
    import torch
    import torch.distributed as dist
    t = torch.tensor([x], dtype=torch.float64)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def barrier(ws: int):
    if ws > 1:
        import torch.distributed as dist
        dist.barrier()


def cpu_sample(steps_hint: int, budget_s: float = 20.0, max_steps: int = 2000) -> dict:
    """Time the CPU implementation on a bounded sample of the same workload:
    the first steps of the same grid, as many as the one-step probe says fit in
    budget_s seconds (the probe's step includes the threads' start-up, so the
    sample takes about two thirds of that), at least steps_hint, at most
    max_steps."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle as O
    if not os.path.exists(os.path.join(O.BUILD, "liboracle.so")):
        O.build(with_reference=False)
    kind = "reference" if O.reference_available() else "port"
    backend = O.load("ref" if kind == "reference" else "oracle")
    threads = O.load("oracle").lib.oracle_num_threads()
    p = O.shear_layer(N_SIDE, steps=1)
    r = backend.run_2d(p)                        # probe: one step
    per_step = max(r.seconds, 1e-3)
    n = int(min(max_steps, max(steps_hint, 2, budget_s / per_step)))
    p = O.shear_layer(N_SIDE, steps=n)
    r = backend.run_2d(p)
    value = N_SIDE * N_SIDE * n / r.seconds
    return {"value": value, "unit": "cell-updates/s", "cores": int(threads), "kind": kind,
            "sample": f"first {n} steps of the {N_SIDE}x{N_SIDE} shear layer "
                      f"({r.seconds:.1f} s, OpenMP {threads} threads)",
            "seconds": r.seconds, "steps": n}


def fp_roofline(prec, value, fp64_tflops, fp32_tflops, H, workload="shear_layer",
                sms: int = 0, sm_mhz: float = 0.0) -> dict:
    """The binding roof of the step kernel beyond HBM.

    FP64 form: its FP64 pipe.  achieved = FP64 warp instructions issued per
    second (ncu count per cell-update x measured cell-updates/s); peak = the
    FP64 FMA rate hydro_gpu_calibrate measures in the same run, as warp
    instructions per second (one warp instruction takes one pipe slot per
    lane).  FP32 form: instruction issue, which binds it (its FP32 pipe is
    far from busy).  achieved = all warp instructions per second; peak = 4
    per SM per clock at the SM clock sampled during the timed region.  Each
    carries the other figure beside it."""
    fp64 = prec == H.PRECISION_FP64
    name = "fp64" if fp64 else "fp32"
    out = {"bound": "fp64_pipe" if fp64 else "issue", "peak_tflops_fp64": fp64_tflops,
           "peak_tflops_fp32": fp32_tflops}
    counts = profile_counts(name)
    if not (counts and workload == "shear_layer" and N_SIDE == 2048):
        return out
    per_cell = counts[f"{name}_warp_inst_per_cell_update"]
    pipe_achieved = value * per_cell
    pipe_peak = (fp64_tflops if fp64 else fp32_tflops) * 1e12 / 2 / 32
    pipe = {"achieved": pipe_achieved, "peak": pipe_peak, "unit": f"{name.upper()} warp instructions/s",
            "frac": pipe_achieved / pipe_peak, "of": "measured (hydro_gpu_calibrate)"}
    issue = None
    all_per_cell = counts.get("warp_inst_per_cell_update_all_pipes")
    if all_per_cell and sms > 0 and sm_mhz > 0:
        ia, ip = value * all_per_cell, 4.0 * sms * sm_mhz * 1e6
        issue = {"achieved": ia, "peak": ip, "unit": "warp instructions/s", "frac": ia / ip,
                 "of": f"4 per SM per clock, {sms} SMs at the sampled {sm_mhz:.0f} MHz",
                 "warp_inst_per_cell_update": all_per_cell}
    if fp64:
        out.update(pipe)
        if issue:
            out["issue"] = issue
    else:
        if issue:
            out.update(issue)
        out[f"{name}_pipe"] = pipe
    out.update({f"{name}_warp_inst_per_cell_update": per_cell,
                f"{name}_thread_inst_per_cell_update": counts[f"{name}_thread_inst_per_cell_update"],
                "issue_active_pct": counts.get("issue_active_pct"),
                "counts_source": counts["source"]})
    return out


def shear_config(args, ws: int) -> dict:
    """config of the headline line; the reference arm prints the same dict."""
    return {"workload": WORKLOAD, "grid": [N_SIDE, N_SIDE], "ghost_cells": 2,
            "limiter": "monotonized_central", "cfl": 0.8, "boundaries": "periodic",
            "steps_per_run": args.steps,
            "l2": "state larger than the 129 MB L2 (no flush needed)" if N_SIDE * N_SIDE >= 1 << 20
                  else "state fits in L2 (profiling size)",
            "parallelism": "replicas" if ws > 1 else "single"}


BLAST_SIDE = 8192


def blast_leg(args, H, device: int, ws: int) -> dict:
    """The precision study's grid: the 8192^2 point blast (Van Leer,
    reflective, CFL 0.4), FP64 and FP32 over the line's K steps from the
    initial condition (W warm-up steps and a rewind first), CUDA-event time
    of the stepping; relative L1 error of the FP32 state against the FP64
    state per field, and the conserved-total drift of both."""
    from hydrofv_gb300.problems import point_blast
    p = point_blast(BLAST_SIDE, steps=args.steps)
    cells = p.nx * p.ny
    out, finals = {}, {}
    for name, prec in (("fp64", H.PRECISION_FP64), ("fp32", H.PRECISION_FP32)):
        with H.Solver2D(p.nx, p.ny, p.g, (p.x_min, p.x_max, p.y_min, p.y_max), p.gamma, p.W, p.U,
                        bc=p.bc, slope_limiter=p.slope_limiter, cfl=p.cfl,
                        options=H.default_options(device=device, precision=prec)) as s:
            s.advance(args.warmup)
            s.restart()
            tot0 = s.conserved_totals()
            l0 = s.kernel_launches()
            barrier(ws)
            clk = ClockSampler(device)
            with clk:
                st, ms = s.advance(args.steps)
            launches = s.kernel_launches() - l0
            assert st.num_steps == args.steps, st.num_steps
            tot1 = s.conserved_totals()
            finals[name] = s.download()[0]
        ms = max_over_ranks(ms, ws)
        drift = (tot1 - tot0) / np.where(tot0 != 0, np.abs(tot0), 1.0)
        out[name] = {"value": ws * cells * args.steps / (ms * 1e-3), "ms_per_step": ms / args.steps,
                     "gpu_launches": int(launches), "clocks": clk.summary(),
                     "conserved_drift": {"mass": float(drift[0]), "energy": float(drift[3])}}
    g = p.g
    W64, W32 = finals["fp64"], finals["fp32"]
    num = np.abs(W32[:, g:-g, g:-g] - W64[:, g:-g, g:-g]).sum(axis=(1, 2))
    den = np.abs(W64[:, g:-g, g:-g]).sum(axis=(1, 2))
    l1 = num / den
    out["fp32"]["speedup_vs_fp64"] = out["fp32"]["value"] / out["fp64"]["value"]
    out["fp32"]["rel_l1_vs_fp64"] = {"density": float(l1[0]), "velocity_x": float(l1[1]),
                                     "velocity_y": float(l1[2]), "pressure": float(l1[3])}
    out["config"] = {"workload": f"point_blast_{BLAST_SIDE}x{BLAST_SIDE}_muscl_hancock_hllc_vl",
                     "grid": [BLAST_SIDE, BLAST_SIDE], "ghost_cells": p.g, "limiter": p.slope_limiter,
                     "cfl": p.cfl, "boundaries": p.bc[0], "steps_per_run": args.steps,
                     "l2": "state larger than the 129 MB L2 (no flush needed)"}
    return out


ENSEMBLE_STEPS = 500
ADJOINT_SIDE, ADJOINT_STEPS, ADJOINT_K = 1024, 400, 50


def ensemble_leg(args, H, device: int, ws: int) -> dict:
    """The batched-ensemble configuration beside the headline: 256
    four-quadrant problems (sides log-uniform in [128, 1024], minmod,
    transmissive, CFL 0.8, per-instance dt), 500 steps each, one launch per
    step for the whole batch, FP64 and FP32 on the same instances (W
    warm-up steps and a rewind first); relative L1 of the FP32 state against
    FP64 over all instances."""
    from hydrofv_gb300.problems import four_quadrant_ensemble
    probs = four_quadrant_ensemble(count=256, steps=ENSEMBLE_STEPS)
    cells = sum(p.nx * p.ny for p in probs)
    out, finals = {}, {}
    for name, prec in (("fp64", H.PRECISION_FP64), ("fp32", H.PRECISION_FP32)):
        with H.Batch2D(probs, options=H.default_options(device=device, precision=prec)) as b:
            b.advance(args.warmup)
            b.restart()
            l0 = b.kernel_launches()
            barrier(ws)
            clk = ClockSampler(device)
            with clk:
                st, ms = b.advance(ENSEMBLE_STEPS)
            launches = b.kernel_launches() - l0
            assert all(x[0] == ENSEMBLE_STEPS for x in st)
            finals[name] = b.download()
        ms = max_over_ranks(ms, ws)
        out[name] = {"value": ws * cells * ENSEMBLE_STEPS / (ms * 1e-3), "ms_per_step": ms / ENSEMBLE_STEPS,
                     "gpu_launches": int(launches), "clocks": clk.summary()}
    num = np.zeros(4)
    den = np.zeros(4)
    for (W64, _), (W32, _), p in zip(finals["fp64"], finals["fp32"], probs):
        g = p.g
        num += np.abs(W32[:, g:-g, g:-g] - W64[:, g:-g, g:-g]).sum(axis=(1, 2))
        den += np.abs(W64[:, g:-g, g:-g]).sum(axis=(1, 2))
    l1 = num / den
    out["fp32"]["speedup_vs_fp64"] = out["fp32"]["value"] / out["fp64"]["value"]
    out["fp32"]["rel_l1_vs_fp64"] = {"density": float(l1[0]), "velocity_x": float(l1[1]),
                                     "velocity_y": float(l1[2]), "pressure": float(l1[3])}
    out["config"] = {"workload": "ensemble_256x_four_quadrant", "instances": 256, "interior_cells": cells,
                     "limiter": "minmod", "cfl": 0.8, "boundaries": "transmissive",
                     "steps_per_instance": ENSEMBLE_STEPS}
    return out


def adjoint_leg(args, H, device: int) -> dict:
    """The discrete-adjoint configuration beside the headline: the 1024^2
    shear layer (MC, periodic), 400 steps, a checkpoint every 50; forward
    pass, then dJ/dW0 for J = sum_{x > 0.5} rho^2 V (segment recomputation +
    reverse sweep), device times; one seeded direction in (rho, p) checked
    by the dot-product test against the tangent-linear model and by central
    differences (eps 1e-6) of the branch-frozen replay."""
    import math
    from hydrofv_gb300.problems import right_half_density_squared, shear_layer
    p = shear_layer(ADJOINT_SIDE, steps=ADJOINT_STEPS)
    interior = np.zeros(p.W.shape[1:], dtype=bool)
    interior[p.g:-p.g, p.g:-p.g] = True

    def dot(a, b):
        return math.fsum((a[:, interior] * b[:, interior]).ravel())

    with H.Adjoint2D(p, steps=ADJOINT_STEPS, checkpoint_every=ADJOINT_K,
                     options=H.default_options(device=device)) as ad:
        WN = ad.forward()                      # warm-up pass
        J, seed = right_half_density_squared(p, WN)
        ad.backward(seed)
        WN = ad.forward()
        st_f = ad.stats()
        J, seed = right_half_density_squared(p, WN)
        grad = ad.backward(seed)
        st = ad.stats()
        back_ms = st["recompute_ms"] + st["vjp_ms"]
        rng = np.random.default_rng(2024)
        d = np.zeros_like(p.W)
        d[0] = rng.normal(size=d[0].shape) * np.abs(p.W[0])
        d[3] = rng.normal(size=d[3].shape) * np.abs(p.W[3])
        d[:, ~interior] = 0.0
        an = dot(grad, d)
        _, dwN = ad.tangent(d)
        eps = 1e-6
        jp = right_half_density_squared(p, ad.replay_frozen(p.W + eps * d))[0]
        jm = right_half_density_squared(p, ad.replay_frozen(p.W - eps * d))[0]
    cells = p.nx * p.ny
    return {"forward_ms": st_f["forward_ms"],
            "forward_cell_updates_per_s": cells * ADJOINT_STEPS / (st_f["forward_ms"] * 1e-3),
            "backward_ms": back_ms, "backward_vs_forward": back_ms / st_f["forward_ms"],
            "recompute_mismatches": st["recompute_mismatches"],
            "dot_product_rel": abs(dot(seed, dwN) - an) / abs(an),
            "fd_frozen_rel": abs((jp - jm) / (2 * eps) - an) / abs(an), "eps": eps,
            "config": {"workload": f"adjoint_shear_layer_{ADJOINT_SIDE}x{ADJOINT_SIDE}_mc_fp64",
                       "steps": ADJOINT_STEPS, "checkpoint_every": ADJOINT_K,
                       "objective": "sum_{x>0.5} rho^2 V at step N", "directions": 1}}


def run_reference_arm(args) -> None:
    ws, rank, _ = dist_env()
    if rank != 0:
        return
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle as O
    if not os.path.exists(os.path.join(O.BUILD, "liboracle.so")):
        O.build(with_reference=False)
    kind = "reference" if O.reference_available() else "port"
    backend = O.load("ref" if kind == "reference" else "oracle")
    threads = O.load("oracle").lib.oracle_num_threads()
    # warm-up: W steps, then K timed steps from the initial condition
    warm = O.shear_layer(N_SIDE, steps=args.warmup)
    backend.run_2d(warm)
    p = O.shear_layer(N_SIDE, steps=args.steps)
    r = backend.run_2d(p)
    value = N_SIDE * N_SIDE * args.steps / r.seconds
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": "cell-updates/s",
        "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": r.seconds * 1e3 / args.steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": shear_config(args, ws),
        "cpu_baseline": {"value": value, "unit": "cell-updates/s", "cores": int(threads),
                         "kind": kind,
                         "sample": f"{args.steps} steps of the {N_SIDE}x{N_SIDE} shear layer, "
                                   f"OpenMP {threads} threads"},
        "e2e": {"value": value, "unit": "cell-updates/s", "h2d_bytes_per_step": 0,
                "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line))


def run_ensemble(args, H, device, ws, rank) -> None:
    """Batched ensemble: every instance steps args.steps times, one launch per
    step for the whole batch, FP64 and FP32 on the same instances."""
    from hydrofv_gb300.problems import four_quadrant_ensemble
    probs = four_quadrant_ensemble(count=args.instances, steps=args.steps)
    cells = sum(p.nx * p.ny for p in probs)
    res = {}
    finals = {}
    for name, prec in (("fp64", H.PRECISION_FP64), ("fp32", H.PRECISION_FP32)):
        opts = H.default_options(device=device, precision=prec, autotune=1 if args.autotune else 0)
        with H.Batch2D(probs, options=opts) as b:
            b.advance(args.warmup)
            b.restart()
            l0 = b.kernel_launches()
            barrier(ws)
            clk = ClockSampler(device)
            with clk:
                st, ms = b.advance(args.steps)
            launches = b.kernel_launches() - l0
            assert all(s[0] == args.steps for s in st)
            finals[name] = b.download()
        ms = max_over_ranks(ms, ws)
        res[name] = {"value": ws * cells * args.steps / (ms * 1e-3), "ms_per_step": ms / args.steps,
                     "gpu_launches": int(launches), "clocks": clk.summary()}
    num = np.zeros(4)
    den = np.zeros(4)
    for (W64, _), (W32, _), p in zip(finals["fp64"], finals["fp32"], probs):
        g = p.g
        num += np.abs(W32[:, g:-g, g:-g] - W64[:, g:-g, g:-g]).sum(axis=(1, 2))
        den += np.abs(W64[:, g:-g, g:-g]).sum(axis=(1, 2))
    l1 = num / den
    if rank != 0:
        return
    main_form = "fp32" if args.precision == "fp32" else "fp64"
    r = res[main_form]
    pk = peaks()
    bpc = BYTES_PER_CELL_FP64 if main_form == "fp64" else BYTES_PER_CELL_FP64 // 2
    achieved = bpc * r["value"] / ws / 1e9
    line = {
        "metric": METRIC, "value": r["value"], "unit": "cell-updates/s", "n_gpus": ws,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": r["ms_per_step"],
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f64" if main_form == "fp64" else "f32",
        "data": "synthetic (seeded four-quadrant ensemble)",
        "config": {"workload": f"ensemble_{args.instances}x_four_quadrant_{main_form}",
                   "instances": args.instances, "interior_cells": cells,
                   "sides": [int(p.nx) for p in probs][:8] + ["..."],
                   "limiter": "minmod", "cfl": 0.8, "boundaries": "transmissive",
                   "steps_per_instance": args.steps, "autotune": bool(args.autotune)},
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": pk["hbm_gbs"], "unit": "GB/s",
                     "frac": achieved / pk["hbm_gbs"], "traffic": None, "peak_source": pk["source"],
                     "bytes_per_cell_update": bpc},
        "forms": {"fp64": res["fp64"],
                  "fp32": dict(res["fp32"], speedup_vs_fp64=res["fp32"]["value"] / res["fp64"]["value"],
                               rel_l1_vs_fp64={"density": l1[0], "velocity_x": l1[1],
                                               "velocity_y": l1[2], "pressure": l1[3]})},
        "gpu_launches": r["gpu_launches"],
        "clocks": r["clocks"],
    }
    print(json.dumps(line))


def adjoint_checks(ad, p, seed, grad, n_dirs: int, rng_seed: int = 2024) -> dict:
    """Checks of dJ/dW0 on n_dirs seeded random directions in (rho, p): the
    dot-product test against the tangent-linear model, central differences
    (eps 1e-6) of the branch-frozen replay, and of the free replay (dt
    frozen, branches free) with the number of steps whose branch signature
    flipped under either perturbation."""
    import math
    interior = np.zeros(p.W.shape[1:], dtype=bool)
    interior[p.g:-p.g, p.g:-p.g] = True

    def dot(a, b):
        return math.fsum((a[:, interior] * b[:, interior]).ravel())

    from hydrofv_gb300.problems import right_half_density_squared
    checks = {"dot_product_rel": [], "fd_frozen_rel": [], "fd_free_rel": [], "fd_free_flipped_steps": []}
    rng = np.random.default_rng(rng_seed)
    _, base_sig = ad.replay(p.W) if n_dirs else (None, None)
    eps = 1e-6
    for _ in range(n_dirs):
        d = np.zeros_like(p.W)
        d[0] = rng.normal(size=d[0].shape) * np.abs(p.W[0])
        d[3] = rng.normal(size=d[3].shape) * np.abs(p.W[3])
        d[:, ~interior] = 0.0
        an = dot(grad, d)
        _, dwN = ad.tangent(d)
        checks["dot_product_rel"].append(abs(dot(seed, dwN) - an) / abs(an))
        jp = right_half_density_squared(p, ad.replay_frozen(p.W + eps * d))[0]
        jm = right_half_density_squared(p, ad.replay_frozen(p.W - eps * d))[0]
        checks["fd_frozen_rel"].append(abs((jp - jm) / (2 * eps) - an) / abs(an))
        Wp, sp = ad.replay(p.W + eps * d)
        Wm, sm = ad.replay(p.W - eps * d)
        fd = (right_half_density_squared(p, Wp)[0] - right_half_density_squared(p, Wm)[0]) / (2 * eps)
        checks["fd_free_rel"].append(abs(fd - an) / abs(an))
        checks["fd_free_flipped_steps"].append(int(((sp != base_sig) | (sm != base_sig)).sum()))
    # the free map's central differences against eps on the first two
    # directions: where the error does not shrink with eps, the map jumps
    # (Riemann regime switches of the star-pressure guess), not only kinks
    rng = np.random.default_rng(rng_seed)
    by_eps = {}
    for k in range(min(2, n_dirs)):
        d = np.zeros_like(p.W)
        d[0] = rng.normal(size=d[0].shape) * np.abs(p.W[0])
        d[3] = rng.normal(size=d[3].shape) * np.abs(p.W[3])
        d[:, ~interior] = 0.0
        an = dot(grad, d)
        for e in (1e-6, 1e-8, 1e-10):
            Wp, sp = ad.replay(p.W + e * d)
            Wm, sm = ad.replay(p.W - e * d)
            fd = (right_half_density_squared(p, Wp)[0] - right_half_density_squared(p, Wm)[0]) / (2 * e)
            by_eps.setdefault(f"{e:.0e}", []).append(
                {"rel": abs(fd - an) / abs(an), "flipped_steps": int(((sp != base_sig) | (sm != base_sig)).sum())})
    checks["fd_free_by_eps"] = by_eps
    unflipped = [r for r, f in zip(checks["fd_free_rel"], checks["fd_free_flipped_steps"]) if f == 0]
    checks["fd_free_rel_max_unflipped"] = max(unflipped) if unflipped else None
    checks["directions_unflipped"] = len(unflipped)
    checks["eps"] = eps
    checks["directions"] = n_dirs
    return checks


def run_adjoint(args, H, device, ws, rank) -> None:
    """Discrete adjoint of the shear layer (MC, periodic, FP64): forward pass
    with checkpoints, then the reverse pass (segment recomputation + reverse
    sweep) for dJ/dW0, J = sum_{x > 0.5} rho^2 V at the last step.  Checks
    on --fd-directions seeded random directions (adjoint_checks).  The same
    checks run on a differentiable variant of the state: rho and p carry
    seeded relative noise of amplitude --rho-p-noise, so no limiter of those
    fields sits at its a = b = 0 kink and the free map has a derivative."""
    from hydrofv_gb300.problems import right_half_density_squared, shear_layer
    side = args.size if args.size != 2048 else 1024
    steps = args.steps
    K = args.checkpoint_every
    p = shear_layer(side, steps=steps)
    cells = p.nx * p.ny
    opts = H.default_options(device=device)

    with H.Adjoint2D(p, steps=steps, checkpoint_every=K, options=opts) as ad:
        for _ in range(max(1, args.warmup // 3)):
            WN = ad.forward()
            J, seed = right_half_density_squared(p, WN)
            ad.backward(seed)
        barrier(ws)
        WN = ad.forward()
        st_f = ad.stats()
        J, seed = right_half_density_squared(p, WN)
        l0 = st_f["kernel_launches"]
        clk = ClockSampler(device)
        with clk:
            t0 = time.perf_counter()
            grad = ad.backward(seed)
            wall = time.perf_counter() - t0
        st = ad.stats()
        launches = st["kernel_launches"] - l0
        back_ms = st["recompute_ms"] + st["vjp_ms"]
        checks = adjoint_checks(ad, p, seed, grad, args.fd_directions)
        st_all = ad.stats()
    variant = None
    if args.rho_p_noise > 0.0 and args.fd_directions > 0:
        q = shear_layer(side, steps=steps, rho_p_noise=args.rho_p_noise)
        with H.Adjoint2D(q, steps=steps, checkpoint_every=K, options=opts) as ad:
            WN = ad.forward()
            Jq, seed_q = right_half_density_squared(q, WN)
            grad_q = ad.backward(seed_q)
            stq = ad.stats()
            variant = {"rho_p_noise": args.rho_p_noise, "J": Jq,
                       "backward_vs_forward": (stq["recompute_ms"] + stq["vjp_ms"]) / stq["forward_ms"],
                       "checks": adjoint_checks(ad, q, seed_q, grad_q, args.fd_directions)}
    if rank != 0:
        return
    line = {
        "metric": "discrete adjoint of the 2D MUSCL-HLLC step: cell-steps/s of the reverse pass",
        "value": ws * cells * steps / (back_ms * 1e-3), "unit": "cell-steps/s", "n_gpus": ws,
        "steps": steps, "warmup": args.warmup, "ms_per_step": back_ms / steps,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
        "data": "synthetic (seeded shear layer)",
        "config": {"workload": f"adjoint_shear_layer_{side}x{side}_mc_fp64", "grid": [side, side],
                   "steps": steps, "checkpoint_every": K, "objective": "sum_{x>0.5} rho^2 V at step N",
                   "gradient_of": "initial rho and p (all four primitives returned)",
                   "l2": "state larger than the 129 MB L2" if cells >= 1 << 20 else "fits in L2"},
        "forward": {"ms": st_f["forward_ms"], "ms_per_step": st_f["forward_ms"] / steps,
                    "cell_updates_per_s": cells * steps / (st_f["forward_ms"] * 1e-3)},
        "backward": {"ms": back_ms, "recompute_ms": st["recompute_ms"], "reverse_sweep_ms": st["vjp_ms"],
                     "cost_vs_forward": back_ms / st_f["forward_ms"],
                     "reverse_sweep_vs_forward": st["vjp_ms"] / st_f["forward_ms"],
                     "recompute_mismatches": st["recompute_mismatches"],
                     "device_bytes": st_all["device_bytes"]},
        "checks": dict(checks, tangent_ms=st_all["tangent_ms"], replay_ms=st_all["replay_ms"]),
        "differentiable_variant": variant,
        "e2e": {"value": ws * cells * steps / wall, "unit": "cell-steps/s",
                "h2d_bytes_per_step": 4 * p.W[0].size * 8 / steps,
                "d2h_bytes_per_step": 4 * p.W[0].size * 8 / steps,
                "note": "hydro_gpu_adjoint_backward with host seed in and host gradient out"},
        "gpu_launches": int(launches),
        "clocks": clk.summary(),
    }
    print(json.dumps(line))


def run_snapshots(args, H, device, ws, rank) -> None:
    """Snapshot overlap: the config-2 shear layer through the drop-in call with
    a snapshot every ~10 steps, written synchronously (stepping waits for each
    file) and asynchronously (side-stream copy, host-thread writer).  Wall
    clock of the whole call; the files are identical."""
    import shutil
    import tempfile
    from hydrofv_gb300.problems import shear_layer
    side = args.size
    p = shear_layer(side, steps=-1)
    cells = p.nx * p.ny
    # dt of the first steps (CFL 0.8 after the 10 shrunk steps) sets the interval
    with H.Solver2D(p.nx, p.ny, p.g, (0, 1, 0, 1), p.gamma, p.W, p.U, bc=p.bc,
                    slope_limiter=p.slope_limiter, cfl=p.cfl,
                    options=H.default_options(device=device)) as s:
        st, _ = s.advance(20)
        dt = st.dt
    steps = args.steps
    tf = st.t + (steps - 20) * dt
    interval = tf / max(1, steps // 10)
    res = {}
    root = tempfile.mkdtemp(prefix="hydro_snap_", dir=os.environ.get("HYDRO_SNAPSHOT_DIR", None))
    try:
        for name, sync in (("sync", 1), ("async", 0)):
            out = os.path.join(root, name) + "/"
            os.makedirs(out, exist_ok=True)
            with H.Simulation2D(p.nx, p.ny, p.g, (0, 1, 0, 1), p.gamma, p.W, p.U, bc=p.bc,
                                slope_limiter=p.slope_limiter, cfl=p.cfl, tf=tf, max_steps=-1,
                                options=H.default_options(device=device, sync_snapshots=sync),
                                storing={"interval": interval, "output_dir": out,
                                         "store_initial": False}) as sim:
                t0 = time.perf_counter()
                code, msg, st, _ = sim.launch()
                wall = time.perf_counter() - t0
            assert code == 0, msg
            files = sorted(os.listdir(out))
            res[name] = {"seconds": wall, "steps": st.num_steps, "snapshots": len(files),
                         "cell_updates_per_s": cells * st.num_steps / wall,
                         "bytes_per_snapshot": os.path.getsize(out + files[0]) if files else 0}
        same = all(open(os.path.join(root, "sync", f), "rb").read() == open(os.path.join(root, "async", f), "rb").read()
                   for f in sorted(os.listdir(os.path.join(root, "sync"))))
    finally:
        shutil.rmtree(root, ignore_errors=True)
    if rank != 0:
        return
    line = {
        "metric": "2D MUSCL-HLLC cell-updates/s with snapshots (drop-in call, wall clock)",
        "value": res["async"]["cell_updates_per_s"], "unit": "cell-updates/s", "n_gpus": ws,
        "steps": res["async"]["steps"], "warmup": 0, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded shear layer)",
        "config": {"workload": f"snapshots_shear_layer_{side}x{side}_fp64", "snapshot_interval": interval,
                   "tf": tf},
        "sync": res["sync"], "async": res["async"],
        "speedup_async_vs_sync": res["sync"]["seconds"] / res["async"]["seconds"],
        "files_identical": same,
    }
    print(json.dumps(line))


def run_sod(args, H, device, ws, rank) -> None:
    """The Sod tube (1000 cells, Godunov first order + exact solver, CFL 0.9,
    t = 0.2: 496 time steps) through the drop-in call.  One "step" here is one
    whole run: a latency workload, reported as time per run and as
    cell-updates/s (cells x time steps per second).  value: the device time of
    the stepping (CUDA events inside the call); e2e: the wall clock of the
    call with the host arrays (upload, stepping, download).  cpu_baseline:
    the serial CPU implementation (the reference's 1D OpenMP loops race, so
    the serial build is the one to compare with)."""
    from hydrofv_gb300.problems import sod_1d
    p = sod_1d(1000)
    opts = H.default_options(device=device)

    def run():
        return H.run_1d(p.nx, p.g, (p.x_min, p.x_max), p.gamma, p.W, p.U, bc=p.bc,
                        integrator=p.integrator, riemann_solver=p.riemann_solver,
                        slope_limiter=p.slope_limiter, cfl=p.cfl, tf=p.tf, max_steps=-1,
                        options=opts)

    for _ in range(args.warmup):
        r = run()
        assert r.code == 0, r.message
    barrier(ws)
    walls, device_ms, launches = [], [], 0
    clk = ClockSampler(device)
    with clk:
        for _ in range(args.steps):
            t0 = time.perf_counter()
            r = run()
            walls.append(time.perf_counter() - t0)
            assert r.code == 0, r.message
            device_ms.append(r.stats["step_ms"])
            launches += int(r.stats["kernel_launches"])
    steps = r.num_steps
    dev_s = max_over_ranks(statistics.median(device_ms) * 1e-3, ws)
    wall_s = max_over_ranks(statistics.median(walls), ws)
    if rank != 0:
        return
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle as O
    if not os.path.exists(os.path.join(O.BUILD, "liboracle.so")):
        O.build(with_reference=False)
    orc = O.load("oracle")
    kind = "reference" if O.reference_available() else "port"
    cpu = O.load("ref_serial") if kind == "reference" else orc
    ref = orc.run_1d(p)
    max_rel = float(np.max(np.abs(r.U - ref.U)) / np.max(np.abs(ref.U)))
    cpu_s = []
    budget = time.perf_counter() + 10.0
    while len(cpu_s) < 3 or (time.perf_counter() < budget and len(cpu_s) < 50):
        cpu_s.append(cpu.run_1d(p).seconds)
    cpu_run = statistics.median(cpu_s)
    cells_steps = p.nx * steps
    line = {
        "metric": "1D Godunov + exact Riemann solver: time per Sod run (cell-updates/s)",
        "value": ws * cells_steps / dev_s, "unit": "cell-updates/s", "n_gpus": ws,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": dev_s * 1e3,
        "ms_per_run_device": dev_s * 1e3, "ms_per_run_e2e": wall_s * 1e3,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
        "data": "synthetic (Sod tube, the reference example's initial states)",
        "config": {"workload": "sod_1000_godunov_first_order_exact_fp64", "cells": p.nx,
                   "ghost_cells": p.g, "cfl": p.cfl, "tf": p.tf, "time_steps_per_run": steps,
                   "step": "one whole run to t = 0.2"},
        "e2e": {"value": ws * cells_steps / wall_s, "unit": "cell-updates/s",
                "h2d_bytes_per_step": int(r.stats["h2d_bytes"]),
                "d2h_bytes_per_step": int(r.stats["d2h_bytes"]),
                "note": "one hydro_gpu_launch_simulation call per run, host arrays in and out"},
        "cpu_baseline": {"value": cells_steps / cpu_run, "unit": "cell-updates/s", "cores": 1,
                         "kind": kind, "ms_per_run": cpu_run * 1e3,
                         "sample": f"{len(cpu_s)} whole runs, serial"},
        "max_rel_diff_U_vs_oracle": max_rel,
        "gpu_launches": launches,
        "clocks": clk.summary(),
    }
    print(json.dumps(line))


def main() -> None:
    global N_SIDE, WORKLOAD
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=200)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="gpu", choices=["gpu", "reference"])
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-blast", action="store_true",
                    help="leave out the other configurations of the default line (the 8192^2 point "
                         "blast, the 256-instance ensemble and the 1024^2 adjoint; profiling runs)")
    ap.add_argument("--size", type=int, default=N_SIDE,
                    help="grid side (the headline workload is 2048; smaller sizes are for profiling)")
    ap.add_argument("--precision", default="fp64", choices=["fp64", "fp32"],
                    help="state precision of the timed path (fp64 is the drop-in)")
    ap.add_argument("--workload", default="shear_layer",
                    choices=["shear_layer", "point_blast", "ensemble", "adjoint", "snapshots", "sod"],
                    help="shear_layer: MC, periodic, CFL 0.8; point_blast: Van Leer, reflective, "
                         "CFL 0.4; ensemble: 256 four-quadrant problems, side log-uniform in "
                         "[128, 1024], minmod, transmissive, one launch per step for all; "
                         "sod: the 1000-cell Sod tube, Godunov + exact solver, one step = one run")
    ap.add_argument("--instances", type=int, default=256, help="ensemble size")
    ap.add_argument("--checkpoint-every", type=int, default=50, help="adjoint checkpoint interval")
    ap.add_argument("--fd-directions", type=int, default=2,
                    help="adjoint: random directions checked by dot product and finite differences")
    ap.add_argument("--rho-p-noise", type=float, default=1e-3,
                    help="adjoint: relative noise on rho and p of the differentiable variant (0: none)")
    ap.add_argument("--autotune", action="store_true",
                    help="let the library time work-item shapes before stepping")
    ap.add_argument("--compare", action="store_true",
                    help="also run the other precision on the same steps and report the relative "
                         "L1 error per field and the conserved-total drift of both")
    args = ap.parse_args()
    args.warmup = max(args.warmup, 3)
    if args.size != N_SIDE:
        N_SIDE = args.size
        WORKLOAD = WORKLOAD.replace("2048x2048", f"{N_SIDE}x{N_SIDE}")

    ws, rank, local = dist_env()
    if ws > 1:
        import torch.distributed as dist
        dist.init_process_group("gloo")
    if args.impl == "reference":
        run_reference_arm(args)
        return

    import hydrofv_gb300 as H
    if not os.path.exists(H.LIB_PATH):
        from hydrofv_gb300 import build as B
        B.build()
    from hydrofv_gb300.problems import point_blast, shear_layer
    if args.workload == "ensemble":
        run_ensemble(args, H, local, ws, rank)
        return
    if args.workload == "adjoint":
        run_adjoint(args, H, local, ws, rank)
        return
    if args.workload == "snapshots":
        run_snapshots(args, H, local, ws, rank)
        return
    if args.workload == "sod":
        run_sod(args, H, local, ws, rank)
        return

    device = local
    prec = H.PRECISION_FP32 if args.precision == "fp32" else H.PRECISION_FP64
    make = shear_layer if args.workload == "shear_layer" else point_blast
    p = make(N_SIDE, steps=args.steps)
    bounds = (p.x_min, p.x_max, p.y_min, p.y_max)
    cells = p.nx * p.ny
    bytes_per_cell = BYTES_PER_CELL_FP64 if prec == H.PRECISION_FP64 else BYTES_PER_CELL_FP64 // 2

    def session(precision):
        return H.Solver2D(p.nx, p.ny, p.g, bounds, p.gamma, p.W, p.U, bc=p.bc,
                          slope_limiter=p.slope_limiter, cfl=p.cfl,
                          options=H.default_options(device=device, precision=precision))

    def timed_run(precision, sampler=None):
        """W warm-up steps, rewind, K timed steps; returns (ms, launches, W, U, drift)."""
        with session(precision) as s:
            s.advance(args.warmup)
            s.restart()
            tot0 = s.conserved_totals()
            l0 = s.kernel_launches()
            barrier(ws)
            if sampler is not None:
                with sampler:
                    st, ms = s.advance(args.steps)
            else:
                st, ms = s.advance(args.steps)
            launches = s.kernel_launches() - l0
            assert st.num_steps == args.steps, st.num_steps
            tot1 = s.conserved_totals()
            W, U = s.download()
        drift = ((tot1 - tot0) / np.where(tot0 != 0, np.abs(tot0), 1.0)).tolist()
        return ms, launches, W, U, {"mass": drift[0], "energy": drift[3]}

    # ---- device-resident value ----
    clk = ClockSampler(device)
    step_ms, launches, W_main, U_main, drift_main = timed_run(prec, clk)
    step_ms = max_over_ranks(step_ms, ws)
    value = ws * cells * args.steps / (step_ms * 1e-3)

    # ---- the other precision on the same steps: L1 error of the FP32 form ----
    other = H.PRECISION_FP32 if prec == H.PRECISION_FP64 else H.PRECISION_FP64
    ms_o, _, W_o, U_o, drift_o = timed_run(other)
    W64, W32 = (W_main, W_o) if prec == H.PRECISION_FP64 else (W_o, W_main)
    g = p.g
    l1 = (np.abs(W32[:, g:-g, g:-g] - W64[:, g:-g, g:-g]).sum(axis=(1, 2))
          / np.abs(W64[:, g:-g, g:-g]).sum(axis=(1, 2)))
    del W_main, U_main, W_o, U_o

    # ---- end to end through the drop-in call (host arrays in and out) ----
    # The System and parameter structs are set up outside the timed region, as
    # a program calling the reference API holds them; the timed region is the
    # hydro_gpu_launch_simulation call: upload, steps, download.  Three calls
    # from the same initial state (reloaded between calls, outside the timed
    # region); the median is reported: the host side of the pageable copies
    # varies from call to call (one download seen at 7 ms against 1.5 ms).
    e2e_calls = []
    # the median of five calls (every call's time is reported): the copies are
    # pageable-host traffic, which a busy host can slow for a while
    n_calls = 5 if cells * args.steps <= 2_000_000_000 else 1   # long runs: one call
    with H.Simulation2D(p.nx, p.ny, p.g, bounds, p.gamma, p.W, p.U, bc=p.bc,
                        slope_limiter=p.slope_limiter, cfl=p.cfl, tf=p.tf, max_steps=args.steps,
                        options=H.default_options(device=device, precision=prec)) as sim:
        for _ in range(n_calls):
            sim.load(p.W, p.U)
            barrier(ws)
            t0 = time.perf_counter()
            code, msg, _, stats_k = sim.launch()
            secs = time.perf_counter() - t0
            assert code == 0, msg
            e2e_calls.append((max_over_ranks(secs, ws), stats_k))
    e2e_s, e2e_stats = sorted(e2e_calls, key=lambda c: c[0])[len(e2e_calls) // 2]
    e2e_value = ws * cells * args.steps / e2e_s

    # ---- the other configurations beside the headline: the precision study's
    #      8192^2 point blast, the 256-instance ensemble, the 1024^2 adjoint ----
    blast = ensemble = adjoint = None
    if args.workload == "shear_layer" and not args.no_blast:
        blast = blast_leg(args, H, device, ws)
        ensemble = ensemble_leg(args, H, device, ws)
        adjoint = adjoint_leg(args, H, device)

    if rank != 0:
        return

    pk = peaks()
    per_launch_s = step_ms * 1e-3 / args.steps
    achieved_gbs = bytes_per_cell * cells / per_launch_s / 1e9
    clocks = clk.summary()      # (reads and removes the sample file: once)
    sms = H.sm_count(device)
    clock_mhz = clocks.get("sm_mhz") or clocks.get("sm_max_mhz") or 0.0
    fp64_tflops, fp32_tflops = H.calibrate(device)
    traffic = profile_traffic() if (prec == H.PRECISION_FP64 and args.workload == "shear_layer"
                                    and N_SIDE == 2048) else None
    fp32_ms = step_ms if prec == H.PRECISION_FP32 else ms_o
    fp64_ms = step_ms if prec == H.PRECISION_FP64 else ms_o
    line = {
        "metric": METRIC, "value": value, "unit": "cell-updates/s", "n_gpus": ws,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": step_ms / args.steps,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f64" if prec == H.PRECISION_FP64 else "f32",
        "data": f"synthetic (seeded {args.workload})",
        "config": shear_config(args, ws) if args.workload == "shear_layer" and prec == H.PRECISION_FP64 else
                  {"workload": f"{args.workload}_{N_SIDE}x{N_SIDE}_{args.precision}",
                   "grid": [N_SIDE, N_SIDE], "ghost_cells": 2,
                   "limiter": p.slope_limiter, "cfl": p.cfl, "boundaries": p.bc[0],
                   "steps_per_run": args.steps,
                   "l2": "state larger than the 129 MB L2 (no flush needed)" if cells >= 1 << 20
                         else "state fits in L2 (profiling size)",
                   "parallelism": "replicas" if ws > 1 else "single"},
        "roofline": {"bound": "hbm", "achieved": achieved_gbs, "peak": pk["hbm_gbs"],
                     "unit": "GB/s", "frac": achieved_gbs / pk["hbm_gbs"],
                     "traffic": traffic, "peak_source": pk["source"],
                     "bytes_per_cell_update": bytes_per_cell,
                     "note": "HBM is not the binding roof of this stencil: the FP64 step is bound by "
                             "its FP64 pipe, the FP32 form by instruction issue; fp_roofline reports "
                             "them"},
        "fp_roofline": fp_roofline(prec, value, fp64_tflops, fp32_tflops, H, args.workload,
                                   sms=sms, sm_mhz=clock_mhz),
        "forms": {
            "fp64": {"value": cells * args.steps / (fp64_ms * 1e-3), "ms_per_step": fp64_ms / args.steps,
                     "conserved_drift": drift_main if prec == H.PRECISION_FP64 else drift_o},
            "fp32": {"value": cells * args.steps / (fp32_ms * 1e-3), "ms_per_step": fp32_ms / args.steps,
                     "speedup_vs_fp64": fp64_ms / fp32_ms,
                     "rel_l1_vs_fp64": {"density": l1[0], "velocity_x": l1[1],
                                        "velocity_y": l1[2], "pressure": l1[3]},
                     "conserved_drift": drift_main if prec == H.PRECISION_FP32 else drift_o,
                     "fp_roofline": fp_roofline(H.PRECISION_FP32, cells * args.steps / (fp32_ms * 1e-3),
                                                fp64_tflops, fp32_tflops, H, args.workload,
                                                sms=sms, sm_mhz=clock_mhz),
                     "roofline": hbm_roofline(cells * args.steps / (fp32_ms * 1e-3), BYTES_PER_CELL_FP64 // 2,
                                              pk, profile_traffic("fp32") if args.workload == "shear_layer"
                                              and N_SIDE == 2048 else None)},
        },
        "e2e": {"value": e2e_value, "unit": "cell-updates/s",
                "h2d_bytes_per_step": e2e_stats["h2d_bytes"] / args.steps,
                "d2h_bytes_per_step": e2e_stats["d2h_bytes"] / args.steps,
                "seconds": e2e_s, "h2d_ms": e2e_stats["h2d_ms"], "d2h_ms": e2e_stats["d2h_ms"],
                "calls_seconds": [c[0] for c in e2e_calls],
                "note": "hydro_gpu_launch_simulation on host System arrays: upload, K steps, "
                        "download (copies inside the timed call); median of the calls"},
        "gpu_launches": int(launches),
        "clocks": clocks,
    }
    if blast is not None:
        line["forms"]["point_blast_8192"] = blast
        line["forms"]["ensemble_256"] = ensemble
        line["forms"]["adjoint_1024"] = adjoint
    if not args.no_cpu_baseline:
        line["cpu_baseline"] = cpu_sample(args.steps)
    print(json.dumps(line))


if __name__ == "__main__":
    main()
