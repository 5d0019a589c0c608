"""Benchmark: cell-updates/s of the full FP64 time step on one GB300.

Workload: the 512x256x256 sessile drop (density ratio 1000, viscosity ratio 100,
60/120 deg checkerboard lower wall, dt = 1e-5) in reference axis order (ni,
nj_wall, nk) = (512, 256, 256), the largest single-GPU configuration the metric is
quoted on.  One "step" is one full time step (main.f90:473-697).  value = interior
cells x timed steps / device time (CUDA events on the library's stream,
device-resident state, inputs larger than L2).  e2e = the same through the C-ABI
with host buffers (fmf_ctx_step_host every step: the state's 10 input fields up
from pinned host memory, the 12 result fields back), over the same steps.

Beside the headline: the mixed-precision step on the same workload (value,
speed-up, per-field error against the FP64 step after the timed steps and over the
workload's 500 steps), the 256x128x128 Couette case in both precisions, the
adjoint/forward cost of the 128x64x64 rollout (K = 200, checkpoints every 16), the
adjoint with a mixed-precision forward on the 256x128x128 sessile drop (K = 500,
ceil(sqrt(K)) checkpoints: gradient error against the FP64 adjoint, device bytes,
cost), and the CPU baseline.

`--impl reference` times the CPU restatement of the reference's algorithm
(oracle/, the reference Fortran cannot be built here: no Fortran compiler) on
the host cores, same workload, metric and config.
"""
from __future__ import annotations

import argparse
import ctypes
import json
import math
import os
import statistics
import subprocess
import sys
import time

REPO = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(REPO, "fel-multi-phase-flow_gb300"))
sys.path.insert(0, os.path.join(REPO, "oracle"))

WORKLOAD = "droplet512"
METRIC = "cell-updates/s/step plain FP64 vs mixed at stated error; adjoint/forward cost"
UNIT = "cell-updates/s"

# The dominant kernel's counters per interior cell of one launch (k_weno2, one
# velocity level: the advection of (u, v, w); the (uo, vo, wo) level is carried
# over from the previous step).  DRAM bytes read + written from the ncu capture of
# one one-level launch at 256x128x128 (113.5 MB + 68.7 MB over 4,194,304 cells;
# python bench.py --profile --workload couette256 --warmup 2 --steps 1 under
# ncu --set full -k regex:k_weno2 -s 1 -c 1 --clock-control none).  FP64
# instructions (DADD + DMUL + DFMA thread instructions; flops count an FMA twice):
# half of a two-level launch's (955.7 M + 1219.5 M + 1885.8 M at 256x128x128),
# both levels running the same loop body.
WENO_CAPTURE = ("ncu --set full of one one-level k_weno2 launch, couette256 256x128x128 (DRAM bytes); "
                "FP64 instruction counts: half of a two-level launch's at the same size")
WENO_TRAFFIC_PER_CELL = (113.540352e6 + 68.679168e6) / 4194304
WENO_FP64_INST_PER_CELL = (955711488 + 1219493888 + 1885798400) / 2 / 4194304
WENO_FP64_FLOPS_PER_CELL = (955711488 + 1219493888 + 2 * 1885798400) / 2 / 4194304
# weno5.h's own formula (both one-sided reconstructions) per cell and level
WENO_REFERENCE_FLOPS_PER_CELL = 1383.0

# The FP64-accurate step's WENO5 kernel (k_weno2_df, one level, FP32-pair
# arithmetic): FP32 thread instructions (FADD + FMUL + FFMA) per interior cell from
# the ncu capture of one one-level launch at 256x128x128 (13,157.6 per cycle over
# 1,736,058 cycles, 4,194,304 cells; python bench.py --profile --precision fp64e
# --workload couette256 --warmup 2 --steps 1 under ncu --set full -k
# regex:k_weno2_df -s 1 -c 1 --clock-control none)
PAIR_WENO_CAPTURE = ("ncu --set full of one one-level k_weno2_df launch, couette256 256x128x128: FADD + FMUL + "
                     "FFMA thread instructions")
PAIR_WENO_FP32_INST_PER_CELL = (10113.089172 + 1495.997566 + 1548.534517) * 1736057.75 / 4194304
PAIR_WENO_TRAFFIC_PER_CELL = (113.535232e6 + 70.033408e6) / 4194304

# Algorithmic bytes of one cell-update: 83 words outside the viscous solve and 21
# words per outer iteration of it (each stage's external arrays read once and
# written once, FP64)
B_CELL_FIXED = 664
B_CELL_PER_SOR = 168


def _peaks():
    try:
        with open(os.path.join(REPO, "MEASURED_PEAKS.json")) as f:
            return json.load(f), "measured"
    except Exception:
        return {"hbm_gbs": 6800.0, "bf16_tflops": 1900.0}, "fallback"


def config_dict(cfg, world: int) -> dict:
    """The workload description both arms print (identical keys and values)."""
    return {"workload": f"{cfg.name} {cfg.ni}x{cfg.nj}x{cfg.nk} (ni,nj_wall,nk)", "precision": "fp64",
            "l2": "inputs larger than L2 (each field of the state is " f"{8 * math.prod(cfg.shape) / 1e6:.0f} MB)",
            "parallelism": "replicas" if world > 1 else "single"}


class Clocks:
    """nvidia-smi sampling during the timed region (clocks, throttle reasons)."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self):
        self.p = None
        self.path = None

    def start(self):
        try:
            import tempfile
            fd, self.path = tempfile.mkstemp(prefix="fmf_clocks_", suffix=".csv")
            self.f = os.fdopen(fd, "w")
            self.p = subprocess.Popen(["nvidia-smi", f"--query-gpu={self.Q}", "--format=csv,noheader,nounits",
                                       "-lms", "200", "-i", os.environ.get("CUDA_VISIBLE_DEVICES", "0").split(",")[0]],
                                      stdout=self.f, stderr=subprocess.DEVNULL)
        except Exception:
            self.p = None

    def stop(self):
        if not self.p:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.p.terminate()
        self.p.wait()
        self.f.close()
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in open(self.path):
            parts = [x.strip() for x in line.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                mx.append(float(parts[2]))
            except ValueError:
                continue
            for nm, val in zip(names, parts[5:9]):
                if val.lower() == "active":
                    reasons.add(nm)
        try:
            os.remove(self.path)
        except OSError:
            pass
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": sorted(reasons), "samples": len(sm)}


def _oracle_env():
    """All host threads, bound close, for the oracle's OpenMP loops (read when its
    library loads)."""
    os.environ.setdefault("OMP_NUM_THREADS", str(os.cpu_count() or 1))
    os.environ.setdefault("OMP_PROC_BIND", "close")
    return int(os.environ["OMP_NUM_THREADS"])


def cpu_baseline_sample(cfg, warmup=1, steps=2):
    """The oracle (C++/OpenMP restatement, all host threads) on a bounded sample:
    `steps` full steps after `warmup`, from the workload's initial state."""
    cores = _oracle_env()
    import oracle
    s = oracle.Solver(cfg)
    st = s.initial_state()
    s.step(st, warmup)
    t0 = time.perf_counter()
    s.step(st, steps)
    dt = time.perf_counter() - t0
    s.close()
    return cfg.cells * steps / dt, dt, cores


def run_reference(args):
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    from fmf import config as C
    cfg = C.get(args.workload)
    cores = _oracle_env()
    import oracle
    s = oracle.Solver(cfg)
    st = s.initial_state()
    s.step(st, args.warmup)
    t0 = time.perf_counter()
    s.step(st, args.steps)
    dt = time.perf_counter() - t0
    s.close()
    v = cfg.cells * args.steps / dt
    line = {"impl": "reference", "metric": METRIC, "value": v, "unit": UNIT, "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * dt / args.steps,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
            "data": "synthetic", "config": config_dict(cfg, args.gpus),
            "cpu_baseline": {"value": v, "unit": UNIT, "cores": cores, "kind": "port",
                             "sample": f"{args.steps} full steps of {cfg.name} after {args.warmup} warm-up "
                                       "steps, OMP_PROC_BIND=close; the reference Fortran cannot be built here (no "
                                       "Fortran compiler), so its C++/OpenMP restatement oracle/fmf_oracle.cpp "
                                       "(g++ -O3 -fopenmp -ffp-contract=off) runs"},
            "e2e": {"value": v, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def _rel(a, b, cfg):
    from fmf import config as C
    x, y = C.interior(a), C.interior(b)
    import numpy as np
    return float(np.abs(x - y).max() / max(np.abs(y).max(), 1e-300))


FIELDS = {"phi": 9, "u": 0, "v": 1, "w": 2, "p": 6}


def mixed_case(cfg, st0, steps, warmup, stream, fp64_ms=None):
    """The mixed-precision step against the FP64 step on one workload: CUDA-event
    time per step of each (state resident, `steps` after `warmup`), and the
    per-field error of the mixed state against the FP64 state after warmup + steps
    from the same initial state."""
    import torch

    from fmf import capi

    out = {"workload": f"{cfg.name} {cfg.ni}x{cfg.nj}x{cfg.nk}", "steps": steps, "warmup": warmup}
    states = {}
    for prec, key in ((capi.FMF_FP64, "fp64"), (capi.FMF_MIXED, "mixed")):
        g = capi.Stepper(cfg, precision=prec, stream=stream.cuda_stream)
        g.upload(st0)
        g.step(warmup)
        g.sync()
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        g.step(steps)
        e1.record(stream)
        e1.synchronize()
        out[key + "_ms_per_step"] = e0.elapsed_time(e1) / steps
        states[key] = g.get_state()
        g.close()
    if fp64_ms is not None:
        out["fp64_ms_per_step"] = fp64_ms
    ref, mix = states["fp64"], states["mixed"]
    out["value_fp64"] = cfg.cells / (out["fp64_ms_per_step"] * 1e-3)
    out["value_mixed"] = cfg.cells / (out["mixed_ms_per_step"] * 1e-3)
    out["unit"] = UNIT
    out["speedup_vs_fp64"] = out["fp64_ms_per_step"] / out["mixed_ms_per_step"]
    out["steps_compared"] = warmup + steps
    out["max_rel_err_vs_fp64"] = {k: _rel(mix[f], ref[f], cfg) for k, f in FIELDS.items()}
    return out


def fp64e_case(cfg, st0, steps, warmup, stream, fp64_ms):
    """The FP64-accurate step (FMF_FP64E: the FP64 step with its FP64-pipe-bound
    stencils in FP32-pair arithmetic) on the workload: CUDA-event time per step (state resident, `steps`
    after `warmup`), and against the FP64 step from the same initial state after
    warmup + steps: each field's largest difference relative to the FP64 field's
    largest magnitude, and whether every viscous solve took the same iterations."""
    import torch

    from fmf import capi

    states, iters = {}, {}
    out = {"workload": f"{cfg.name} {cfg.ni}x{cfg.nj}x{cfg.nk}", "steps": steps, "warmup": warmup}
    for prec, key in ((capi.FMF_FP64E, "fp64e"), (capi.FMF_FP64, "fp64")):
        g = capi.Stepper(cfg, precision=prec, stream=stream.cuda_stream)
        g.upload(st0)
        g.step(warmup)
        its = g.sor_iterations()
        g.sync()
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        g.step(steps)
        e1.record(stream)
        e1.synchronize()
        iters[key] = its + g.sor_iterations()
        if key == "fp64e":
            out["ms_per_step"] = e0.elapsed_time(e1) / steps
            # the dominant pair kernel, WENO5 of (u, v, w) (stage 4: the split of the
            # three fields into pairs, then k_weno2_df), against the FP32 pipe
            ms_stage = ctypes.c_float()
            capi.check(capi.lib().fmf_ctx_time_stage(g.h, 4, 5, ctypes.byref(ms_stage)), "time_stage")
            fp32 = ctypes.c_double()
            capi.lib().fmf_measure_fma_rate.argtypes = [ctypes.c_int, ctypes.POINTER(ctypes.c_double)]
            capi.check(capi.lib().fmf_measure_fma_rate(0, ctypes.byref(fp32)), "fma rate")
            rate = PAIR_WENO_FP32_INST_PER_CELL * cfg.cells / (ms_stage.value * 1e-3) / 1e12
            out["roofline"] = {"bound": "fp32", "achieved": rate, "peak": fp32.value / 2.0,
                               "unit": "T FP32 instructions/s", "frac": rate / (fp32.value / 2.0),
                               "traffic": PAIR_WENO_TRAFFIC_PER_CELL * cfg.cells,
                               "kernel": "k_weno2_df, one level (with the split of u, v, w into pairs before it)",
                               "kernel_ms": ms_stage.value,
                               "fp32_inst_per_cell": PAIR_WENO_FP32_INST_PER_CELL,
                               "counters_source": PAIR_WENO_CAPTURE + ", scaled to the workload by its cell count",
                               "peak_source": "FP32 FMA chains measured live (fmf_measure_fma_rate), one "
                                              "instruction per FMA"}
        states[key] = g.get_state()
        g.close()
    out["fp64_ms_per_step"] = fp64_ms
    out["value"] = cfg.cells / (out["ms_per_step"] * 1e-3)
    out["unit"] = UNIT
    out["speedup_vs_fp64"] = fp64_ms / out["ms_per_step"]
    out["steps_compared"] = warmup + steps
    out["max_rel_err_vs_fp64"] = {k: _rel(states["fp64e"][f], states["fp64"][f], cfg) for k, f in FIELDS.items()}
    out["same_viscous_iterations"] = iters["fp64e"] == iters["fp64"]
    out["precision"] = ("the FP64 step with its WENO5 advection, CSF force, viscous momentum factors and explicit "
                        "viscous term in FP32-pair arithmetic (two floats per value, about 48 significant bits) on "
                        "the FP32 pipe; state, viscous sweeps, pressure solve, projection and volume sums FP64; "
                        "parity with the oracle at the FP64 step's 1e-10 (tests/test_gpu_fp64e.py)")
    return out


def mixed_horizon(cfg, st0, steps, every, stream):
    """FP64 and mixed steps side by side from the same initial state over `steps`
    steps: the largest relative error of each field (interior, against the FP64
    field's largest magnitude) at every `every`-th step, and there the next mixed
    viscous solve re-formed in FP64 (fmf_ctx_check_sor: one FP64 outer iteration
    from its result over the FP64 solve's first-iteration change, which the
    reference's rule wants at or below 1e-3)."""
    import numpy as np

    from fmf import capi

    ref = capi.Stepper(cfg, stream=stream.cuda_stream)
    ref.upload(st0)
    mix = capi.Stepper(cfg, precision=capi.FMF_MIXED, stream=stream.cuda_stream)
    mix.upload(st0)
    worst = {k: 0.0 for k in FIELDS}
    worst_rule = 0.0
    table = []
    done = 0
    t0 = time.perf_counter()
    while done < steps:
        n = min(every, steps - done)
        ref.step(n)
        mix.step(n)
        done += n
        a, b = mix.get_state(), ref.get_state()
        finite = bool(np.isfinite(a).all() and np.isfinite(b).all())
        errs = {k: _rel(a[f], b[f], cfg) for k, f in FIELDS.items()}
        for k in FIELDS:
            worst[k] = max(worst[k], errs[k])
        # the next mixed viscous solve against the FP64 stop rule (the state is left
        # as it was)
        chk = mix.check_sor()
        worst_rule = max(worst_rule, chk["fp64_ratio"])
        table.append({"step": done, "finite": finite, **{k: errs[k] for k in FIELDS},
                      "viscous_solve_fp64_rule": {k: chk[k] for k in ("iterations", "own_ratio", "fp64_ratio",
                                                                       "fp64_ratio_of_fp64_solve",
                                                                       "rel_diff_vs_fp64_solve")}})
    ref.close()
    mix.close()
    return {"workload": f"{cfg.name} {cfg.ni}x{cfg.nj}x{cfg.nk}", "steps_compared": steps, "every": every,
            "max_rel_err_vs_fp64": worst, "viscous_solve_max_fp64_ratio": worst_rule, "sor_tol": 1e-3,
            "per_check": table, "seconds": time.perf_counter() - t0}


def adjoint_cost(K, stream, every, workload="couette128"):
    """Adjoint/forward wall-clock ratio of the K-step rollout on a workload (default
    the 128x64x64 Couette workload, per-wall-cell angle 75 +- 5 deg), checkpoints
    every `every` steps (16 for K = 200 as the workload states, about sqrt(K);
    0: ceil(sqrt(K))):
    fmf_adj_rollout (J and all gradients) against fmf_adj_forward (J) with the same
    solver settings (viscous solve to the reference's 1e-3, transposed solve to
    1e-6), and against the graph-replayed production step (fmf_ctx_step)."""
    from fmf import capi
    from fmf import config as C
    from fmf.adjoint import Adjoint

    cfg = C.get(workload)
    st0 = C.raw_state(cfg)
    walls = [w.copy() for w in C.wall_arrays(cfg)]
    every = every if every > 0 else int(math.ceil(math.sqrt(K)))
    A = Adjoint(cfg, sor_tol=1e-3, sor_max=21, adj_tol=1e-6, adj_max=200)
    A.forward(2, st0, walls)
    # allocates the checkpoint and record slots (two segments: the recomputing worker's too)
    A.rollout(min(K, 2 * every), st0, walls, every=every)
    t0 = time.perf_counter()
    J = A.forward(K, st0, walls)
    t_fwd = time.perf_counter() - t0
    t0 = time.perf_counter()
    Ja, _ = A.rollout(K, st0, walls, every=every)
    t_adj = time.perf_counter() - t0
    phases = A.phase_seconds()
    its = A.iterations()
    A.close()
    S = capi.Stepper(cfg, stream=stream.cuda_stream)
    # every CUDA graph the timed steps replay captured first (six rotations of the
    # state buffers, the first step after an upload, the steps after it)
    S.upload(st0)
    S.init_bc()
    S.step(13)
    S.sync()
    S.upload(st0)
    S.init_bc()
    S.sync()
    t0 = time.perf_counter()
    S.step(K)
    S.sync()
    t_ctx = time.perf_counter() - t0
    S.close()
    return {"workload": f"{workload} {cfg.ni}x{cfg.nj}x{cfg.nk}", "K": K, "checkpoint_every": every,
            "objective": "find_interface_positions_lower after K steps", "J": J,
            "parameters": "theta0, zeta, l1, l2 (wall planes), initial phi",
            "forward_s": t_fwd, "rollout_s": t_adj, "adjoint_over_forward": t_adj / t_fwd,
            "adjoint_over_graph_forward": t_adj / t_ctx, "graph_forward_s": t_ctx,
            "phases_s": {"forward": phases[0], "recompute": phases[1], "reverse": phases[2]},
            "viscous_iterations": {"forward_all": its[0], "transposed": its[1]},
            "weno5_reverse": "FP32 pairs on the FP64 differences (FMF_ADJ_PAIR_REVERSE=0: FP64)",
            "tolerances": {"sor": 1e-3, "adjoint": 1e-6}}


def adjoint_mixed(K, stream, workload="droplet256", every=0):
    """The adjoint of the K-step rollout with a mixed-precision forward (FP32 WENO5,
    MTHINC, CSF and viscous corrections in the forward and recomputed steps; FP64
    reverse) on the sessile drop at 256x128x128, checkpoints every ceil(sqrt(K))
    steps: the relative error of each gradient against the FP64 adjoint's (largest
    |difference| over the largest |FP64 gradient|, and the same over the L2 norm),
    the device bytes each handle holds (own accounting, and the device memory in use
    after the rollout less that before the handle), and the rollout time against the
    handle's own forward and against the graph-replayed product step of the same
    precision.  The FP64 adjoint runs first and is closed before the mixed one
    (their record slots do not fit together)."""
    import numpy as np
    import torch

    from fmf import capi
    from fmf import config as C
    from fmf.adjoint import Adjoint

    cfg = C.get(workload)
    st0 = C.raw_state(cfg)
    walls = [w.copy() for w in C.wall_arrays(cfg)]
    every = every if every > 0 else int(math.ceil(math.sqrt(K)))
    runs = {}
    grads = {}
    for prec, key in ((capi.FMF_FP64, "fp64"), (capi.FMF_MIXED, "mixed")):
        torch.cuda.synchronize()
        free0, _ = torch.cuda.mem_get_info()
        A = Adjoint(cfg, sor_tol=1e-3, sor_max=21, adj_tol=1e-6, adj_max=200, precision=prec)
        A.forward(2, st0, walls)
        A.rollout(min(K, 2 * every), st0, walls, every=every)  # allocates checkpoints and record slots
        t0 = time.perf_counter()
        J = A.forward(K, st0, walls)
        t_fwd = time.perf_counter() - t0
        t0 = time.perf_counter()
        Ja, g = A.rollout(K, st0, walls, every=every)
        t_adj = time.perf_counter() - t0
        torch.cuda.synchronize()
        free1, _ = torch.cuda.mem_get_info()
        ph = A.phase_seconds()
        its = A.iterations()
        dev_bytes = A.device_bytes()
        A.close()
        S = capi.Stepper(cfg, precision=prec, stream=stream.cuda_stream)
        S.upload(st0)
        S.init_bc()
        S.step(13)
        S.sync()
        S.upload(st0)
        S.init_bc()
        S.sync()
        t0 = time.perf_counter()
        S.step(K)
        S.sync()
        t_ctx = time.perf_counter() - t0
        S.close()
        runs[key] = {"J": J, "forward_s": t_fwd, "rollout_s": t_adj, "graph_forward_s": t_ctx,
                     "weno5_reverse": "FP32 pairs on the FP64 differences" if key == "fp64" else "FP32",
                     "adjoint_over_forward": t_adj / t_fwd, "adjoint_over_graph_forward": t_adj / t_ctx,
                     "phases_s": {"forward": ph[0], "recompute": ph[1], "reverse": ph[2]},
                     "handle_device_bytes": dev_bytes, "device_bytes_in_use_delta": int(free0 - free1),
                     "viscous_iterations": {"forward_all": its[0], "transposed": its[1]}}
        grads[key] = g
    names = ("theta0", "zeta", "l1", "l2", "phi")
    err = {n: {"max": float(np.abs(a - b).max() / max(np.abs(b).max(), 1e-300)),
               "l2": float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300))}
           for n, a, b in zip(names, grads["mixed"], grads["fp64"])}
    return {"workload": f"{workload} {cfg.ni}x{cfg.nj}x{cfg.nk}", "K": K, "checkpoint_every": every,
            "objective": "find_interface_positions_lower after K steps",
            "gradient_rel_err_mixed_vs_fp64": err,
            "J_rel_err_mixed_vs_fp64": abs(runs["mixed"]["J"] - runs["fp64"]["J"]) / max(abs(runs["fp64"]["J"]),
                                                                                          1e-300),
            "mixed": runs["mixed"], "fp64": runs["fp64"], "tolerances": {"sor": 1e-3, "adjoint": 1e-6}}


def profile(args):
    """No timing: start-up pass, --warmup steps, then --steps steps (for ncu)."""
    from fmf import build as fbuild
    from fmf import capi
    from fmf import config as C
    fbuild.build()
    if args.precision in ("adjoint", "adjoint_mixed"):
        # --steps K of the adjoint rollout on the workload (for ncu launch lists);
        # adjoint_mixed: with the mixed-precision forward
        from fmf.adjoint import Adjoint
        cfg = C.get(args.workload)
        A = Adjoint(cfg, sor_tol=1e-3, sor_max=21, adj_tol=1e-6, adj_max=200,
                    precision=capi.FMF_MIXED if args.precision == "adjoint_mixed" else capi.FMF_FP64)
        st0 = C.raw_state(cfg)
        walls = C.wall_arrays(cfg)
        A.rollout(max(1, args.warmup), st0, walls)
        J, _ = A.rollout(args.steps, st0, walls)
        print(json.dumps({"profile": args.workload, "adjoint_steps": args.steps, "J": J,
                          "iterations": A.iterations()}))
        A.close()
        return
    prec = {"mixed": capi.FMF_MIXED, "fp64e": capi.FMF_FP64E}.get(args.precision, capi.FMF_FP64)
    g = capi.Stepper(C.get(args.workload), precision=prec)
    g.initial_state()
    g.step(args.warmup)
    g.sync()
    g.step(args.steps)
    g.sync()
    print(json.dumps({"profile": args.workload, "sor_iterations": g.sor_iterations()}))
    g.close()


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="fmf", choices=["fmf", "reference"])
    ap.add_argument("--workload", default=WORKLOAD)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--mixed-horizon", type=int, default=500,
                    help="steps of the side-by-side FP64/mixed error check on the workload (0: skip)")
    ap.add_argument("--second-workload", default="couette256",
                    help="FP64 and mixed step times on a second workload ('' to skip)")
    ap.add_argument("--adjoint-steps", type=int, default=200,
                    help="K of the adjoint-cost measurement (0: skip)")
    ap.add_argument("--adjoint-every", type=int, default=16,
                    help="checkpoint interval of the adjoint rollout (0: ceil(sqrt(K)))")
    ap.add_argument("--adjoint-workload", default="couette128",
                    help="workload of the adjoint-cost measurement")
    ap.add_argument("--adjoint-mixed-steps", type=int, default=500,
                    help="K of the mixed-forward adjoint on the 256x128x128 sessile drop (0: skip)")
    ap.add_argument("--fp64e", type=int, default=1,
                    help="1: time the FP64-accurate step with FP32-pair stencils (FMF_FP64E) on the workload too")
    ap.add_argument("--precision", default="fp64", choices=["fp64", "mixed", "fp64e", "adjoint", "adjoint_mixed"],
                    help="--profile only")
    ap.add_argument("--profile", action="store_true",
                    help="no timing: start-up pass, --warmup steps, then --steps steps (for ncu launch lists)")
    args = ap.parse_args()
    if args.impl == "reference":
        run_reference(args)
        return
    if args.profile:
        profile(args)
        return

    import numpy as np
    import torch

    from fmf import build as fbuild
    from fmf import capi
    from fmf import config as C
    from fmf import replicas

    rank, world = replicas.world()
    local = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(local)
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
    fbuild.build()
    L = capi.load()
    cfg = C.get(args.workload)
    stream = torch.cuda.Stream()
    g = capi.Stepper(cfg, stream=stream.cuda_stream)
    st = g.initial_state()
    g.step(args.warmup)
    g.sync()

    def barrier():
        torch.cuda.synchronize()
        replicas.barrier()

    # ---- headline: FP64 steps, state resident -------------------------------
    clocks = Clocks()
    barrier()
    clocks.start()
    l0 = L.fmf_kernel_launches()
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    g.step(args.steps)
    e1.record(stream)
    e1.synchronize()
    launches = L.fmf_kernel_launches() - l0
    ms = e0.elapsed_time(e1)
    barrier()
    clk = clocks.stop()
    iters = g.sor_iterations()
    ms = replicas.max_over_ranks(ms)
    value = replicas.throughput(cfg.cells, args.steps, ms * 1e-3)
    n_sor = float(np.mean(iters)) if iters else 0.0

    # ---- e2e: host buffers through the C-ABI, the same number of steps -------
    # every step uploads the 10 input fields of the state from pinned host memory
    # (phin is written by the step before it is read) and returns the 12 result
    # fields to it (fmf_ctx_step_host: part of the upload and the result fields that
    # are final early overlap the step); the host buffer carries the state from step
    # to step, as a caller's time loop does
    pinned = torch.empty((12,) + cfg.shape, dtype=torch.float64, pin_memory=True)
    host = pinned.numpy()
    host[:] = g.get_state()
    bytes_field = math.prod(cfg.shape) * 8
    g.step_host(host, host)  # the host-buffer path's own first call (copy stream, events)
    barrier()
    t0 = time.perf_counter()
    for _ in range(args.steps):
        g.step_host(host, host)
    e2e_dt = replicas.max_over_ranks(time.perf_counter() - t0)
    e2e_value = replicas.throughput(cfg.cells, args.steps, e2e_dt)
    del pinned, host

    # ---- rooflines ------------------------------------------------------------
    # Dominant kernel: WENO5 advection of (u, v, w) (k_weno2, one level: stage 4),
    # FP64-pipe bound.  Executed FP64 instructions per second (ncu DADD + DMUL +
    # DFMA per cell of one launch, WENO_FP64_INST_PER_CELL) against the FP64 pipe's
    # instruction rate, half the FMA-chain flop rate fmf_measure_fma_rate measures
    # live (an FMA is one instruction and two flops).  Also reported: executed flops
    # and the rate of weno5.h's own formula (both one-sided reconstructions), which
    # exceeds the FMA peak because the kernel evaluates the upwind side only, in
    # fewer operations; and the kernel against HBM (6 words per cell algorithmic).
    ms_stage = ctypes.c_float()
    capi.check(L.fmf_ctx_time_stage(g.h, 4, 5, ctypes.byref(ms_stage)), "time_stage")
    ms_stage2 = ctypes.c_float()
    capi.check(L.fmf_ctx_time_stage(g.h, 0, 3, ctypes.byref(ms_stage2)), "time_stage")
    peaks, peak_kind = _peaks()
    fp64 = ctypes.c_double()
    L.fmf_measure_fma_rate.argtypes = [ctypes.c_int, ctypes.POINTER(ctypes.c_double)]
    capi.check(L.fmf_measure_fma_rate(1, ctypes.byref(fp64)), "fma rate")
    t_weno = ms_stage.value * 1e-3
    inst_rate = WENO_FP64_INST_PER_CELL * cfg.cells / t_weno / 1e12
    inst_peak = fp64.value / 2.0
    gbs = 6 * 8 * cfg.cells / t_weno / 1e9
    roofline = {"bound": "fp64", "achieved": inst_rate, "peak": inst_peak, "unit": "T FP64 instructions/s",
                "frac": inst_rate / inst_peak,
                "traffic": WENO_TRAFFIC_PER_CELL * cfg.cells,
                "kernel": "k_weno2, one level (the step's cal_advu_weno5 of u, v, w)", "kernel_ms": ms_stage.value,
                "kernel_ms_both_levels": ms_stage2.value,
                "fp64_inst_per_cell": WENO_FP64_INST_PER_CELL,
                "counters_source": WENO_CAPTURE + ", scaled to the workload by its cell count",
                "executed_tflops": WENO_FP64_FLOPS_PER_CELL * cfg.cells / t_weno / 1e12,
                "reference_formula_tflops": WENO_REFERENCE_FLOPS_PER_CELL * cfg.cells / t_weno / 1e12,
                "fma_peak_tflops": fp64.value,
                "peak_source": "FP64 FMA chains measured live (fmf_measure_fma_rate), one instruction per FMA; "
                               "HBM peak " + peak_kind + " (MEASURED_PEAKS.json hbm_gbs)",
                "hbm": {"achieved": gbs, "peak": peaks["hbm_gbs"], "unit": "GB/s", "frac": gbs / peaks["hbm_gbs"]}}
    b_cell = B_CELL_FIXED + B_CELL_PER_SOR * n_sor
    step_gbs = b_cell * cfg.cells / (ms / args.steps * 1e-3) / 1e9
    step_roofline = {"bytes_per_cell": b_cell, "formula": "664 + 168 * mean viscous iterations",
                     "sor_iterations_mean": n_sor, "achieved": step_gbs, "peak": peaks["hbm_gbs"], "unit": "GB/s",
                     "frac": step_gbs / peaks["hbm_gbs"],
                     "note": "the FP64 step is bound by the FP64 pipe (its largest kernels issue FP64 instructions "
                             "near the pipe's rate), not by HBM"}

    # ---- mixed precision on the same workload -----------------------------------
    mixed = None
    horizon = None
    second = None
    fp64e = None
    if rank == 0:
        g.close()
        mixed = mixed_case(cfg, st, args.steps, args.warmup, stream, fp64_ms=ms / args.steps)
        mixed["precision"] = ("fp32: WENO5, MTHINC Newton + Gauss-point fluxes, CSF normals and curvature, viscous "
                              "sweeps on FP32 corrections (one refinement step); fp32 pairs: explicit viscous term, "
                              "momentum factors under the FP64 residual; fp64: state, residual, pressure FFT+TDMA, "
                              "projection, divergence, volume sums")
        if args.mixed_horizon > 0:
            horizon = mixed_horizon(cfg, st, args.mixed_horizon, 100, stream)
        if args.fp64e:
            fp64e = fp64e_case(cfg, st, args.steps, args.warmup, stream, ms / args.steps)
        del st
        if args.second_workload:
            cfg2 = C.get(args.second_workload)
            g2 = capi.Stepper(cfg2, stream=stream.cuda_stream)
            st2 = g2.initial_state()
            g2.close()
            second = mixed_case(cfg2, st2, args.steps, args.warmup, stream)
    adjoint = None
    if rank == 0 and args.adjoint_steps > 0:
        adjoint = adjoint_cost(args.adjoint_steps, stream, args.adjoint_every, args.adjoint_workload)
    adjoint_m = None
    if rank == 0 and args.adjoint_mixed_steps > 0:
        adjoint_m = adjoint_mixed(args.adjoint_mixed_steps, stream)
    cpu = None
    if rank == 0 and not args.no_cpu_baseline:
        v, dt, cores = cpu_baseline_sample(cfg, 1, 2)
        cpu = {"value": v, "unit": UNIT, "cores": cores, "kind": "port",
               "sample": f"2 full steps of {cfg.name} after 1 warm-up step ({dt:.1f} s), oracle/fmf_oracle.cpp "
                         "C++/OpenMP restatement (g++ -O3), all host threads, OMP_PROC_BIND=close"}
    if rank == 0:
        line = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
                "warmup": args.warmup, "ms_per_step": ms / args.steps, "higher_is_better": True,
                "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
                "config": config_dict(cfg, world),
                "e2e": {"value": e2e_value, "unit": UNIT, "h2d_bytes_per_step": 10 * bytes_field,
                        "d2h_bytes_per_step": 12 * bytes_field, "steps": args.steps},
                "gpu_launches": int(launches),
                "gpu_launches_note": "this library's kernels in the timed steps (fmf_kernel_launches), including "
                                     "the viscous-solve iterations run inside the CUDA graph's conditional loop "
                                     "(the device-side stop rule), which an ncu launch list does not show "
                                     "(FMF_DEVICE_LOOP=0 runs the same kernels from the host)",
                "clocks": clk, "roofline": roofline, "step_roofline": step_roofline,
                "cpu_baseline": cpu, "mixed": mixed, "mixed_horizon": horizon, "fp64_pairs": fp64e,
                "second_workload": second,
                "adjoint": adjoint, "adjoint_mixed_forward": adjoint_m}
        print(json.dumps(line), flush=True)
    else:
        g.close()


if __name__ == "__main__":
    main()
