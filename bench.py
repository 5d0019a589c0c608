"""Benchmark: cell-updates/s of the full FP64 time step on one GB300.

Workload (the 256x128x128 case the metric is quoted on): two-phase Couette flow
with contact lines, density and viscosity ratio 10, perturbed x-stripe
interface, 60 deg walls, dt=2e-5 -- in reference axis order (ni, nj_wall, nk) =
(256, 128, 128).  One "step" is one full time step (main.f90:473-697).
value = interior cells x timed steps / device time (CUDA events on the
library's stream, device-resident state).  e2e = the same through the C-ABI with
host buffers (fmf_ctx_step_host): every step uploads the state's 10 input fields
from pinned host memory, steps, and returns the 12 result fields to host memory.

`--impl reference` times the CPU restatement of the reference's algorithm
(oracle/, the reference Fortran cannot be built here: no Fortran compiler) on
the host cores, same workload and metric.
"""
from __future__ import annotations

import argparse
import ctypes
import json
import os
import statistics
import subprocess
import sys
import time

REPO = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(REPO, "fel-multi-phase-flow_gb300"))
sys.path.insert(0, os.path.join(REPO, "oracle"))

WORKLOAD = "couette256"
# Per interior cell of one k_weno2 launch, from the ncu capture summarised in
# profiles/k_weno2_couette256.md (4,194,304 cells): DRAM bytes read + written
# (228.2 MB + 173.3 MB), and the executed FP64 instructions (DADD 955.7 M, DMUL
# 1219.5 M, DFMA 1885.8 M thread instructions); scaled to the workload by its cell
# count
WENO_TRAFFIC_PER_CELL = (228.228864e6 + 173.254144e6) / 4194304
WENO_FP64_INST_PER_CELL = (955711488 + 1219493888 + 1885798400) / 4194304
WENO_FP64_FLOPS_PER_CELL = (955711488 + 1219493888 + 2 * 1885798400) / 4194304
METRIC = "cell-updates/s/step plain FP64 vs mixed at stated error; adjoint/forward cost"
UNIT = "cell-updates/s"


def _peaks():
    try:
        with open(os.path.join(REPO, "MEASURED_PEAKS.json")) as f:
            return json.load(f), "measured"
    except Exception:
        return {"hbm_gbs": 6800.0, "bf16_tflops": 1900.0}, "fallback"


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


def cpu_baseline_sample(cfg, steps=1):
    """The oracle (C++/OpenMP restatement, all host threads) on a bounded sample."""
    import oracle
    from fmf import config as C
    s = oracle.Solver(cfg)
    st = s.initial_state()
    s.step(st, 1)  # warm
    t0 = time.perf_counter()
    s.step(st, steps)
    dt = time.perf_counter() - t0
    return cfg.cells * steps / dt, dt


def run_reference(args):
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    from fmf import config as C
    cfg = C.get(WORKLOAD)
    import oracle
    s = oracle.Solver(cfg)
    st = s.initial_state()
    s.step(st, args.warmup)
    t0 = time.perf_counter()
    s.step(st, args.steps)
    dt = time.perf_counter() - t0
    v = cfg.cells * args.steps / dt
    cores = os.cpu_count()
    line = {"impl": "reference", "metric": METRIC, "value": v, "unit": UNIT, "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * dt / args.steps,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
            "data": "synthetic",
            "config": {"workload": f"{WORKLOAD} 256x128x128 (ni,nj_wall,nk)", "precision": "fp64"},
            "cpu_baseline": {"value": v, "unit": UNIT, "cores": cores, "kind": "port",
                             "sample": f"{args.steps} full steps of {WORKLOAD} after {args.warmup} warm-up "
                                       "steps; the reference Fortran cannot be built here (no Fortran "
                                       "compiler), so its C++/OpenMP restatement oracle/fmf_oracle.cpp runs"},
            "e2e": {"value": v, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def mixed_case(name, steps, warmup, stream):
    """FP64 and mixed-precision steps on one workload: CUDA-event time per step of
    each (inputs resident, steps after `warmup`), and the per-field error of the mixed
    state against the FP64 state after the same warmup + steps from the same initial
    state."""
    import numpy as np
    import torch

    from fmf import capi
    from fmf import config as C

    cfg = C.get(name)
    out = {"workload": f"{name} {cfg.ni}x{cfg.nj}x{cfg.nk}", "steps": steps, "warmup": warmup}
    states = {}
    st = None
    for prec, key in ((capi.FMF_FP64, "fp64"), (capi.FMF_MIXED, "mixed")):
        g = capi.Stepper(cfg, precision=prec, stream=stream.cuda_stream)
        if st is None:
            st = g.initial_state()  # after the start-up boundary pass; the mixed run starts from it too
        else:
            g.upload(st)
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
    ref, mix = states["fp64"], states["mixed"]

    def rel(f):
        a, b = C.interior(mix[f]), C.interior(ref[f])
        return float(np.abs(a - b).max() / max(np.abs(b).max(), 1e-300))

    out["value_fp64"] = cfg.cells / (out["fp64_ms_per_step"] * 1e-3)
    out["value_mixed"] = cfg.cells / (out["mixed_ms_per_step"] * 1e-3)
    out["unit"] = UNIT
    out["speedup_vs_fp64"] = out["fp64_ms_per_step"] / out["mixed_ms_per_step"]
    out["steps_compared"] = warmup + steps
    out["max_rel_err_vs_fp64"] = {"phi": rel(9), "u": rel(0), "v": rel(1), "w": rel(2), "p": rel(6)}
    return out


def adjoint_cost(K, stream, every, workload="couette128"):
    """Adjoint/forward wall-clock ratio of the K-step rollout on a workload (default
    the 128x64x64 Couette workload, per-wall-cell angle 75 +- 5 deg), checkpoints
    every `every` steps (16 for K = 200 as the workload states, about sqrt(K);
    0: ceil(sqrt(K))):
    fmf_adj_rollout (J and all gradients) against fmf_adj_forward (J) with the same
    solver settings (viscous solve to the reference's 1e-3, transposed solve to
    1e-6), and against the graph-replayed production step (fmf_ctx_step)."""
    import math

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
    S.upload(st0)
    S.init_bc()
    S.step(2)
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
            "tolerances": {"sor": 1e-3, "adjoint": 1e-6}}


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="fmf", choices=["fmf", "reference"])
    ap.add_argument("--workload", default=WORKLOAD)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--adjoint-steps", type=int, default=200,
                    help="K of the adjoint-cost measurement (0: skip)")
    ap.add_argument("--mixed-workload", default="droplet512",
                    help="second FP64-vs-mixed measurement (the sessile-drop workload; '' to skip)")
    ap.add_argument("--adjoint-every", type=int, default=16,
                    help="checkpoint interval of the adjoint rollout (0: ceil(sqrt(K)))")
    ap.add_argument("--adjoint-workload", default="couette128",
                    help="workload of the adjoint-cost measurement (droplet256 with --adjoint-steps 500 "
                         "--adjoint-every 0: the 256x128x128 sessile drop, K = 500, ceil(sqrt(K)) = 23)")
    ap.add_argument("--precision", default="fp64", choices=["fp64", "mixed", "adjoint"], help="--profile only")
    ap.add_argument("--profile", action="store_true",
                    help="no timing: start-up pass, --warmup steps, then --steps steps (for ncu launch lists)")
    args = ap.parse_args()
    if args.impl == "reference":
        run_reference(args)
        return
    if args.profile:
        from fmf import build as fbuild
        from fmf import capi
        from fmf import config as C
        fbuild.build()
        if args.precision == "adjoint":
            # --steps K of the adjoint rollout on the workload (for ncu launch lists)
            from fmf.adjoint import Adjoint
            cfg = C.get(args.workload)
            A = Adjoint(cfg, sor_tol=1e-3, sor_max=21, adj_tol=1e-6, adj_max=200)
            st0 = C.raw_state(cfg)
            walls = C.wall_arrays(cfg)
            A.rollout(max(1, args.warmup), st0, walls)
            J, _ = A.rollout(args.steps, st0, walls)
            print(json.dumps({"profile": args.workload, "adjoint_steps": args.steps, "J": J,
                              "iterations": A.iterations()}))
            A.close()
            return
        prec = capi.FMF_MIXED if args.precision == "mixed" else capi.FMF_FP64
        g = capi.Stepper(C.get(args.workload), precision=prec)
        g.initial_state()
        g.step(args.warmup)
        g.sync()
        g.step(args.steps)
        g.sync()
        print(json.dumps({"profile": args.workload, "sor_iterations": g.sor_iterations()}))
        g.close()
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

    # e2e: host buffers through the C-ABI, every step uploads the 10 input fields of
    # the state from pinned host memory (phin is written by the step before it is
    # read) and returns the 12 result fields to it (fmf_ctx_step_host: part of the
    # upload and the result fields that are final early overlap the step)
    pinned = torch.empty((12,) + cfg.shape, dtype=torch.float64, pin_memory=True)
    host = pinned.numpy()
    host[:] = g.get_state()
    bytes_field = cfg.shape[0] * cfg.shape[1] * cfg.shape[2] * 8
    e2e_steps = max(1, min(args.steps, 5))
    g.step_host(host, host)  # the host-buffer path's own first call (copy stream, events)
    barrier()
    t0 = time.perf_counter()
    for _ in range(e2e_steps):
        g.step_host(host, host)
    e2e_dt = replicas.max_over_ranks(time.perf_counter() - t0)
    e2e_value = replicas.throughput(cfg.cells, e2e_steps, e2e_dt)

    # Dominant kernel: WENO5 advection of both velocity levels (k_weno2, stage 0),
    # FP64-pipe bound.  The FP64 roofline counts executed FP64 instructions (ncu
    # DADD + DMUL + DFMA per cell, WENO_FP64_INST_PER_CELL) against the FP64 pipe's
    # instruction rate, half the FMA-chain flop rate fmf_measure_fma_rate measures
    # live (an FMA is one instruction and two flops).  Also reported: the executed
    # flops (FMA = 2) and the rate of the reference formula's flops (weno5.h, both
    # one-sided reconstructions: 2766 per cell for the two calls), which exceeds
    # the peak because the kernel evaluates the upwind side only, in fewer
    # operations.  Algorithmic bytes 12 words per cell (6 fields in, 6 out); HBM
    # peak from MEASURED_PEAKS.json.
    ms_stage = ctypes.c_float()
    capi.check(L.fmf_ctx_time_stage(g.h, 0, 5, ctypes.byref(ms_stage)), "time_stage")
    peaks, peak_kind = _peaks()
    fp64 = ctypes.c_double()
    L.fmf_measure_fma_rate.argtypes = [ctypes.c_int, ctypes.POINTER(ctypes.c_double)]
    capi.check(L.fmf_measure_fma_rate(1, ctypes.byref(fp64)), "fma rate")
    t_weno = ms_stage.value * 1e-3
    inst_rate = WENO_FP64_INST_PER_CELL * cfg.cells / t_weno / 1e12
    inst_peak = fp64.value / 2.0
    gbs = 12 * 8 * cfg.cells / t_weno / 1e9
    roofline = {"bound": "fp64", "achieved": inst_rate, "peak": inst_peak, "unit": "T FP64 instructions/s",
                "frac": inst_rate / inst_peak,
                "traffic": WENO_TRAFFIC_PER_CELL * cfg.cells,
                "kernel": "k_weno2 (both cal_advu_weno5 calls of the step)", "kernel_ms": ms_stage.value,
                "fp64_inst_per_cell": WENO_FP64_INST_PER_CELL,
                "executed_tflops": WENO_FP64_FLOPS_PER_CELL * cfg.cells / t_weno / 1e12,
                "reference_formula_tflops": 2766.0 * cfg.cells / t_weno / 1e12,
                "fma_peak_tflops": fp64.value,
                "peak_source": "FP64 FMA chains measured live (fmf_measure_fma_rate), one instruction per FMA; "
                               "HBM peak " + peak_kind,
                "hbm": {"achieved": gbs, "peak": peaks["hbm_gbs"], "unit": "GB/s", "frac": gbs / peaks["hbm_gbs"]}}
    # Mixed precision (FP32 WENO5 / MTHINC Newton+fluxes / SOR sweeps, FP64 pressure,
    # projection, divergence, volume sums and state): throughput on the same workload,
    # and the error of phi, u, v, w, p against the FP64 step after the same steps
    # from the same initial state.
    gm = capi.Stepper(cfg, precision=capi.FMF_MIXED, stream=stream.cuda_stream)
    gm.upload(st)
    gm.step(args.warmup)
    gm.sync()
    barrier()
    e0.record(stream)
    gm.step(args.steps)
    e1.record(stream)
    e1.synchronize()
    ms_mixed = replicas.max_over_ranks(e0.elapsed_time(e1))
    n_err = args.warmup + args.steps
    g.upload(st)
    g.step(n_err)
    ref = g.get_state()
    gm.upload(st)
    gm.step(n_err)
    mix = gm.get_state()
    ms_stage_m = ctypes.c_float()
    capi.check(L.fmf_ctx_time_stage(gm.h, 0, 5, ctypes.byref(ms_stage_m)), "time_stage mixed")
    gm.close()

    def rel(f):
        a, b = C.interior(mix[f]), C.interior(ref[f])
        return float(np.abs(a - b).max() / max(np.abs(b).max(), 1e-300))

    mixed = {"value": replicas.throughput(cfg.cells, args.steps, ms_mixed * 1e-3), "unit": UNIT,
             "ms_per_step": ms_mixed / args.steps, "speedup_vs_fp64": ms / ms_mixed,
             "steps_compared": n_err,
             "max_rel_err_vs_fp64": {"phi": rel(9), "u": rel(0), "v": rel(1), "w": rel(2), "p": rel(6)},
             "weno5_ms": ms_stage_m.value,
             "precision": "fp32: WENO5, MTHINC Newton + Gauss-point fluxes, CSF normals and curvature, viscous "
                          "sweeps on FP32 corrections (FP64 residual, one refinement step); fp64: state, "
                          "pressure FFT+TDMA, projection, divergence, volume sums"}
    mixed_droplet = None
    if rank == 0 and args.mixed_workload:
        g.close()
        mixed_droplet = mixed_case(args.mixed_workload, 5, 3, stream)
    adjoint = None
    if rank == 0 and args.adjoint_steps > 0:
        adjoint = adjoint_cost(args.adjoint_steps, stream, args.adjoint_every, args.adjoint_workload)
    cpu = None
    if rank == 0 and not args.no_cpu_baseline:
        v, dt = cpu_baseline_sample(cfg, 1)
        cpu = {"value": v, "unit": UNIT, "cores": os.cpu_count(), "kind": "port",
               "sample": f"1 full step of {args.workload} after 1 warm-up step ({dt:.1f} s), oracle/fmf_oracle.cpp "
                         "C++/OpenMP restatement, all host threads"}
    if rank == 0:
        line = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
                "warmup": args.warmup, "ms_per_step": ms / args.steps, "higher_is_better": True,
                "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
                "config": {"workload": f"{args.workload} {cfg.ni}x{cfg.nj}x{cfg.nk} (ni,nj_wall,nk)",
                           "precision": "fp64", "l2": "inputs larger than L2 (state + work arrays ~GBs/step)",
                           "sor_iterations_mean": float(np.mean(iters)) if iters else None,
                           "parallelism": "replicas" if world > 1 else "single"},
                "e2e": {"value": e2e_value, "unit": UNIT, "h2d_bytes_per_step": 10 * bytes_field,
                        "d2h_bytes_per_step": 12 * bytes_field},
                "gpu_launches": int(launches), "clocks": clk, "roofline": roofline, "cpu_baseline": cpu,
                "mixed": mixed, "mixed_droplet": mixed_droplet, "adjoint": adjoint}
        print(json.dumps(line), flush=True)
    g.close()


if __name__ == "__main__":
    main()
