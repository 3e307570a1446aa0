"""Benchmark of the convective hot path: FP64 cell-updates/s per SSPRK3 substep.

Workload (default): 2D five-equation Allaire model, two species
(gamma 1.4 / 1.67, density ratio 3), one 1024x1024 FP64 patch, ghost width 4,
WCNS6-LD + HLLC-HLL, tanh interface with a seeded 16-mode perturbation hit by
a Mach 1.5 shock (seeded synthetic inputs with the benchmark's shapes).  A
step is one SSPRK3 time step (three substeps) of the level, run by the batched
form (one persistent kernel per substep, each substep a captured CUDA graph).

  value   device-timed cell-updates/s with the state resident in HBM
  e2e     the same through the public API (hamers_gb300.flow.BatchedLevel)
          with the state copied host->device (pinned) and back every step,
          advancing the same trajectory as the device-timed loop
Working set per step (~0.5 GB of state and scratch) exceeds L2 (129 MB).

--impl reference times the reference algorithm on the host cores: the CPU
oracle (a restatement of the reference's FP64 code; the reference itself
needs SAMRAI/MPI/HDF5 and is not built here) with one std::thread per core
advancing one sub-patch each, as one MPI rank per core would.
"""
import argparse
import ctypes
import json
import os
import platform
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

METRIC = "FP64 cell-updates/s per RK substep"
UNIT = "cell-updates/s"
WORKLOAD = "2D five-eqn Allaire 1024x1024, WCNS6-LD + HLLC-HLL, Mach 1.5 shock-interface, SSPRK3"
NEQ, NCOMP = 6, 7
# Algorithmic FP64 operations per cell-update of this workload (add, sub, mul,
# div, sqrt, fabs, fmin, fmax counted 1 each), counted by running the oracle
# on an operation-counting scalar type (oracle/hmr_opcount.cpp) on this
# problem at its full size, 1024x1024 (oracle/opcount_workloads.py).
ALG_FP64_OPS_PER_CELL = 6006.0
# Algorithmic HBM bytes per cell-update: SSPRK3 stage 0 reads Q^n and writes
# Q^(1) (2*8*neq B), stages 1 and 2 read Q^n, Q^(k) and write Q^(k+1)
# (3*8*neq B); averaged over the three substeps.
ALG_BYTES_PER_CELL = 8 * NEQ * (2 + 3 + 3) / 3.0


# Algorithmic FP64 operations per cell-update of the other workloads, counted the same way
# over every patch of each workload (oracle/opcount_workloads.py).
ALG_FP64_OPS_C1 = 1886.4      # 2D single species WCNS5-JS, one 256^2 patch
ALG_FP64_OPS_C3 = 3583.1      # 3D single species WCNS5-JS, 512 uneven cubic patches
ALG_FP64_OPS_C5 = 11061.9     # 3D five-equation WCNS6-LD, 3-level layout of 474 uneven patches


def alg_bytes(neq, stages=(0, 1, 2)):
    """Algorithmic HBM bytes per cell-update, averaged over the given SSPRK3 stages: stage 0
    reads Q^n and writes Q^(1); stages 1 and 2 read two states and write one."""
    return sum(8 * neq * (2 if s == 0 else 3) for s in stages) / len(stages)


def bench_config(n):
    """The workload both arms time (identical in the GPU and the reference arm's lines)."""
    return {"workload": WORKLOAD, "cells": n * n, "substeps_per_step": 3,
            "l2": "working set per step ~0.5 GB > 129 MB L2 (no flush)", "parallelism": "replicas"}


def roofline_fracs(cell_updates_per_s, ops_per_cell, bytes_per_cell, fp64_peak, hbm_peak):
    """FP64 (algorithmic ops against the measured DFMA peak) and HBM (algorithmic bytes against
    the measured copy bandwidth) fractions of a cell-update rate."""
    out = {}
    if ops_per_cell:
        tf = ops_per_cell * cell_updates_per_s / 1e12
        out["fp64"] = {"achieved": tf, "peak": fp64_peak, "unit": "TFLOP/s", "ops_per_cell_update": ops_per_cell,
                       "frac": tf / fp64_peak if fp64_peak else None}
    gbs = bytes_per_cell * cell_updates_per_s / 1e9
    out["hbm"] = {"achieved": gbs, "peak": hbm_peak, "unit": "GB/s", "bytes_per_cell_update": bytes_per_cell,
                  "frac": gbs / hbm_peak}
    return out


# DRAM traffic of one level_kernel launch of the default workload, bytes (ncu capture).
LEVEL_KERNEL_TRAFFIC_BYTES = 413476608 + 248229120


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--n", type=int, default=1024)
    ap.add_argument("--precision", default="fast", choices=["fast", "exact"])
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--form", default="batched", choices=["batched", "patch"],
                    help="batched: one persistent kernel per substep; patch: per-phase kernels of one patch")
    ap.add_argument("--no-uneven", action="store_true",
                    help="skip the batched-vs-per-patch measurement on uneven 3D patches")
    ap.add_argument("--no-peak", action="store_true", help="skip the FP64 peak microbenchmark")
    ap.add_argument("--no-adjoint", action="store_true", help="skip the adjoint/forward cost measurement")
    ap.add_argument("--c4-only", action="store_true",
                    help="time only the C4 forward (Navier-Stokes Taylor-Green 128^3) for --steps steps after "
                         "--warmup steps and print its line (used for the C4 launch list)")
    ap.add_argument("--c4", action="store_true",
                    help="check the 3D Navier-Stokes Taylor-Green gradient along 16 directions (default 4)")
    ap.add_argument("--no-c4", action="store_true",
                    help="skip the 3D Navier-Stokes Taylor-Green workload (128^3) and its adjoint")
    ap.add_argument("--no-c5", action="store_true",
                    help="skip the 3-level 3D five-equation batched substep + amplitude adjoint")
    ap.add_argument("--no-c1", action="store_true",
                    help="skip the 2D single-species 256^2 per-patch workload")
    ap.add_argument("--uneven-patches", type=int, default=512)
    ap.add_argument("--per-patch-busy", action="store_true",
                    help="run one extra per-patch uneven-patch step inside an NVTX range (per_patch_step) for "
                         "an ncu launch list of exactly that step")
    ap.add_argument("--uneven-only", action="store_true",
                    help="run only the uneven-patch batched-vs-per-patch measurement and print it")
    return ap.parse_args()


def dist_env():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return rank, world, local


def replica_throughput(local_ms, cells_per_step, steps, world, device):
    """Whole-job throughput of `world` independent replicas (one per GPU, no
    data-path collective): the timed region is the slowest rank's (max over
    ranks), every rank advanced cells_per_step * steps cell-updates.
    Returns (max_ms, cell-updates/s)."""
    total_ms = float(local_ms)
    if world > 1:
        import torch
        import torch.distributed as dist
        t = torch.tensor([total_ms], dtype=torch.float64, device=device)
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        total_ms = float(t.item())
    return total_ms, world * cells_per_step * steps / (total_ms * 1e-3)


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled during the timed region."""

    FIELDS = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.hw_slowdown,"
              "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
              "clocks_event_reasons.sw_power_cap")

    def __init__(self, index=0):
        self.index = index
        self.samples = []
        self._stop = threading.Event()
        self._t = None

    def _run(self):
        while not self._stop.is_set():
            try:
                out = subprocess.run(["nvidia-smi", "-i", str(self.index), "--query-gpu=" + self.FIELDS,
                                      "--format=csv,noheader,nounits"], capture_output=True, text=True,
                                     timeout=5).stdout.strip()
                if out:
                    self.samples.append([v.strip() for v in out.split(",")])
            except Exception:
                pass
            self._stop.wait(0.2)

    def __enter__(self):
        self._t = threading.Thread(target=self._run, daemon=True)
        self._t.start()
        return self

    def __exit__(self, *a):
        self._stop.set()
        self._t.join(timeout=10)

    def summary(self):
        if not self.samples:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"], "samples": 0}
        sm = [float(s[0]) for s in self.samples if s[0].replace(".", "").isdigit()]
        mx = [float(s[1]) for s in self.samples if s[1].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for s in self.samples for i in range(4) if "Active" in s[3 + i]
                          and not s[3 + i].startswith("Not")})
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": reasons, "samples": len(self.samples)}


def measured_peaks():
    path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    try:
        with open(path) as f:
            return json.load(f), "measured"
    except Exception:
        return {"hbm_gbs": 6800.0}, "fallback"


def fp64_peak_tflops():
    from hamers_gb300 import build as B
    lib = ctypes.CDLL(B.PEAK_LIB)
    lib.hmr_measure_fp64_fma.argtypes = [ctypes.POINTER(ctypes.c_double)] * 2
    tf, ms = ctypes.c_double(), ctypes.c_double()
    rc = lib.hmr_measure_fp64_fma(ctypes.byref(tf), ctypes.byref(ms))
    return tf.value if rc == 0 else None


def workload(n):
    from hamers_gb300 import problems as P
    Q, dx, dt = P.shock_interface_2d(N=n, seed=1)
    return Q, dx, dt


def uneven_batched_vs_patch(args, flow):
    """3D single species, WCNS5-JS, 2 levels of uneven cubic patches (side U{16..64},
    seed 2), ~45 M cells: one SSPRK3 step of every patch, batched (one persistent kernel
    per substep over the level worklist, CUDA graph) vs per-patch launches (the
    drop-in path, patch after patch on one stream).  Ghosts are refilled per
    stage by each patch's own zero-gradient fill in both forms."""
    import torch
    from hamers_gb300 import problems as P
    patches = P.blobs_patches_3d_device(num_patches=args.uneven_patches)
    cells = sum(n[0] * n[1] * n[2] for n, _, _ in patches)
    fm = flow.FlowModel("SINGLE_SPECIES", 3, [1.4])
    rec = flow.ConvectiveFluxReconstructor("WCNS5_JS_HLLC_HLL", fm, precision=args.precision)
    dt = 0.2 * min(dx[0] for _, dx, _ in patches) / 2.5
    Q0 = [Q.clone() for _, _, Q in patches]
    stream = torch.cuda.current_stream()
    # batched
    lv = flow.BatchedLevel(rec, [(n, dx) for n, dx, _ in patches])
    for i, (_, _, Q) in enumerate(patches):
        lv.bind(i, Q)
    tuned = lv.autotune(dt)
    split = lv.work_split()
    for i, (_, _, Q) in enumerate(patches):
        Q.copy_(Q0[i])
    lv.step(dt)
    torch.cuda.synchronize()
    lv.check()
    reps = 2
    e = [torch.cuda.Event(enable_timing=True) for _ in range(2)]
    e[0].record(stream)
    for _ in range(reps):
        lv.step(dt)
    e[1].record(stream)
    torch.cuda.synchronize()
    lv.check()
    t_batched = e[0].elapsed_time(e[1]) / reps
    lv.close()
    # per-patch
    for i, (_, _, Q) in enumerate(patches):
        Q.copy_(Q0[i])
    eu = flow.Euler(rec)
    work = []
    big = max(patches, key=lambda t: t[0][0] * t[0][1] * t[0][2])
    rec.reserve(flow.Patch(big[0], big[1], big[2]))
    for n, dx, Q in patches:
        work.append([flow.Patch(n, dx, q) for q in (Q, torch.empty_like(Q), torch.empty_like(Q))])

    def step_patches():
        for views in work:
            Qs = [v.data for v in views]
            for s_ in range(3):
                eu.fillGhosts(views[s_], [0, 0, 0])
                eu.substep(views[s_], s_, Qs[:s_ + 1], dt, Qs[0] if s_ == 2 else Qs[s_ + 1])

    step_patches()
    torch.cuda.synchronize()
    e[0].record(stream)
    for _ in range(reps):
        step_patches()
    e[1].record(stream)
    torch.cuda.synchronize()
    t_patch = e[0].elapsed_time(e[1]) / reps
    if args.per_patch_busy:
        mark_per_patch_step(step_patches)
    rec.close()
    cu = 3 * cells
    return {"workload": f"3D single species WCNS5-JS + HLLC-HLL, {len(patches)} uneven cubic patches "
                        f"(side 16-64, 2 levels), {cells} cells, SSPRK3 step", "cells": cells,
            "batched_cell_updates_per_s": cu / (t_batched * 1e-3),
            "per_patch_cell_updates_per_s": cu / (t_patch * 1e-3),
            "batched_over_per_patch": t_patch / t_batched,
            "batched_ms_per_step": t_batched, "per_patch_ms_per_step": t_patch,
            "launch_shape": {"threads": tuned[0], "blocks_per_sm": tuned[1]},
            "work_split": {"chunk_blocks": split[0], "cell_phases": "grid-stride" if split[1] & 1 else "chunks",
                           "faces": "sorted" if split[1] & 2 else "in order"},
            "batched_roofline": roofline_fracs(cu / (t_batched * 1e-3), ALG_FP64_OPS_C3, alg_bytes(5),
                                               args.fp64_peak, args.hbm_peak),
            "per_patch_roofline": roofline_fracs(cu / (t_patch * 1e-3), ALG_FP64_OPS_C3, alg_bytes(5),
                                                 args.fp64_peak, args.hbm_peak)}


def mark_per_patch_step(step):
    """Runs one more per-patch step inside an NVTX range named per_patch_step, so that a launch
    list (ncu --nvtx --nvtx-include per_patch_step/) holds exactly that step's kernels; their
    summed device time against the step's device-timed wall time gives the share of the step the
    GPU spends in kernels."""
    import torch
    torch.cuda.synchronize()
    torch.cuda.nvtx.range_push("per_patch_step")
    step()
    torch.cuda.synchronize()
    torch.cuda.nvtx.range_pop()


def adjoint_cost(args, flow, Qnp, n, dx, dt, reps=3):
    """Cost of the hand-written adjoint against the forward on the same workload.

    One SSPRK3 step of the patch (zero-gradient x, periodic y): forward = ghost
    fill + fused substep for the three stages (per-patch form); adjoint = the
    three substep VJPs plus the three ghost-fill VJPs of the same step, given its
    stage states.  Both device-timed with CUDA events, mean of `reps` steps."""
    import torch
    fm = flow.FlowModel("FIVE_EQN_ALLAIRE", 2, [1.4, 1.67])
    per = [0, 1]
    out = {}
    Q0 = torch.from_numpy(Qnp).cuda()
    stream = torch.cuda.current_stream()
    e = [torch.cuda.Event(enable_timing=True) for _ in range(2)]
    for prec in ("fast", "exact"):
        rec = flow.ConvectiveFluxReconstructor("WCNS6_LD_HLLC_HLL", fm, precision=prec)
        drv = PatchDriver(flow, rec, n, dx, Q0.clone(), per)
        drv.step(dt)
        torch.cuda.synchronize()
        e[0].record(stream)
        for _ in range(reps):
            drv.step(dt)
        e[1].record(stream)
        torch.cuda.synchronize()
        out["forward_%s_ms_per_step" % prec] = e[0].elapsed_time(e[1]) / reps
        if prec == "exact":
            # stage states of one step, ghost-filled as the forward sees them
            eu = drv.eu
            X = Q0.clone()
            S1, S2 = torch.empty_like(X), torch.empty_like(X)
            views = [flow.Patch([n, n], dx, q) for q in (X, S1, S2)]
            eu.fillGhosts(views[0], per)
            eu.substep(views[0], 0, [X], dt, S1)
            eu.fillGhosts(views[1], per)
            eu.substep(views[1], 1, [X, S1], dt, S2)
            eu.fillGhosts(views[2], per)
            Xb = torch.randn_like(X)
            bufs = [torch.zeros_like(X) for _ in range(3)]

            def reverse():
                for b in bufs:
                    b.zero_()
                eu.substepVJP(views[0], 2, [X, S1, S2], dt, Xb, bufs)
                eu.fillGhostsVJP(flow.Patch([n, n], dx, bufs[2]), per)
                eu.substepVJP(views[0], 1, [X, S1], dt, bufs[2], bufs[:2])
                eu.fillGhostsVJP(flow.Patch([n, n], dx, bufs[1]), per)
                eu.substepVJP(views[0], 0, [X], dt, bufs[1], bufs[:1])
                eu.fillGhostsVJP(flow.Patch([n, n], dx, bufs[0]), per)

            reverse()
            torch.cuda.synchronize()
            e[0].record(stream)
            for _ in range(reps):
                reverse()
            e[1].record(stream)
            torch.cuda.synchronize()
            out["adjoint_ms_per_step"] = e[0].elapsed_time(e[1]) / reps
        rec.close()
    out["adjoint_over_forward_fast"] = out["adjoint_ms_per_step"] / out["forward_fast_ms_per_step"]
    out["adjoint_over_forward_exact"] = out["adjoint_ms_per_step"] / out["forward_exact_ms_per_step"]
    out["workload"] = f"{WORKLOAD}; one SSPRK3 step, per-patch form, adjoint with given stage states"
    return out


def c5_level_and_adjoint(args, flow, base=128, reps=3):
    """3D five-equation shock / perturbed interface (gamma 1.4/1.09, density ratio 3, Mach 1.5)
    on a seeded 3-level layout (ratio 2, ~512^3 finest-equivalent) of uneven patches with sides
    U{16..64} (seed 4), WCNS6-LD + HLLC-HLL: one batched RK substep over every patch of every
    level (one persistent kernel, ghosts from the analytic initial state) against per-patch
    launches, and the adjoint of that substep with respect to the 64 interface-mode amplitudes
    (per-patch VJPs chained through the differentiable initial condition)."""
    import torch
    from hamers_gb300 import problems as P
    layout = P.amr_layout_3d(base=base, seed=4)
    amps, waves, phases = P.shock_interface_3d_modes(64, seed=4)
    a = torch.tensor(amps, dtype=torch.float64, device="cuda")
    finest = min(dx[0] for _, _, _, dx in layout)
    fm = flow.FlowModel("FIVE_EQN_ALLAIRE", 3, [1.4, 1.09])
    rec = flow.ConvectiveFluxReconstructor("WCNS6_LD_HLLC_HLL", fm, precision=args.precision)
    states = [P.shock_interface_3d_patch(lo, n, dx, a, waves, phases, finest) for _, lo, n, dx in layout]
    cells = sum(n[0] * n[1] * n[2] for _, _, n, _ in layout)
    # dt at CFL 0.4 on the finest level (post-shock speed + sound speed bound)
    dt = 0.4 * finest / (3.0 * 3.0)
    lv = flow.BatchedLevel(rec, [(n, dx) for _, _, n, dx in layout])
    for p, Q in enumerate(states):
        lv.bind(p, Q)
        lv.set_periodic(p, [2, 2, 2])
    tuned = lv.autotune(dt)   # substep 0 reads the bound state and writes the level's own output
    split = lv.work_split()
    stream = torch.cuda.current_stream()
    e = [torch.cuda.Event(enable_timing=True) for _ in range(2)]
    lv.substep(0, dt)
    torch.cuda.synchronize()
    lv.check()
    e[0].record(stream)
    for _ in range(reps):
        lv.substep(0, dt)
    e[1].record(stream)
    torch.cuda.synchronize()
    lv.check()
    t_batched = e[0].elapsed_time(e[1]) / reps
    # per-patch launches of the same substep
    eu = flow.Euler(rec)
    big = max(range(len(layout)), key=lambda i: np.prod(layout[i][2]))
    rec.reserve(flow.Patch(layout[big][2], layout[big][3], states[big]))
    outs = [torch.empty_like(Q) for Q in states]
    views = [flow.Patch(n, dx, Q) for (_, _, n, dx), Q in zip(layout, states)]

    def per_patch():
        for v, Q, o in zip(views, states, outs):
            eu.substep(v, 0, [Q], dt, o)

    per_patch()
    torch.cuda.synchronize()
    e[0].record(stream)
    for _ in range(reps):
        per_patch()
    e[1].record(stream)
    torch.cuda.synchronize()
    t_patch = e[0].elapsed_time(e[1]) / reps
    # adjoint of J = sum_p <w_p, Q_out,p> (w_p seeded) with respect to the 64 amplitudes
    gen = torch.Generator(device="cuda")
    gen.manual_seed(4)
    W = [torch.randn(Q.shape, dtype=torch.float64, device="cuda", generator=gen) for Q in states]
    bars = [torch.zeros_like(Q) for Q in states]

    def reverse():
        for v, Q, w, b in zip(views, states, W, bars):
            b.zero_()
            eu.substepVJP(v, 0, [Q], dt, w, [b])

    reverse()
    torch.cuda.synchronize()
    e[0].record(stream)
    for _ in range(reps):
        reverse()
    e[1].record(stream)
    torch.cuda.synchronize()
    t_adj = e[0].elapsed_time(e[1]) / reps
    # the same adjoint batched over the level (hmr_level_substep_vjp), at the stage state the
    # level's forward substep leaves (slot 0: the bound states, ghosts provided)
    bars_b = [[torch.zeros_like(Q)] for Q in states]

    def reverse_batched():
        for b in bars_b:
            b[0].zero_()
        lv.substepVJP(0, dt, W, bars_b)

    reverse_batched()
    torch.cuda.synchronize()
    e[0].record(stream)
    for _ in range(reps):
        reverse_batched()
    e[1].record(stream)
    torch.cuda.synchronize()
    t_adj_b = e[0].elapsed_time(e[1]) / reps
    same_bits = all(torch.equal(b[0], q) for b, q in zip(bars_b, bars))
    a_req = a.clone().requires_grad_(True)
    grad = torch.zeros_like(a)
    for (_, lo, n, dx), b in zip(layout, bars):
        Qa = P.shock_interface_3d_patch(lo, n, dx, a_req, waves, phases, finest)
        grad += torch.autograd.grad(Qa, a_req, grad_outputs=b)[0]
    lv.close()
    rec.close()
    return {"workload": "3D five-eqn Allaire shock/interface, 3 levels (ratio 2, 512^3 finest-equivalent), "
                        f"{len(layout)} uneven patches (side 16-64, seed 4), WCNS6-LD + HLLC-HLL, one RK substep; "
                        "adjoint w.r.t. 64 interface-mode amplitudes",
            "cells": cells, "patches": len(layout), "precision": args.precision,
            "batched_substep_ms": t_batched, "batched_cell_updates_per_s": cells / (t_batched * 1e-3),
            "per_patch_substep_ms": t_patch, "per_patch_cell_updates_per_s": cells / (t_patch * 1e-3),
            "batched_over_per_patch": t_patch / t_batched,
            "launch_shape": {"threads": tuned[0], "blocks_per_sm": tuned[1]},
            "work_split": {"chunk_blocks": split[0], "cell_phases": "grid-stride" if split[1] & 1 else "chunks",
                           "faces": "sorted" if split[1] & 2 else "in order"},
            "batched_roofline": roofline_fracs(cells / (t_batched * 1e-3), ALG_FP64_OPS_C5, alg_bytes(7, (0,)),
                                               args.fp64_peak, args.hbm_peak),
            "per_patch_roofline": roofline_fracs(cells / (t_patch * 1e-3), ALG_FP64_OPS_C5, alg_bytes(7, (0,)),
                                                 args.fp64_peak, args.hbm_peak),
            "adjoint_per_patch_substep_ms": t_adj, "adjoint_batched_substep_ms": t_adj_b,
            "adjoint_batched_over_batched_forward": t_adj_b / t_batched,
            "adjoint_per_patch_over_per_patch_forward": t_adj / t_patch,
            "adjoint_batched_equals_per_patch": same_bits,
            "grad_amplitudes_norm": float(grad.norm())}


def c4_navier_stokes(args, flow, N=128, nsteps=100, every=10, fd_dirs=16, fd_steps=10):
    """3D Navier-Stokes Taylor-Green vortex, 128^3 periodic on [0, 2 pi)^3 (Mach 0.1, Re 1600,
    Pr 0.72, gamma 1.4), WCNS5-JS + HLLC-HLL with the fourth-order midpoint diffusive flux,
    per-patch fused substeps: 100 SSPRK3 steps checkpointed every 10, then the reverse sweep
    (recompute + substep VJPs) for the gradient of the final kinetic energy.  The gradient is
    checked against central differences along 16 seeded directions (seed 3) over the first
    checkpoint segment (10 steps) of the same problem."""
    import torch
    from hamers_gb300 import problems as P
    Qnp, dx = P.taylor_green_3d(N)
    tr = P.taylor_green_transport()
    dt = P.taylor_green_dt(Qnp[:, 4:-4, 4:-4, 4:-4], dx, mu=tr["species_mu"], prandtl=tr["species_Pr"])
    fm = flow.FlowModel("SINGLE_SPECIES", 3, [1.4], transport=tr)
    rec = flow.ConvectiveFluxReconstructor("WCNS5_JS_HLLC_HLL", fm, precision=args.precision,
                                           diffusive_flux_reconstructor="MIDPOINT_FOURTH_ORDER")
    ns = flow.NavierStokes(rec)
    n, per = [N] * 3, [1, 1, 1]
    dV = dx[0] * dx[1] * dx[2]
    Q0 = torch.from_numpy(Qnp).cuda()
    stream = torch.cuda.current_stream()
    e = [torch.cuda.Event(enable_timing=True) for _ in range(4)]

    def kinetic_and_grad(Q):
        rho = Q[0]
        u = Q[1:4] / rho
        G = torch.zeros_like(Q)
        G[0, 4:-4, 4:-4, 4:-4] = (-0.5 * (u * u).sum(dim=0) * dV)[4:-4, 4:-4, 4:-4]
        G[1:4, 4:-4, 4:-4, 4:-4] = (u * dV)[:, 4:-4, 4:-4, 4:-4]
        J = 0.5 * float(((Q[1:4] * Q[1:4]).sum(dim=0) / rho)[4:-4, 4:-4, 4:-4].sum()) * dV
        return J, G

    # warm-up (graph-free per-patch path: fill + 4-5 kernels per substep)
    Qw = Q0.clone()
    flow.RungeKuttaLevelIntegrator(ns, flow.Patch(n, dx, Qw), per).advance(dt, nsteps=2)
    torch.cuda.synchronize()
    Q = Q0.clone()
    integ = flow.RungeKuttaLevelIntegrator(ns, flow.Patch(n, dx, Q), per)
    e[0].record(stream)
    integ.advance(dt, nsteps=nsteps, checkpoint_every=every)
    e[1].record(stream)
    torch.cuda.synchronize()
    t_fwd = e[0].elapsed_time(e[1])
    J, G = kinetic_and_grad(Q)
    e[2].record(stream)
    grad = integ.adjoint(G)
    e[3].record(stream)
    torch.cuda.synchronize()
    t_adj = e[2].elapsed_time(e[3])
    cells = N ** 3
    out = {"workload": "3D Navier-Stokes Taylor-Green vortex 128^3 periodic, Mach 0.1, Re 1600, Pr 0.72, "
                       "WCNS5-JS + HLLC-HLL + 4th-order midpoint diffusive flux, 100 SSPRK3 steps, "
                       "checkpoint every 10, gradient of the final kinetic energy",
           "precision": args.precision, "dt": dt, "steps": nsteps,
           "forward_ms": t_fwd, "forward_cell_updates_per_s": cells * 3 * nsteps / (t_fwd * 1e-3),
           "adjoint_ms": t_adj, "adjoint_over_forward": t_adj / t_fwd,
           "vjp_over_forward_est": (t_adj - t_fwd) / t_fwd,
           "note": "adjoint = the whole reverse sweep: each segment's forward recomputed from its checkpoint "
                   "(about one forward) plus the substep and ghost-fill VJPs; vjp_over_forward_est subtracts "
                   "one forward",
           "final_kinetic_energy": J}
    # gradient with respect to the initial velocity: for u -> u + du at fixed rho and p,
    # d(rho u) = rho du and dE = rho u.du, so dJ/du = rho (dJ/d(rho u) + u dJ/dE)
    rho0 = Q0[0]
    u0 = Q0[1:4] / rho0
    grad_u = rho0 * (grad[1:4] + u0 * grad[4])
    out["grad_initial_velocity_norm"] = float(grad_u[:, 4:-4, 4:-4, 4:-4].norm())
    # gradient check over the first checkpoint segment, at the vortex with smooth 0.05
    # perturbations (the exact vortex sits on non-differentiable points of the flux: w = 0
    # and mirror-symmetric faces), along 16 smooth random initial-velocity directions (seed 3)
    Qp0 = torch.from_numpy(P.taylor_green_3d(N, perturb=0.05)[0]).cuda()
    Qa = Qp0.clone()
    seg = flow.RungeKuttaLevelIntegrator(ns, flow.Patch(n, dx, Qa), per)
    seg.advance(dt, nsteps=fd_steps, checkpoint_every=fd_steps)
    _, Gs = kinetic_and_grad(Qa)
    gs = seg.adjoint(Gs)
    rng = np.random.default_rng(3)
    ax = (torch.arange(N, dtype=torch.float64, device="cuda") + 0.5) * dx[0]
    z, y, x = torch.meshgrid(ax, ax, ax, indexing="ij")
    rho_p = Qp0[0]
    u_p = Qp0[1:4] / rho_p
    errs = []
    for _ in range(fd_dirs):
        du = torch.zeros_like(Qp0[1:4])
        for q in range(3):
            k = rng.integers(1, 4, size=(3, 3))
            ph = rng.uniform(0, 2 * np.pi, 3)
            a = rng.standard_normal(3)
            du[q, 4:-4, 4:-4, 4:-4] = sum(
                float(a[m]) * torch.sin(int(k[m, 0]) * x + int(k[m, 1]) * y + int(k[m, 2]) * z + float(ph[m]))
                for m in range(3))
        v = torch.zeros_like(Qp0)                       # the state direction of the velocity direction
        v[1:4] = rho_p * du
        v[4] = rho_p * (u_p * du).sum(dim=0)
        ad = float((gs * v).sum())
        e_h = []
        for h in (1e-6, 1e-7):
            Js = []
            for sgn in (1.0, -1.0):
                Qs = Qp0 + sgn * h * v
                flow.RungeKuttaLevelIntegrator(ns, flow.Patch(n, dx, Qs), per).advance(dt, nsteps=fd_steps)
                Js.append(kinetic_and_grad(Qs)[0])
            e_h.append(abs((Js[0] - Js[1]) / (2 * h) - ad) / max(abs(ad), 1e-300))
        errs.append(min(e_h))
    out["fd_check"] = {"directions": fd_dirs, "steps": fd_steps, "h": [1e-6, 1e-7], "seed": 3,
                       "space": "initial velocity (smooth random modes), rho and p fixed",
                       "base": "Taylor-Green vortex + smooth perturbations of amplitude 0.05",
                       "max_rel_err": max(errs), "median_rel_err": float(np.median(errs))}
    rec.close()
    return out


def c4_forward_only(args, flow, N=128):
    """The C4 forward alone: --warmup then --steps SSPRK3 steps of the Navier-Stokes
    Taylor-Green vortex (per-patch fused substeps), device-timed."""
    import torch
    from hamers_gb300 import problems as P
    Qnp, dx = P.taylor_green_3d(N)
    tr = P.taylor_green_transport()
    dt = P.taylor_green_dt(Qnp[:, 4:-4, 4:-4, 4:-4], dx, mu=tr["species_mu"], prandtl=tr["species_Pr"])
    fm = flow.FlowModel("SINGLE_SPECIES", 3, [1.4], transport=tr)
    rec = flow.ConvectiveFluxReconstructor("WCNS5_JS_HLLC_HLL", fm, precision=args.precision,
                                           diffusive_flux_reconstructor="MIDPOINT_FOURTH_ORDER")
    ns = flow.NavierStokes(rec)
    Q = torch.from_numpy(Qnp).cuda()
    integ = flow.RungeKuttaLevelIntegrator(ns, flow.Patch([N] * 3, dx, Q), [1, 1, 1])
    integ.advance(dt, nsteps=args.warmup)
    torch.cuda.synchronize()
    e = [torch.cuda.Event(enable_timing=True) for _ in range(2)]
    stream = torch.cuda.current_stream()
    e[0].record(stream)
    integ.advance(dt, nsteps=args.steps)
    e[1].record(stream)
    torch.cuda.synchronize()
    ms = e[0].elapsed_time(e[1])
    rec.close()
    return {"workload": "3D Navier-Stokes Taylor-Green vortex 128^3 (C4 forward only)", "precision": args.precision,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms / max(args.steps, 1),
            "cell_updates_per_s": N ** 3 * 3 * args.steps / (ms * 1e-3)}


def c1_per_patch(args, flow, N=256, steps=20):
    """2D single species density wave (gamma 1.4, rho = 1 + 0.2 sin(2 pi (x + y)), u = v = 1,
    p = 1, periodic), one 256^2 patch, WCNS5-JS + HLLC-HLL, SSPRK3 at CFL 0.4: the per-patch
    drop-in form (periodic ghost fill + fused substep per stage), device-timed over `steps`
    steps after 3 warm-up steps."""
    import torch
    from hamers_gb300 import problems as P
    Qnp, dx, dt = P.density_wave_2d(N)
    fm = flow.FlowModel("SINGLE_SPECIES", 2, [1.4])
    rec = flow.ConvectiveFluxReconstructor("WCNS5_JS_HLLC_HLL", fm, precision=args.precision)
    drv = PatchDriver(flow, rec, N, dx, torch.from_numpy(Qnp).cuda(), [1, 1])
    for _ in range(3):
        drv.step(dt)
    torch.cuda.synchronize()
    stream = torch.cuda.current_stream()
    e = [torch.cuda.Event(enable_timing=True) for _ in range(2)]
    e[0].record(stream)
    for _ in range(steps):
        drv.step(dt)
    e[1].record(stream)
    torch.cuda.synchronize()
    ms = e[0].elapsed_time(e[1]) / steps
    # the same patch as a one-patch level: one persistent kernel per substep in a CUDA graph
    lv = flow.BatchedLevel(rec, [([N, N], dx)])
    Qb = torch.from_numpy(Qnp).cuda()
    lv.bind(0, Qb)
    lv.set_periodic(0, [1, 1])
    lv.autotune(dt)
    split_b = lv.work_split()
    for _ in range(3):
        lv.step(dt)
    torch.cuda.synchronize()
    e[0].record(stream)
    for _ in range(steps):
        lv.step(dt)
    e[1].record(stream)
    torch.cuda.synchronize()
    lv.check()
    ms_b = e[0].elapsed_time(e[1]) / steps
    lv.close()
    rec.close()
    rate = N * N * 3 / (ms * 1e-3)
    rate_b = N * N * 3 / (ms_b * 1e-3)
    return {"workload": "2D single species density wave 256x256, WCNS5-JS + HLLC-HLL, periodic, SSPRK3 at CFL 0.4",
            "form": "per-patch (ghost fill + fused substep per stage)", "precision": args.precision,
            "cells": N * N, "steps": steps, "ms_per_step": ms, "cell_updates_per_s": rate,
            "roofline": roofline_fracs(rate, ALG_FP64_OPS_C1, alg_bytes(4), args.fp64_peak, args.hbm_peak),
            "batched": {"form": "one-patch level, one persistent kernel per substep in a CUDA graph",
                        "ms_per_step": ms_b, "cell_updates_per_s": rate_b,
                        "work_split": {"chunk_blocks": split_b[0],
                                       "cell_phases": "grid-stride" if split_b[1] & 1 else "chunks",
                                       "faces": "sorted" if split_b[1] & 2 else "in order"},
                        "roofline": roofline_fracs(rate_b, ALG_FP64_OPS_C1, alg_bytes(4), args.fp64_peak,
                                                   args.hbm_peak)},
            "l2": "working set 2.4 MB fits in L2: HBM fraction is an upper bound on DRAM use"}


def cpu_baseline_oracle(Q, n, dx, dt, budget_s=15.0, threads=None):
    """Oracle stage throughput on the host cores on a bounded sample (rows of the patch)."""
    from oracle import oracle as O
    threads = threads or os.cpu_count() or 1
    cfg = O.Config(O.MODEL_FIVE_EQN_ALLAIRE, 2, [1.4, 1.67], O.SCHEME_WCNS6_LD)
    # Sample: a band of rows of the full-width patch, grown until one stage takes ~1 s.
    rows = max(threads, 8)
    G = 4
    best = None
    total_cells = 0
    total_time = 0.0
    t_start = time.time()
    while True:
        rows = min(rows, n)
        sub = Q[:, :, : rows + 2 * G, :].copy()
        t0 = time.perf_counter()
        cells = O.stage_threads(cfg, [n, rows], dx, dt, sub, threads)
        el = time.perf_counter() - t0
        total_cells += cells
        total_time += el
        best = (rows, el)
        if el > 1.0 or rows == n or time.time() - t_start > budget_s:
            break
        rows *= 2
    # repeat the largest sample until the budget is used
    while time.time() - t_start < budget_s:
        rows = best[0]
        sub = Q[:, :, : rows + 2 * G, :].copy()
        t0 = time.perf_counter()
        cells = O.stage_threads(cfg, [n, rows], dx, dt, sub, threads)
        el = time.perf_counter() - t0
        total_cells += cells
        total_time += el
    # one core, as one MPI rank of the reference advances its patch: a band of 128 rows
    rows1 = min(128, n)
    sub = Q[:, :, : rows1 + 2 * G, :].copy()
    t0 = time.perf_counter()
    cells1 = O.stage_threads(cfg, [n, rows1], dx, dt, sub, 1)
    el1 = time.perf_counter() - t0
    return {"value": total_cells / total_time, "unit": UNIT, "cores": threads, "kind": "port",
            "sample": f"{best[0]} x {n} rows of the patch, one RK stage per call, "
                      f"{threads} std::threads (one sub-patch each), {total_time:.1f} s of CPU work",
            "host": f"{platform.machine()}, {os.cpu_count()} hardware threads",
            "one_core": {"value": cells1 / el1, "unit": UNIT,
                         "sample": f"{rows1} x {n} rows, one RK stage, one thread, {el1:.1f} s"}}


def run_reference(args):
    rank, world, _ = dist_env()
    if rank != 0:
        return
    from oracle import oracle as O
    O.build()
    Q, dx, dt = workload(args.n)
    n = args.n
    threads = os.cpu_count() or 1
    cfg = O.Config(O.MODEL_FIVE_EQN_ALLAIRE, 2, [1.4, 1.67], O.SCHEME_WCNS6_LD)
    # The whole patch per substep (about 0.1 s on 16 Grace cores), so that every thread's
    # sub-patch is tall enough for its 4-row ghost halo not to dominate; fewer rows only for
    # runs of more than 200 steps, to keep the arm within a few minutes.
    rows = min(n, max(16 * threads, (n * 200) // max(args.steps, 1)))
    G = 4
    sub = Q[:, :, : rows + 2 * G, :].copy()
    for _ in range(max(0, min(args.warmup, 1))):
        O.stage_threads(cfg, [n, rows], dx, dt, sub, threads)
    t0 = time.perf_counter()
    cells = 0
    for _ in range(args.steps):
        for _s in range(3):
            cells += O.stage_threads(cfg, [n, rows], dx, dt, sub, threads)
    el = time.perf_counter() - t0
    value = cells / el
    line = {"impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": el * 1e3 / args.steps,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
            "data": "synthetic", "config": bench_config(n),
            "cpu_baseline": {"value": value, "unit": UNIT, "cores": threads, "kind": "port",
                             "sample": f"{rows} x {n} rows of the {n}x{n} patch per substep "
                                       f"({n * rows} cells), {threads} std::threads (one sub-patch each)"},
            "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


class PatchDriver:
    """Per-patch form with the BatchedLevel call surface used by the timing loop."""

    def __init__(self, flow, rec, n, dx, Q, periodic):
        import torch
        self.flow = flow
        self.rec = rec
        self.eu = flow.Euler(rec)
        self.periodic = periodic
        self.Q = [Q, torch.empty_like(Q), torch.empty_like(Q)]
        self.views = [flow.Patch([n, n], dx, q) for q in self.Q]
        rec.reserve(self.views[0])

    def substep(self, s, dt):
        self.eu.fillGhosts(self.views[s], self.periodic)
        out = self.Q[0] if s == 2 else self.Q[s + 1]
        self.eu.substep(self.views[s], s, self.Q[:s + 1], dt, out)

    def step(self, dt):
        for s in range(3):
            self.substep(s, dt)

    def check(self):
        pass


def main():
    args = parse()
    if args.impl == "reference":
        run_reference(args)
        return
    import torch
    import torch.distributed as dist

    rank, world, local = dist_env()
    torch.cuda.set_device(local)
    if world > 1:
        dist.init_process_group("nccl")

    from hamers_gb300 import build as B
    B.build()
    from hamers_gb300 import flow
    peaks, peak_kind = measured_peaks()
    args.hbm_peak = float(peaks.get("hbm_gbs", 6800.0))
    args.fp64_peak = None if args.no_peak else fp64_peak_tflops()
    if args.c4_only:
        if rank == 0:
            print(json.dumps({"c4_forward": c4_forward_only(args, flow)}), flush=True)
        return
    if args.uneven_only:
        if rank == 0:
            print(json.dumps({"batched_vs_per_patch": uneven_batched_vs_patch(args, flow)}), flush=True)
        return

    n = args.n
    Qnp, dx, dt = workload(n)
    fm = flow.FlowModel("FIVE_EQN_ALLAIRE", 2, [1.4, 1.67])
    rec = flow.ConvectiveFluxReconstructor("WCNS6_LD_HLLC_HLL", fm, precision=args.precision)
    Q0 = torch.from_numpy(Qnp).cuda()
    Q = Q0.clone()
    stream = torch.cuda.current_stream()
    if args.form == "batched":
        lv = flow.BatchedLevel(rec, [([n, n], dx)])
        lv.bind(0, Q)
        lv.set_periodic(0, [0, 1])
        tuned = lv.autotune(dt)
        split = lv.work_split()
        launches_per_substep = 1
    else:
        lv = PatchDriver(flow, rec, n, dx, Q, [0, 1])
        tuned = (128, None)
        split = None
        launches_per_substep = 6
    Q.copy_(Q0)

    for _ in range(args.warmup):
        lv.step(dt)
    torch.cuda.synchronize()
    lv.check()
    Q.copy_(Q0)
    torch.cuda.synchronize()

    # Device-timed region: CUDA events around every substep (one persistent kernel each).
    ev = [[torch.cuda.Event(enable_timing=True) for _ in range(4)] for _ in range(args.steps)]
    if world > 1:
        dist.barrier()
    torch.cuda.synchronize()
    with ClockSampler(local) as clk:
        t_host0 = time.perf_counter()
        for k in range(args.steps):
            ev[k][0].record(stream)
            for s in range(3):
                lv.substep(s, dt)
                ev[k][s + 1].record(stream)
        torch.cuda.synchronize()
        t_host = time.perf_counter() - t_host0
    lv.check()
    Q_device_loop = Q.clone()
    step_ms = [ev[k][0].elapsed_time(ev[k][3]) for k in range(args.steps)]
    sub_ms = [ev[k][s].elapsed_time(ev[k][s + 1]) for k in range(args.steps) for s in range(3)]
    total_ms = ev[0][0].elapsed_time(ev[-1][3])
    cells_per_step = n * n * 3
    total_ms, value = replica_throughput(total_ms, cells_per_step, args.steps, world, "cuda")

    # End-to-end through the public API: every step copies the host state in (pinned), advances
    # it and copies the result out, and the next step starts from that result, so the timed
    # steps follow the device-timed loop's trajectory from the same initial state.
    host = [Q0.cpu().pin_memory(), torch.empty_like(Q0, device="cpu").pin_memory()]
    for _ in range(2):
        Q.copy_(host[0], non_blocking=True)
        lv.step(dt)
        host[1].copy_(Q, non_blocking=True)
    torch.cuda.synchronize()
    host[0].copy_(Q0.cpu())
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for k in range(args.steps):
        src, dst = host[k % 2], host[(k + 1) % 2]
        Q.copy_(src, non_blocking=True)
        lv.step(dt)
        dst.copy_(Q, non_blocking=True)
    e1.record(stream)
    torch.cuda.synchronize()
    lv.check()
    e2e_ms = e0.elapsed_time(e1)
    e2e_same = bool(torch.equal(host[args.steps % 2], Q_device_loop.cpu()))
    e2e_value = world * cells_per_step * args.steps / (e2e_ms * 1e-3)
    state_bytes = Q.numel() * 8

    hbm = args.hbm_peak
    avg_sub_ms = sum(sub_ms) / len(sub_ms)
    achieved_gbs = ALG_BYTES_PER_CELL * n * n / (avg_sub_ms * 1e-3) / 1e9
    fp64 = args.fp64_peak
    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": total_ms / args.steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": bench_config(n),
        "form": {"form": ("batched persistent kernel, one CUDA graph per substep" if args.form == "batched"
                          else "per-patch kernels (fill, cells, sensor, faces x/y, update) per substep"),
                 "precision": args.precision,
                 "launch_shape": {"threads": tuned[0], "blocks_per_sm": tuned[1]},
                 "work_split": None if split is None else {
                     "chunk_blocks": split[0], "cell_phases": "grid-stride" if split[1] & 1 else "chunks",
                     "faces": "sorted" if split[1] & 2 else "in order"}},
        "e2e": {"value": e2e_value, "unit": UNIT, "h2d_bytes_per_step": state_bytes,
                "d2h_bytes_per_step": state_bytes,
                "note": "every step copies the host state in from pinned memory, advances it and copies the "
                        "result out; the next step starts from that result, so the steps follow the "
                        "device-timed loop's trajectory from the same initial state",
                "same_final_state_as_device_loop": e2e_same},
        "gpu_launches": 3 * launches_per_substep * args.steps,
        "roofline": {"bound": "hbm", "achieved": achieved_gbs, "peak": hbm, "unit": "GB/s",
                     "frac": achieved_gbs / hbm,
                     # ncu dram__bytes_read.sum + dram__bytes_write.sum of one level_kernel launch
                     # of this workload at the autotuned shape
                     "traffic": LEVEL_KERNEL_TRAFFIC_BYTES if (n == 1024 and args.form == "batched") else None,
                     "note": f"peak {peak_kind}; algorithmic {ALG_BYTES_PER_CELL:.1f} B/cell-update; traffic: ncu "
                             "DRAM bytes of one launch (scratch round trips of the persistent kernel's "
                             "phases); the kernel is FP64-pipe bound, see fp64"},
        "fp64": {"achieved": ALG_FP64_OPS_PER_CELL * n * n / (avg_sub_ms * 1e-3) / 1e12,
                 "peak": fp64, "unit": "TFLOP/s", "frac": (ALG_FP64_OPS_PER_CELL * n * n / (avg_sub_ms * 1e-3)
                                                         / 1e12 / fp64) if fp64 else None,
                 "ops_per_cell_update": ALG_FP64_OPS_PER_CELL,
                 "peak_kind": "measured DFMA microbenchmark (hamers_gb300/csrc/hmr_peak.cu)",
                 "note": "divisions and square roots count 1 op each but expand to several FP64 instructions"},
        "substep_ms": {"mean": avg_sub_ms, "min": min(sub_ms), "max": max(sub_ms)},
        "host_wall_ms_per_step": t_host * 1e3 / args.steps,
    }
    with_clocks = None
    if not args.no_adjoint:
        try:
            line["adjoint"] = adjoint_cost(args, flow, Qnp, n, dx, dt)
        except Exception as exc:  # report, never lose the headline line
            line["adjoint"] = {"error": str(exc)[:300]}
    if not args.no_c4:
        try:
            line["c4"] = c4_navier_stokes(args, flow, fd_dirs=16 if args.c4 else 4)
        except Exception as exc:  # report, never lose the headline line
            line["c4"] = {"error": str(exc)[:300]}
    if not args.no_c1:
        try:
            line["c1"] = c1_per_patch(args, flow)
        except Exception as exc:  # report, never lose the headline line
            line["c1"] = {"error": str(exc)[:300]}
    if not args.no_c5:
        try:
            line["c5"] = c5_level_and_adjoint(args, flow)
        except Exception as exc:  # report, never lose the headline line
            line["c5"] = {"error": str(exc)[:300]}
    if not args.no_uneven:
        try:
            line["batched_vs_per_patch"] = uneven_batched_vs_patch(args, flow)
        except Exception as exc:  # report, never lose the headline line
            line["batched_vs_per_patch"] = {"error": str(exc)[:300]}
    if rank == 0:
        line["clocks"] = clk.summary()
        if not args.no_cpu_baseline:
            try:
                from oracle import oracle as O
                O.build()
                line["cpu_baseline"] = cpu_baseline_oracle(Qnp, n, dx, dt)
            except Exception as exc:  # report, never fail the GPU line
                line["cpu_baseline"] = {"value": None, "error": str(exc)[:200]}
        print(json.dumps(line), flush=True)
    if world > 1:
        dist.barrier()
        dist.destroy_process_group()
    del with_clocks


if __name__ == "__main__":
    main()
