#!/usr/bin/env python
"""Throughput of the QG-YBJ+ time step on GB300, in cell-steps/s.

Workload: 512 x 512 x 256 (n1 x n2 x n3), mixed precision (FP32 transforms,
products and leapfrog update; FP64 tridiagonal inversions), exponential
stratification, seeded random-phase eddies peaked at k=8 plus a surface wave
(synthetic inputs; the reference ships no initial-condition files).

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

N>1 runs one independent replica per GPU (the step shards only by running
independent ensemble members), with a barrier and the maximum time over
ranks.  The reference arm times the FP64 CPU restatement of the reference's
step (the Fortran reference cannot be built here) on the host cores.
"""
from __future__ import annotations

import argparse
import dataclasses
import json
import math
import os
import statistics
import subprocess
import sys
import threading
import time
from pathlib import Path

ROOT = Path(__file__).resolve().parent
PKG = ROOT / "qg-ybjp-model_gb300"
for _p in (str(ROOT), str(PKG)):
    if _p not in sys.path:
        sys.path.insert(0, _p)

FALLBACK_HBM_GBS = 6800.0
# DRAM bytes per level of a launch (dram__bytes_read.sum + dram__bytes_write.sum,
# L2 not flushed) of each phase-A kernel, from the ncu capture summarised in
# profiles/dram_per_launch_512x512x64_mixed.md (512^2 levels, one batch of 64
# levels whose scratch planes outgrow L2 as the 256-level batch's do).  The
# roofline entry scales it by the levels per launch of the run.
MEASURED_TRAFFIC_PER_LEVEL = {
    ("col_inv", 512, "mixed"): 3.553e6,
    ("row_main", 512, "mixed"): 8.495e6,
    ("col_update", 512, "mixed"): 14.114e6,
    ("row_qw", 512, "mixed"): 4.406e6,
    ("col_qw", 512, "mixed"): 2.605e6,
}


# ---------------------------------------------------------------------------
# distributed helpers (replicas: no collective on the data path)
# ---------------------------------------------------------------------------
def dist_env():
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return world, rank, local


def dist_setup(world: int, backend: str):
    if world <= 1:
        return None
    import torch.distributed as dist
    os.environ.setdefault("MASTER_ADDR", "127.0.0.1")
    dist.init_process_group(backend=backend)
    return dist


def barrier(dist):
    if dist is not None:
        dist.barrier()


def reduce_max(dist, x: float, device=None) -> float:
    if dist is None:
        return x
    import torch
    t = torch.tensor([x], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def whole_job_value(world: int, cells: int, steps: int, max_seconds: float) -> float:
    """Cell-steps/s of all replicas together (weak scaling)."""
    return world * cells * steps / max_seconds


# ---------------------------------------------------------------------------
# clocks during the timed region
# ---------------------------------------------------------------------------
class ClockSampler:
    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
         "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
         "clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index: int):
        self.gpu = gpu_index
        self.lines: list[str] = []
        self.proc = None
        self.thread = None

    def start(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", f"--query-gpu={self.Q}", "--format=csv,noheader,nounits",
                                          "-lms", "100", "-i", str(self.gpu)],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except OSError:
            self.proc = None
            return
        self.thread = threading.Thread(target=self._read, daemon=True)
        self.thread.start()

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self) -> dict:
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"], "samples": 0}
        time.sleep(0.15)
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        self.thread.join(timeout=5)
        sm, mx, reasons = [], [], set()
        names = ("hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap")
        for ln in self.lines:
            parts = [p.strip() for p in ln.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                mx.append(float(parts[2]))
            except ValueError:
                continue
            for nm, v in zip(names, parts[5:9]):
                if v.lower() == "active":
                    reasons.add(nm)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": sorted(reasons), "samples": len(sm)}


def measured_peak_hbm() -> tuple[float, str]:
    p = ROOT / "MEASURED_PEAKS.json"
    try:
        return float(json.loads(p.read_text())["hbm_gbs"]), "measured"
    except Exception:
        return FALLBACK_HBM_GBS, "fallback"


# ---------------------------------------------------------------------------
# algorithmic bytes
# ---------------------------------------------------------------------------
def algorithmic_bytes(n: int, n3: int, zb: int, precision: str) -> dict:
    """Algorithmic bytes per launch of each kernel class: the retained-mode
    field passes the kernel performs, one field = one level of the retained
    modes (the 2/3 disk, L=1) x s bytes, s = 8 (FP32 complex, mixed) or 16
    (FP64).  The step as a whole moves 22 field passes (reads of q, q_old, BR,
    BI, BR_old, BI_old, psi, AR, AI and writes of the seven phase-A results;
    reads of q*, BR, BI and writes of psi, AR, AI in the solves); q is read
    again by k_col_inv and k_col_qw, so the kernels' passes add up to 24 on
    the mixed path, whose k_col_inv reads psi and q only (B's y-transforms are
    kept from the previous step's update), and to 26 in FP64 (k_col_inv also
    reads BR and BI).
    Kernels that touch only the (kx,y) scratch planes perform no field pass:
    those planes are intermediate traffic (see traffic_model)."""
    from qgybj.config import dealias_mask
    s = 8 if precision == "mixed" else 16
    fld = int(dealias_mask(n).sum()) * s      # one state field, one level
    return {
        "col_inv": zb * (2 if precision == "mixed" else 4) * fld,   # psi, q (and BR, BI in FP64)
        "row_main": 0,
        "col_update": zb * 14 * fld,          # 8 read (q, qo, BR, BI, BRo, BIo, AR, AI), 6 written
        "row_qw": 0,
        "col_qw": zb * 2 * fld,               # q read, q* written
        "solve": n3 * 6 * fld,                # q*, BR, BI read; psi, AR, AI written (one launch)
        "solve_A": n3 * 4 * fld,              # BR, BI read; AR, AI written (the A solves on their own)
        "dissipation": n3 * 2 * fld,
        "step": 22 * fld * n3,
        "step_dense": 22 * (n // 2 + 1) * n * n3 * s,
    }


def traffic_model(n: int, zb: int, precision: str) -> dict:
    """Bytes per launch each phase-A kernel moves when the (kx,y) scratch
    planes round-trip through DRAM (one plane = n x (K+1) complex values of
    one level): the state fields it reads and writes plus its plane reads and
    writes.  Measured DRAM traffic per launch is compared with this."""
    from qgybj.config import dealias_mask, kmax
    s = 8 if precision == "mixed" else 16
    fld = int(dealias_mask(n).sum()) * s
    pln = n * (kmax(n) + 1) * s
    return {
        # mixed: psi, q -> u, v, zeta, q planes (B's planes kept); FP64: all six
        "col_inv": zb * ((2 * fld + 4 * pln) if precision == "mixed" else (4 * fld + 6 * pln)),
        "row_main": zb * (6 * pln + 6 * pln),
        "col_update": zb * (6 * pln + 14 * fld + 4 * pln),
        "row_qw": zb * (4 * pln + 2 * pln),
        "col_qw": zb * (2 * pln + 2 * fld),
    }


def transform_flops(n: int, n3: int, precision: str = "mixed") -> dict:
    """Floating-point operations of the transforms of one step as the kernels
    execute them: radix-8/4/2 Stockham passes (a radix-8 butterfly is 56 real
    additions/multiplications, a twiddle 6), column transforms per retained
    kx and level (16 on the mixed path, whose update keeps B's y-transforms
    for the next step: k_col_inv 4, k_col_update 6 + 4, k_col_qw 2; 18 in
    FP64, whose k_col_inv transforms B as well) and 11 complex row transforms
    (two real rows each) per y and level, plus the FP64 column solves (6
    recurrences of 3 operations per level and column, an FMA counted as 2)."""
    from qgybj.config import dealias_mask, kmax
    rad, rem = [], n
    while rem > 1:
        r = 8 if rem >= 8 else (4 if rem >= 4 else 2)
        rad.append(r)
        rem //= r
    bfly = {8: 56, 4: 16, 2: 4}
    per_fft, ns = 0, 1
    for r in rad:
        per_fft += (n // r) * (bfly[r] + (6 * (r - 1) if ns > 1 else 0))
        ns *= r
    K = kmax(n)
    ncol = 16 if precision == "mixed" else 18
    fft = (ncol * (K + 1) + 11 * n) * per_fft * n3
    solve = 6 * n3 * int(dealias_mask(n).sum()) * 5
    return {"transforms": fft, "solve_fp64": solve, "per_complex_fft": per_fft}


# ---------------------------------------------------------------------------
# parity helpers
# ---------------------------------------------------------------------------
CHECK_STEPS = 3          # steps after which the oracle checks the full-size state (Euler + 2 leapfrog)
PARITY_FIELDS = ("psi", "q", "LAr", "LAi", "BR", "BI")


def rel_l2(a, b) -> float:
    import numpy as np
    nb = float(np.linalg.norm(b))
    return float(np.linalg.norm(a - b)) / nb if nb else float(np.linalg.norm(a))


def state_fields(sim, Bu: float) -> dict:
    """psi, q, B and the wave field LA = B + kh^2 A/(4 Bu) (the field the
    reference writes, diagnostics.f90:1698-1706) in the reference layout."""
    from qgybj.config import la_from_b
    g = {f: sim.get_state(f) for f in ("psi", "q", "BR", "BI", "AR", "AI")}
    return {"psi": g["psi"], "q": g["q"], "BR": g["BR"], "BI": g["BI"],
            "LAr": la_from_b(sim.n, Bu, g["BR"], g["AR"]), "LAi": la_from_b(sim.n, Bu, g["BI"], g["AI"])}


def measured_fp64_peak(dev) -> float:
    """FP64 TFLOP/s of cuBLAS DGEMM (8192^3, best of 3) on this GPU."""
    import torch
    a = torch.randn(8192, 8192, dtype=torch.float64, device=dev)
    b = torch.randn(8192, 8192, dtype=torch.float64, device=dev)
    torch.matmul(a, b)
    torch.cuda.synchronize()
    best = 1e30
    for _ in range(3):
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        torch.matmul(a, b)
        e1.record()
        torch.cuda.synchronize()
        best = min(best, e0.elapsed_time(e1))
    del a, b
    torch.cuda.empty_cache()
    return 2.0 * 8192 ** 3 / (best / 1e3) / 1e12


# ---------------------------------------------------------------------------
def run_ours(args, world, rank, local):
    import numpy as np
    import torch

    import qgybj
    from qgybj.config import CONFIGS, make_initial_condition, model_parameters

    dist = dist_setup(world, "nccl")
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    rc = workload(args)
    precision = args.precision or rc.precision
    ic = make_initial_condition(rc)
    params = model_parameters(rc, ic.delt)
    sim = qgybj.Simulation(params, precision, device=local, levels_per_batch=rc.levels_per_batch,
                           solve_columns=rc.solve_columns)

    def init(s):
        s.set_state("psi", ic.psi)
        s.set_state("BR", ic.BR)
        s.set_state("BI", ic.BI)
        s.init_state(True, True)

    init(sim)
    n, n3 = rc.n, rc.n3
    cells = n * n * n3
    # warm-up (the first step is the forward Euler start)
    sim.steps_async(args.warmup, True)
    sim.synchronize()
    # per-kernel device times of one step (events around each launch)
    prof = sim.profile_step(False)
    launches_per_step = sum(c for _, c in prof.values())
    # timed region
    stream = torch.cuda.ExternalStream(sim.stream(), device=dev)
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    clocks = ClockSampler(local)
    barrier(dist)
    torch.cuda.synchronize()
    sim.synchronize()
    clocks.start()
    time.sleep(0.25)
    e0.record(stream)
    sim.steps_async(args.steps, False)
    e1.record(stream)
    sim.synchronize()
    torch.cuda.synchronize()
    clk = clocks.stop()
    barrier(dist)
    ms = e0.elapsed_time(e1)
    ms_max = reduce_max(dist, ms, device=dev)
    value = whole_job_value(world, cells, args.steps, ms_max / 1e3)
    st = sim.diagnostics_fp64()
    finite = all(math.isfinite(v) for v in st.values())

    # end to end through the C-ABI with host buffers: upload the state from
    # pinned host memory, K synchronous qg_step calls each followed by the
    # FP64 diagnostics read back, download psi, BR, BI.
    e2e = None
    if not args.no_e2e:
        shape = (n3, n, n // 2 + 1)
        names_in = ("q", "qo", "BR", "BI", "BRo", "BIo", "psi", "AR", "AI")
        host_in = {}
        for f in names_in:
            t = torch.empty(shape, dtype=torch.complex128, pin_memory=True)
            sim.get_state(f, out=t.numpy())
            host_in[f] = t
        host_out = {f: torch.empty(shape, dtype=torch.complex128, pin_memory=True) for f in ("psi", "BR", "BI")}
        k_e2e = args.e2e_steps or args.steps
        # one untimed pass of the same sequence (first use of the pinned buffers)
        for f in names_in:
            sim.set_state(f, host_in[f])
        for _ in range(3):
            sim.step(False)
            sim.diagnostics_fp64_async()
            sim.diagnostics_fp64_wait()
        for f, t in host_out.items():
            sim.get_state(f, out=t.numpy())
        for f in names_in:
            sim.get_state(f, out=host_in[f].numpy())
        barrier(dist)
        t0 = time.perf_counter()
        for f in names_in:
            sim.set_state(f, host_in[f])
        ta = time.perf_counter()
        t_diag = 0.0
        metrics = []
        # every step's FP64 integrals are read back: queued right after the
        # step, collected after the next step has been queued (they run beside
        # its first kernels)
        for i in range(k_e2e):
            sim.step(False)
            tb = time.perf_counter()
            if i > 0:
                metrics.append(sim.diagnostics_fp64_wait())
            sim.diagnostics_fp64_async()
            t_diag += time.perf_counter() - tb
        tb = time.perf_counter()
        metrics.append(sim.diagnostics_fp64_wait())
        t_diag += time.perf_counter() - tb
        tc = time.perf_counter()
        for f, t in host_out.items():
            sim.get_state(f, out=t.numpy())
        t1 = time.perf_counter()
        e2e_s = reduce_max(dist, t1 - t0, device=torch.device("cuda", local))
        fbytes = int(np.prod(shape)) * 16
        e2e = {"value": whole_job_value(world, cells, k_e2e, e2e_s), "unit": "cell-steps/s",
               "h2d_bytes_per_step": len(names_in) * fbytes / k_e2e,
               "d2h_bytes_per_step": (3 * fbytes + 7 * 8 * k_e2e) / k_e2e,
               "steps": k_e2e, "seconds": e2e_s,
               "path": "qg_set_state x9 (pinned host) + K x (qg_step + qg_diagnostics_fp64_async, collected with "
                       "qg_diagnostics_fp64_wait after the next qg_step) + qg_get_state x3",
               "metrics_read": len(metrics), "finite": all(math.isfinite(v) for m in metrics for v in m.values()),
               "ms": {"set_state_x9": (ta - t0) * 1e3, "steps": (tc - ta - t_diag) * 1e3,
                      "diagnostics_wait": t_diag * 1e3, "get_state_x3": (t1 - tc) * 1e3}}

    # FP64 GPU step on the same workload (the metric compares the two), and
    # parity: the mixed path against the FP64 path after the configuration's
    # step count, per field; snapshots after CHECK_STEPS for the oracle check
    fp64 = parity = None
    snapshots = {}
    if not args.no_fp64 and precision == "mixed":
        psteps = max(rc.steps, CHECK_STEPS + 1)
        sim64 = qgybj.Simulation(params, "fp64", device=local, levels_per_batch=CONFIGS["c1"].levels_per_batch,
                                 solve_columns=rc.solve_columns)
        init(sim64)
        s64 = torch.cuda.ExternalStream(sim64.stream(), device=dev)
        k64 = max(2, min(args.fp64_steps, psteps - CHECK_STEPS - 1))
        sim64.steps_async(CHECK_STEPS, True)
        sim64.synchronize()
        snapshots["fp64"] = state_fields(sim64, params["Bu"])
        sim64.steps_async(1, False)          # warm: the leapfrog graph exists
        sim64.synchronize()
        a0, a1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a0.record(s64)
        sim64.steps_async(k64, False)
        a1.record(s64)
        sim64.synchronize()
        ms64 = a0.elapsed_time(a1)
        sim64.steps_async(psteps - CHECK_STEPS - 1 - k64, False)
        sim64.synchronize()
        ref = state_fields(sim64, params["Bu"])
        sim64.close()
        fl = transform_flops(n, n3, "fp64")
        peak64 = measured_fp64_peak(dev)
        fp64 = {"value": cells * k64 / (ms64 / 1e3), "ms_per_step": ms64 / k64, "steps": k64,
                "flops_per_step": fl["transforms"] + fl["solve_fp64"],
                "achieved_tflops": (fl["transforms"] + fl["solve_fp64"]) / (ms64 / k64 / 1e3) / 1e12,
                "peak_tflops": peak64, "peak_kind": "cuBLAS DGEMM 8192^3, best of 3, measured in this run",
                "frac": (fl["transforms"] + fl["solve_fp64"]) / (ms64 / k64 / 1e3) / 1e12 / peak64}
        init(sim)
        sim.steps_async(CHECK_STEPS, True)
        sim.synchronize()
        snapshots["mixed"] = state_fields(sim, params["Bu"])
        sim.steps_async(psteps - CHECK_STEPS, False)
        sim.synchronize()
        got = state_fields(sim, params["Bu"])
        parity = {"mixed_vs_fp64_gpu": {"steps": psteps, "tolerance": 1e-5,
                                        "relL2": {f: rel_l2(got[f], ref[f]) for f in PARITY_FIELDS}}}

    out = None
    if rank == 0:
        peak, peak_kind = measured_peak_hbm()
        zb = sim_batch(sim)
        ab = algorithmic_bytes(n, n3, zb, precision)
        if prof.get("solve_A", (0, 0))[1]:       # the psi solve alone: q* read, psi written
            ab["solve"] = ab["solve"] // 3
        tm = traffic_model(n, zb, precision)
        dom = max((k for k in prof if prof[k][1] > 0), key=lambda k: prof[k][0])
        dom_ms = prof[dom][0] / prof[dom][1]
        achieved = ab[dom] / (dom_ms / 1e3) / 1e9
        step_ms = ms / args.steps
        fl = transform_flops(n, n3, precision)
        meas = MEASURED_TRAFFIC_PER_LEVEL.get((dom, n, precision))
        out = {
            "metric": "cell-steps/s", "value": value, "unit": "cell-steps/s", "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms_max / args.steps,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "f32" if precision == "mixed" else "f64", "data": "synthetic (seeded)",
            "config": {"workload": rc.name, "n1": n, "n2": n, "n3": n3, "precision": precision,
                       "solves_dtype": "f64", "stratification": rc.stratification, "k0": rc.k0, "seed": rc.seed,
                       "parallelism": f"replicas{world}",
                       "l2": "inputs larger than L2: resident state ~%.1f GB per step" % (ab["step"] / 1e9)},
            "roofline": {"bound": "hbm", "kernel": dom, "achieved": achieved, "peak": peak,
                         "peak_kind": peak_kind, "unit": "GB/s", "frac": achieved / peak,
                         "algorithmic_bytes_per_launch": ab[dom], "ms_per_launch": dom_ms,
                         "traffic": meas * zb if meas else None,
                         "traffic_model": tm.get(dom)},
            "step_roofline": {"bytes_per_step": ab["step"], "achieved": ab["step"] / (step_ms / 1e3) / 1e9,
                              "frac": ab["step"] / (step_ms / 1e3) / 1e9 / peak, "unit": "GB/s",
                              "bytes_per_step_dense_layout": ab["step_dense"],
                              "frac_dense_layout": ab["step_dense"] / (step_ms / 1e3) / 1e9 / peak,
                              "fp32_transform_tflops": fl["transforms"] / (step_ms / 1e3) / 1e12},
            "kernels_ms_per_step": {k: v[0] for k, v in prof.items() if v[1]},
            "launches_per_step": {k: v[1] for k, v in prof.items() if v[1]},
            "gpu_launches": launches_per_step * args.steps,
            "clocks": clk, "e2e": e2e, "fp64_gpu": fp64,
            "mixed_over_fp64": (value / world / fp64["value"]) if fp64 else None,
            "parity": parity,
            "state_finite": finite,
        }
    sim.close()
    return out, snapshots


def workload(args):
    """The run configuration timed: a named configuration, optionally at
    another resolution (--n/--n3, used for small profiling cases)."""
    from qgybj.config import CONFIGS, scaled
    rc = CONFIGS[args.config]
    if args.n or args.n3:
        rc = scaled(rc, args.n or rc.n, args.n3 or rc.n3)
    if getattr(args, "levels_per_batch", 0):
        rc = dataclasses.replace(rc, levels_per_batch=args.levels_per_batch)
    if getattr(args, "solve_columns", 0):
        rc = dataclasses.replace(rc, solve_columns=args.solve_columns)
    return rc


def run_ensemble(args, world, rank, local):
    """The 64-member uneven ensemble (24 at 64^2x32, 24 at 128^2x64, 16 at
    256^2x128, mixed precision) advanced by one graph launch per step, against
    the same members run one after another, each with its own graph."""
    import torch

    import qgybj
    from qgybj.config import ensemble_members, make_initial_condition, model_parameters

    dist = dist_setup(world, "nccl")
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    members = ensemble_members()[: args.members or None]
    ics = [make_initial_condition(rc) for rc in members]
    params = [model_parameters(rc, ic.delt) for rc, ic in zip(members, ics)]
    tuned = {}
    for rc, p in zip(members, params):
        if (rc.n, rc.n3) not in tuned:
            tuned[(rc.n, rc.n3)] = qgybj.autotune(p, "mixed", local, nsteps=3)
    lpb = [tuned[(rc.n, rc.n3)]["levels_per_batch"] for rc in members]
    stc = [tuned[(rc.n, rc.n3)]["solve_columns"] for rc in members]
    cells = sum(rc.n * rc.n * rc.n3 for rc in members)

    def init(sim, ic):
        sim.set_state("psi", ic.psi); sim.set_state("BR", ic.BR); sim.set_state("BI", ic.BI)
        sim.init_state(True, True)

    ens = qgybj.Ensemble(params, "mixed", local, levels_per_batch=lpb, solve_columns=stc)
    for sim, ic in zip(ens.members, ics):
        init(sim, ic)
    # concurrent member chains of the step graph: timed choice among a few
    stream0 = torch.cuda.ExternalStream(ens.stream(), device=dev)
    lane_ms = {}
    for lanes in (1, 2, 3, 4):
        ens.set_lanes(lanes)
        ens.step(2, True)
        ens.synchronize()
        a0, a1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a0.record(stream0)
        ens.step(5, False)
        a1.record(stream0)
        ens.synchronize()
        lane_ms[lanes] = a0.elapsed_time(a1) / 5
    best_lanes = min(lane_ms, key=lane_ms.get)
    ens.set_lanes(best_lanes)
    for sim, ic in zip(ens.members, ics):
        init(sim, ic)
    ens.step(args.warmup, True)
    ens.synchronize()
    stream = torch.cuda.ExternalStream(ens.stream(), device=dev)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    clocks = ClockSampler(local)
    barrier(dist)
    torch.cuda.synchronize()
    clocks.start()
    time.sleep(0.25)
    e0.record(stream)
    ens.step(args.steps, False)
    e1.record(stream)
    ens.synchronize()
    torch.cuda.synchronize()
    clk = clocks.stop()
    barrier(dist)
    ms = reduce_max(dist, e0.elapsed_time(e1), device=dev)
    prof = ens.profile_step(False)
    launches = sum(c for _, c in prof.values())
    ens.close()
    # the same members one after another
    seq_ms = 0.0
    for p, ic, l, tc in zip(params, ics, lpb, stc):
        sim = qgybj.Simulation(p, "mixed", local, levels_per_batch=l, solve_columns=tc)
        init(sim, ic)
        sim.steps_async(args.warmup, True)
        sim.synchronize()
        st = torch.cuda.ExternalStream(sim.stream(), device=dev)
        a0, a1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a0.record(st)
        sim.steps_async(args.steps, False)
        a1.record(st)
        sim.synchronize()
        seq_ms += a0.elapsed_time(a1)
        sim.close()
    if rank != 0:
        return None
    value = whole_job_value(world, cells, args.steps, ms / 1e3)
    return {
        "metric": "cell-steps/s", "value": value, "unit": "cell-steps/s", "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms / args.steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded)",
        "config": {"workload": f"c3_ensemble_{len(members)}_members", "members": len(members),
                   "sizes": {f"{n}x{n}x{n3}": sum(1 for rc in members if (rc.n, rc.n3) == (n, n3))
                             for (n, n3) in tuned},
                   "levels_per_batch": {f"{n}x{n}x{n3}": t["levels_per_batch"] for (n, n3), t in tuned.items()},
                   "solve_columns": {f"{n}x{n}x{n3}": t["solve_columns"] for (n, n3), t in tuned.items()},
                   "precision": "mixed", "parallelism": f"replicas{world}"},
        "lanes": best_lanes, "lanes_ms_per_step": lane_ms,
        "kernels_ms_per_step": {k: v[0] for k, v in prof.items() if v[1]},
        "launches_per_step": {k: v[1] for k, v in prof.items() if v[1]},
        "sequential_value": cells * args.steps / (seq_ms / 1e3),
        "ensemble_over_sequential": seq_ms / (ms / world),
        "gpu_launches": launches * args.steps, "clocks": clk, "e2e": None,
    }


def run_adjoint(args, world, rank, local):
    """Adjoint-to-forward cost at 128^2x64 FP64 (constant N^2): J after
    --steps steps and its gradient with respect to (q0, B0) with checkpoints
    every --ckpt steps, against the forward steps alone on the same handle."""
    import torch

    import qgybj
    from qgybj.config import make_initial_condition, model_parameters

    if rank != 0:
        return None
    rc = workload(args)
    ic = make_initial_condition(rc)
    params = model_parameters(rc, ic.delt)
    sim = qgybj.Simulation(params, "fp64", local)
    sim.set_state("psi", ic.psi); sim.set_state("BR", ic.BR); sim.set_state("BI", ic.BI)
    sim.init_state(True, True)
    q0, BR0, BI0 = sim.get_state("q"), sim.get_state("BR"), sim.get_state("BI")
    nsteps, every = args.steps, args.ckpt
    dev = torch.device("cuda", local)
    st = torch.cuda.ExternalStream(sim.stream(), device=dev)
    sim.steps_async(args.warmup, True)
    sim.synchronize()

    def forward_ms():
        a0, a1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a0.record(st)
        sim.steps_async(1, True)
        sim.steps_async(nsteps - 1, False)
        a1.record(st)
        sim.synchronize()
        return a0.elapsed_time(a1)

    def wall_ms(ckpt, grad=True):
        t0 = time.perf_counter()
        out = sim.adjoint_run(q0, BR0, BI0, nsteps, ckpt, gradient=grad)
        return (time.perf_counter() - t0) * 1e3, out

    wall_ms(every)                                          # warm-up: buffers, graphs
    wall_ms(1)
    fwd = min(forward_ms() for _ in range(3))
    clocks = ClockSampler(local)
    clocks.start()
    time.sleep(0.25)
    reps = [wall_ms(every) for _ in range(3)]
    J = reps[0][1][0]
    adj = min(r[0] for r in reps)
    # every state checkpointed: no recomputation, so the difference to the
    # forward-only call is the transposed steps themselves
    all_ck = min(wall_ms(1)[0] for _ in range(2))
    fwd_ck = min(wall_ms(1, grad=False)[0] for _ in range(2))
    clk = clocks.stop()
    sim.close()
    step_T = (all_ck - fwd_ck) / nsteps
    return {
        "metric": "adjoint/forward time", "value": adj / fwd, "unit": "ratio", "n_gpus": 1,
        "steps": nsteps, "warmup": args.warmup, "ms_per_step": adj / nsteps, "higher_is_better": False,
        "scaling": "none", "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded)",
        "config": {"workload": f"{rc.name}_adjoint", "checkpoint_every": every, "objective": "LA subvolume"},
        "forward_ms": fwd, "gradient_ms": adj, "gradient_ms_reps": [r[0] for r in reps],
        "adjoint_step_ms": step_T, "forward_step_ms": fwd / nsteps,
        "adjoint_step_over_forward_step": step_T / (fwd / nsteps),
        "gradient_all_checkpoints_ms": all_ck, "forward_all_checkpoints_ms": fwd_ck,
        "J": J, "clocks": clk,
    }


def sim_batch(sim) -> int:
    """Levels per phase-A batch as chosen by the library (same rule)."""
    from qgybj.config import kmax
    n, n3 = sim.n, sim.n3
    kxp = ((kmax(n) + 1 + 7) // 8) * 8
    per = 6 * n * kxp * (8 if sim.precision == "mixed" else 16)
    zb = sim.cfg.levels_per_batch or max(1, (1280 << 20) // per)
    zb = min(zb, n3)
    nb = (n3 + zb - 1) // zb
    return (n3 + nb - 1) // nb


# ---------------------------------------------------------------------------
def cpu_oracle_rate(rc, nz: int, steps: int, warm: int, workers: int):
    """Oracle (FP64 numpy/scipy restatement) on a slab of nz levels at the
    workload's horizontal resolution: cell-steps/s and seconds."""
    from oracle import qgybj_oracle as orc
    from qgybj.config import make_initial_condition, model_parameters, scaled
    orc.set_workers(workers)
    sub = scaled(rc, rc.n, nz)
    ic = make_initial_condition(sub)
    params = model_parameters(sub, ic.delt)
    keys = ("n1", "n2", "n3", "dz", "Bu", "Ro", "W2F", "delt", "gamma", "nuh1", "nuh2", "ilap1", "ilap2",
            "nuh1w", "nuh2w", "ilap1w", "ilap2w", "nuz", "a_ell_ut", "r_2ut")
    model = orc.Model(orc.Params(**{k: params[k] for k in keys}))
    st = orc.initial_state(model, ic.psi, ic.BR, ic.BI)
    st = model.step(st, True)
    for _ in range(warm):
        st = model.step(st, False)
    t0 = time.perf_counter()
    for _ in range(steps):
        st = model.step(st, False)
    dt = time.perf_counter() - t0
    return rc.n * rc.n * nz * steps / dt, dt


def cpu_baseline_leg(rc, snapshots: dict):
    """The oracle on the host cores over the full workload: CHECK_STEPS steps
    from the seeded initial condition (Euler start, then leapfrog steps), the
    leapfrog steps timed as the CPU baseline; the states it reaches are the
    checker of the GPU snapshots taken after the same steps (per-field
    relative L2 of the mixed and FP64 paths)."""
    from oracle import qgybj_oracle as orc
    from qgybj.config import make_initial_condition, model_parameters
    workers = os.cpu_count() or 1
    orc.set_workers(workers)
    ic = make_initial_condition(rc)
    params = model_parameters(rc, ic.delt)
    keys = ("n1", "n2", "n3", "dz", "Bu", "Ro", "W2F", "delt", "gamma", "nuh1", "nuh2", "ilap1", "ilap2",
            "nuh1w", "nuh2w", "ilap1w", "ilap2w", "nuz", "a_ell_ut", "r_2ut")
    model = orc.Model(orc.Params(**{k: params[k] for k in keys}))
    st = orc.initial_state(model, ic.psi, ic.BR, ic.BI)
    st = model.step(st, True)
    t0 = time.perf_counter()
    for _ in range(CHECK_STEPS - 1):
        st = model.step(st, False)
    secs = time.perf_counter() - t0
    value = rc.n * rc.n * rc.n3 * (CHECK_STEPS - 1) / secs
    base = {"value": value, "unit": "cell-steps/s", "cores": workers, "kind": "port",
            "sample": f"oracle (FP64 numpy/scipy restatement of the reference step) on the full {rc.n}x{rc.n}x{rc.n3} "
                      f"{rc.name} workload, {CHECK_STEPS - 1} leapfrog steps after the Euler start ({secs:.1f} s)"}
    vs = None
    if snapshots:
        ref = {"psi": st.psi, "q": st.q, "BR": st.BR, "BI": st.BI,
               "LAr": model.la_from_b(st.BR, st.AR), "LAi": model.la_from_b(st.BI, st.AI)}
        vs = {"steps": CHECK_STEPS, "tolerance": {"mixed": 1e-5, "fp64": 1e-12}}
        for prec, got in snapshots.items():
            vs[prec] = {f: rel_l2(got[f], ref[f]) for f in PARITY_FIELDS}
    return base, vs


def ensemble_cost(args, local) -> dict:
    """The C3 ensemble (64 uneven members in one graph launch per step)
    against the same members run one after another, as --config c3
    measures it, with 10 timed steps."""
    a = argparse.Namespace(**vars(args))
    a.config, a.steps, a.warmup, a.members = "c3", 10, 3, 0
    r = run_ensemble(a, 1, 0, local)
    return {"value": r["value"], "unit": r["unit"], "ms_per_step": r["ms_per_step"],
            "sequential_value": r["sequential_value"], "ensemble_over_sequential": r["ensemble_over_sequential"],
            "workload": r["config"]["workload"], "sizes": r["config"]["sizes"], "steps": r["steps"],
            "launches_per_step": sum(r["launches_per_step"].values()), "clocks": r["clocks"]}


def adjoint_cost(args, local) -> dict:
    """The adjoint-to-forward cost on the C4 workload (128^2 x 64 FP64, J
    after 50 steps, checkpoints every 10), as --config c4 measures it."""
    a = argparse.Namespace(**vars(args))
    a.config, a.steps, a.warmup, a.ckpt, a.n, a.n3, a.levels_per_batch = "c4", 50, 3, 10, 0, 0, 0
    r = run_adjoint(a, 1, 0, local)
    return {k: r[k] for k in ("forward_ms", "gradient_ms", "forward_step_ms", "adjoint_step_ms",
                              "adjoint_step_over_forward_step")} | {
        "gradient_over_forward": r["value"], "workload": r["config"]["workload"], "steps": r["steps"],
        "checkpoint_every": r["config"]["checkpoint_every"], "clocks": r["clocks"]}


def run_reference(args, world, rank, local):
    if rank != 0:
        return None
    rc = workload(args)
    workers = os.cpu_count() or 1
    # calibrate the slab depth so that the whole run stays within ~2 minutes
    # (on 32 levels: slabs of 2-8 levels run from the host caches and
    # overstate the rate of a deep, memory-bound one ~2.5x)
    rate, _ = cpu_oracle_rate(rc, min(32, rc.n3), 1, 0, workers)
    budget = float(args.reference_budget_s)
    per_step = budget / max(1, args.steps + args.warmup)
    nz = int(max(2, min(rc.n3, per_step * rate / (rc.n * rc.n))))
    value, secs = cpu_oracle_rate(rc, nz, args.steps, args.warmup, workers)
    sample = (f"oracle (FP64 numpy/scipy restatement of the reference step) on a {rc.n}x{rc.n}x{nz} slab of "
              f"the {rc.name} workload, {args.steps} leapfrog steps after {args.warmup} warm-up")
    return {
        "metric": "cell-steps/s", "value": value, "unit": "cell-steps/s", "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": secs / args.steps * 1e3, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded)",
        "config": {"workload": f"{rc.name}:slab_{rc.n}x{rc.n}x{nz}", "n1": rc.n, "n2": rc.n, "n3": rc.n3,
                   "sample_levels": nz,
                   "note": "cost per cell-step is independent of the level count; the slab keeps the run short"},
        "impl": "reference",
        "cpu_baseline": {"value": value, "unit": "cell-steps/s", "cores": workers, "kind": "port", "sample": sample},
        "e2e": {"value": value, "unit": "cell-steps/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }


def main(argv=None):
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=None,
                    help="timed steps (default 300; c4: the 50 steps the adjoint objective is defined over)")
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", choices=("ours", "reference"), default="ours")
    ap.add_argument("--config", default="c2")
    ap.add_argument("--precision", default=None)
    ap.add_argument("--n", type=int, default=0, help="override n1 = n2 (profiling cases)")
    ap.add_argument("--n3", type=int, default=0, help="override n3 (profiling cases)")
    ap.add_argument("--e2e-steps", type=int, default=20)
    ap.add_argument("--fp64-steps", type=int, default=10)
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-fp64", action="store_true")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-adjoint", action="store_true", help="c2: skip the adjoint/forward cost measurement")
    ap.add_argument("--no-ensemble", action="store_true", help="c2: skip the ensemble-over-sequential measurement")
    ap.add_argument("--reference-budget-s", type=float, default=120.0)
    ap.add_argument("--members", type=int, default=0, help="c3: first M ensemble members only")
    ap.add_argument("--ckpt", type=int, default=10, help="c4: checkpoint spacing of the adjoint")
    ap.add_argument("--levels-per-batch", type=int, default=0, help="override the phase-A batch depth")
    ap.add_argument("--solve-columns", type=int, default=0, help="override the columns per CTA of the solves")
    args = ap.parse_args(argv)
    if args.steps is None:
        args.steps = 50 if args.config == "c4" else 300
    if args.warmup < 3:
        args.warmup = 3
    world, rank, local = dist_env()
    if args.impl == "reference":
        out = run_reference(args, world, rank, local)
    elif args.config == "c3":
        out = run_ensemble(args, world, rank, local)
    elif args.config == "c4":
        out = run_adjoint(args, world, rank, local)
    else:
        out, snapshots = run_ours(args, world, rank, local)
        if out is not None and world == 1 and not args.no_adjoint and args.config == "c2":
            out["adjoint"] = adjoint_cost(args, local)
        if out is not None and world == 1 and not args.no_ensemble and args.config == "c2":
            out["ensemble"] = ensemble_cost(args, local)
        if out is not None and world == 1 and not args.no_cpu_baseline:
            out["cpu_baseline"], vs_oracle = cpu_baseline_leg(workload(args), snapshots)
            if vs_oracle and out.get("parity") is not None:
                out["parity"]["vs_oracle"] = vs_oracle
    if out is not None:
        print(json.dumps(out), flush=True)


if __name__ == "__main__":
    main()
