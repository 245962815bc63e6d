"""Benchmark of the SMAC + FENE-P + IBM time step (Mcell-steps/s).

Workload: the 256 x 128 x 128 channel with no-slip walls in y and 2 x 2
spanwise cylinders (Re 500, Wi 5, beta 0.9, L^2 900, dt 2e-4), synthetic
seeded initial state (Poiseuille + noise), see fortran8_gb300/configs.py.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]
                    [--precision auto|fp64|mixed] [--workload c3_channel]

ours:      K steps through the C ABI with the state resident in HBM, timed by
           CUDA events that the library records on its own stream; the e2e
           number times load-from-host + K single-step calls that read the
           drag history back every step + store-to-host.
reference: the CPU oracle (the reference's algorithm restated in C++, the
           reference itself cannot be compiled here) on all host cores.
Multi-GPU: the step does not shard (one domain per GPU); N ranks run N
independent replicas ("replicas only").
"""
from __future__ import annotations

import argparse
import ctypes as C
import json
import os
import statistics
import subprocess
import sys
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

from fortran8_gb300 import abi, configs  # noqa: E402
from fortran8_gb300.solver import Solver  # noqa: E402

PEAKS_FALLBACK = {"hbm_gbs": 6800.0, "bf16_tflops": 1900.0}

# Algorithmic bytes per cell of each stage: every field a stage must read once
# and write once (FFT-internal passes and marker traffic excluded).
# FP64 step, in words of 8 B:
FP64_STAGE_WORDS = {
    "eigen": 6.125,      # C (6) read, 1-byte selection code written
    "newton": 16.125,    # C, U, V, W read (9) + code; C (6) and f(C) (1) written
    "momentum": 32.0,    # U V W P, C (6), f, A0 (3), T0 (3), F (3) read; Ua (3), B (3), A0, T0 written
    "ibm": 9.0,          # Ua (3), B (3) read, Q (3) written (marker traffic excluded)
    "helmholtz": 6.0,    # Q (3) read, U* (3) written (FFT-internal passes excluded)
    "poisson": 5.0,      # U* (3) read, RHS, Phi written (FFT-internal passes excluded)
    "project": 9.0,      # U*, Phi, P read (5); U, V, W, P written (4)
}
# FP32-mixed step, in bytes.  FP32: C, f, A0, T0, F, the Helmholtz increments
# dU and the defect; double-float (hi + lo FP32, 8 B): U, V, W, P, Phi and the
# Poisson right-hand side.  F is not read when uniform (the channel's force).
MIXED_STAGE_BYTES = {
    "eigen": 25.0,       # C 24 read, code 1 written
    "newton": 65.0,      # C 24, velocity hi 12, code 1 read; C 24, f 4 written
    "momentum": 108.0,   # velocity hi 12, P 8, C 24, f 4, A0 12, T0 12 read; Q 12, A0 12, T0 12 written
    "ibm": 0.0,          # marker stencils only (not a per-cell stage)
    "helmholtz": 24.0,   # 3 x (Q 4 read, dU 4 written)
    "poisson": 96.0,     # rhs: U, V, W 24 + dU 12 read, R 8 written; solve: R hi 4 read, Phi 8 written;
                         # defect: Phi 8 + R 8 read, r 4 written; correction: r 4 read, Phi 8 read + 8 written
    "project": 84.0,     # U, V, W, P 32 + dU 12 + Phi 8 read; U, V, W, P 32 written
}
# kernels of each stage of the mixed step (for the ncu traffic of a stage)
MIXED_STAGE_KERNELS = {
    "eigen": ["k_codes3_f", "k_codes_ghost3_f"],
    "newton": ["k_update3_f", "k_newton_fix_f", "k_update_ghost3_f", "k_bc_c_pet_xz_f"],
    "momentum": ["k_momentum3_f"],
    "ibm": ["k_ibm_interp_f", "k_ibm_spread_f", "k_drag_part", "k_drag_final"],
    "helmholtz": ["3 x (k_xfwd_w, k_plane_walls_c, k_xinv_w)"],
    "poisson": ["k_poisson_rhs_df", "2 x (k_xfwd_w, k_plane_walls_c, k_xinv_w)", "k_defect_df"],
    "project": ["k_march_df", "k_bc_set"],
}


# algorithmic bytes per cell of the single-launch kernels of the mixed step
# (the share of MIXED_STAGE_BYTES each one moves), in the order of abi.KERNEL_NAMES
MIXED_KERNEL_BYTES = {
    "k_codes3_f": 25.0,        # C 24 read, code 1 written
    "k_update3_f": 65.0,       # C 24, velocity hi 12, code 1 read; C 24, f 4 written
    "k_momentum3_f": 108.0,    # the momentum stage
    "k_poisson_rhs_df": 44.0,  # U, V, W 24 + dU 12 read; rhs (hi, lo) 8 written
    "k_defect_df": 20.0,       # Phi 8 + rhs 8 read; defect 4 written
    "k_march_df": 84.0,        # U, V, W, P 32 + dU 12 + Phi 8 read; U, V, W, P 32 written
}


def load_kernel_profiles():
    """Per-kernel ncu figures of the mixed step (DRAM bytes per launch, pipe use)."""
    p = ROOT / "profiles" / "kernels_mixed_c3_channel.json"
    return json.loads(p.read_text()) if p.exists() else {}


def load_traffic(precision):
    """ncu DRAM bytes per launch of the stage kernels (profiles/traffic_<precision>_c3_channel.json)."""
    p = ROOT / "profiles" / f"traffic_{precision}_c3_channel.json"
    if p.exists():
        return json.loads(p.read_text())
    return {}


def load_peaks():
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        d = json.loads(p.read_text())
        return {"hbm_gbs": float(d["hbm_gbs"]), "bf16_tflops": float(d["bf16_tflops"])}, "measured"
    return PEAKS_FALLBACK, "fallback"


class ClockSampler:
    """nvidia-smi clock / throttle sampling during the timed region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index: int):
        self.idx = gpu_index
        self.proc = None
        self.path = Path(os.environ.get("TMPDIR", "/tmp")) / f"f8_clocks_{os.getpid()}.csv"

    def __enter__(self):
        try:
            self.fh = open(self.path, "w")
            self.proc = subprocess.Popen(["nvidia-smi", f"--id={self.idx}", f"--query-gpu={self.FIELDS}",
                                          "--format=csv,noheader,nounits", "-lms", "100"],
                                         stdout=self.fh, stderr=subprocess.DEVNULL)
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

    def summary(self):
        if self.proc is None or not self.path.exists():
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        sm, smax, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in self.path.read_text().splitlines():
            parts = [p.strip() for p in line.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                smax = float(parts[2])
            except ValueError:
                continue
            for n, v in zip(names, parts[5:9]):
                if v.lower() == "active":
                    reasons.add(n)
        self.path.unlink(missing_ok=True)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": smax,
                "reasons": sorted(reasons), "samples": len(sm)}


def dist_init():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if ws > 1:
        import torch.distributed as dist
        dist.init_process_group("gloo")
    return ws, rank, local


def barrier(ws):
    if ws > 1:
        import torch.distributed as dist
        dist.barrier()


def max_over_ranks(ws, x):
    if ws == 1:
        return x
    import torch
    import torch.distributed as dist
    t = torch.tensor([x], dtype=torch.float64)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def state_bytes(st):
    return int(sum(a.nbytes for a in st.arrays.values()))


def pinned_state(st):
    """Copy a state into page-locked host memory (numpy views of pinned tensors)."""
    import torch
    out = {}
    for k, a in st.arrays.items():
        t = torch.empty(a.shape, dtype=torch.float64, pin_memory=True)
        v = t.numpy()
        v[...] = a
        out[k] = (t, v)
    from fortran8_gb300.solver import State
    return State({k: v for k, (t, v) in out.items()}), [t for t, _ in out.values()]


def oracle_fns():
    subprocess.run(["make", "-s", "-C", str(ROOT / "oracle")], check=True)
    lib = C.CDLL(str(ROOT / "oracle" / "liboracle_f8.so"))
    lib.f8o_max_threads.restype = C.c_int
    return abi.bind(lib, "f8o_"), lib


def cpu_baseline(w, steps_cap=2, budget_s=30.0):
    """Oracle on the host cores (all threads) on a bounded sample of the workload,
    and one step on a single thread (the reference's code is serial)."""
    fns, lib = oracle_fns()
    threads = int(lib.f8o_max_threads())
    st0 = configs.initial_state(w)

    def sample(cap, budget):
        with Solver(fns, w.grid, w.phys, w.cyls) as s:
            s.load(st0)
            t0 = time.perf_counter()
            n = 0
            while n < cap:
                s.step(1, want_drag=True)
                n += 1
                if time.perf_counter() - t0 > budget:
                    break
            return n, time.perf_counter() - t0

    n, el = sample(steps_cap, budget_s)
    out = {"value": w.cells * n / el / 1e6, "unit": "Mcell-steps/s", "cores": threads, "kind": "port",
           "sample": f"{n} full step(s) of {w.grid.nx}x{w.grid.ny}x{w.grid.nz} from the seeded initial state, "
                     f"FP64, {threads} OpenMP threads, {el:.1f} s"}
    lib.f8o_set_threads(1)
    try:
        n1, el1 = sample(1, budget_s)
    finally:
        lib.f8o_set_threads(threads)
    out["one_thread"] = {"value": w.cells * n1 / el1 / 1e6, "unit": "Mcell-steps/s", "cores": 1,
                         "sample": f"{n1} full step(s), FP64, 1 thread, {el1:.1f} s"}
    return out


def run_reference(args, w, budget_s=90.0):
    """The CPU oracle on all host cores.  Each step is a full step of the workload;
    the timed sample stops after K steps or once the time budget is spent, so
    the run ends within a few minutes (the sample is stated in the output)."""
    ws, rank, _ = dist_init()
    if rank != 0:
        return 0
    fns, lib = oracle_fns()
    threads = int(lib.f8o_max_threads())
    with Solver(fns, w.grid, w.phys, w.cyls) as s:
        s.load(configs.initial_state(w))
        nw, t0 = 0, time.perf_counter()
        while nw < args.warmup and (nw < 3 or time.perf_counter() - t0 < budget_s / 3):
            s.step(1)
            nw += 1
        t0 = time.perf_counter()
        n = 0
        while n < args.steps:
            s.step(1)
            n += 1
            if time.perf_counter() - t0 > budget_s:
                break
        el = time.perf_counter() - t0
    v = w.cells * n / el / 1e6
    sample = (f"{n} full FP64 steps of {w.grid.nx}x{w.grid.ny}x{w.grid.nz} (of {args.steps} requested, "
              f"{budget_s:.0f} s budget) after {nw} warm-up step(s), {threads} OpenMP threads")
    line = {"impl": "reference", "metric": "Mcell-steps/s", "value": v, "unit": "Mcell-steps/s",
            "n_gpus": args.gpus, "steps": n, "warmup": nw, "ms_per_step": el * 1e3 / n,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": {"workload": w.name, "grid": [w.grid.nx, w.grid.ny, w.grid.nz], "cylinders": len(w.cyls),
                       "poisson": "fft+tridiagonal"},
            "cpu_baseline": {"value": v, "unit": "Mcell-steps/s", "cores": threads, "kind": "port", "sample": sample},
            "e2e": {"value": v, "unit": "Mcell-steps/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line))
    return 0


def run_ours(args, w):
    import torch
    ws, rank, local = dist_init()
    from fortran8_gb300 import build as b, lib as flib
    if rank == 0:
        b.build()
    barrier(ws)
    torch.cuda.set_device(local)
    fns = flib.functions()
    prec = {"fp64": abi.F8_FP64, "mixed": abi.F8_MIXED}[args.precision]
    pois = {"fft": abi.F8_POISSON_FFT, "sor": abi.F8_POISSON_SOR}[args.poisson]
    pois_name = "fft+tridiagonal" if args.poisson == "fft" else "red-black SOR (omega %.2f)" % w.phys.sor_omega
    st0 = configs.initial_state(w)
    cells = w.cells
    peaks, peak_kind = load_peaks()
    with Solver(fns, w.grid, w.phys, w.cyls, precision=prec, poisson=pois) as s:
        s.load(st0)
        s.step(args.warmup)
        # timed region: CUDA events around the f8_step call only (the mixed
        # step then replays its CUDA graphs)
        s.set_timing(False)
        s.timing_reset()
        torch.cuda.synchronize()
        barrier(ws)
        with ClockSampler(local) as clk:
            status, drag = s.step(args.steps)
        torch.cuda.synchronize()
        barrier(ws)
        tot_ms, _, _ = s.timing()
        clocks = clk.summary()
        diag = s.diagnostics()
        launches = int(diag.kernel_launches)
        # stage breakdown: CUDA events at the stage boundaries of each step
        s.set_timing(True)
        s.timing_reset()
        s.step(min(args.steps, 100))
        _, stage_ms, nst = s.timing()
        kern_ms, kern_n = s.kernel_timing() if prec == abi.F8_MIXED else (None, 0)
    ms = max_over_ranks(ws, tot_ms)
    value = cells * args.steps * ws / (ms / 1e3) / 1e6
    # e2e: host arrays in, K single-step calls reading the drag every step, host
    # arrays out; timed on the host clock after one untimed repetition (which
    # touches every page-locked buffer once), median of five (the host is
    # shared).  The store leaves out the body force, an input the caller keeps.
    pst, _keep = pinned_state(st0)
    from fortran8_gb300.solver import empty_state
    pout, _keep_out = pinned_state(empty_state(w.grid))
    for f in ("fx", "fy", "fz"):
        del pout.arrays[f]
    reps, parts = [], []
    with Solver(fns, w.grid, w.phys, w.cyls, precision=prec, poisson=pois) as s:
        s.load(pst)
        s.step(args.warmup)
        for rep in range(6):
            torch.cuda.synchronize()
            barrier(ws)
            t0 = time.perf_counter()
            s.load(pst, step0=0)
            t1 = time.perf_counter()
            for _ in range(args.steps):
                s.step(1)
            t2 = time.perf_counter()
            s.store(pout)
            torch.cuda.synchronize()
            t3 = time.perf_counter()
            if rep > 0:
                reps.append(max_over_ranks(ws, t3 - t0))
                parts.append((t1 - t0, t2 - t1, t3 - t2))
    e2e_s = sorted(reps)[len(reps) // 2]
    e2e_parts = parts[reps.index(e2e_s)]
    out_bytes = int(sum(a.nbytes for a in pout.arrays.values()))
    # the FP64 path on the same workload over the workload's whole horizon and
    # the per-field and drag differences (accuracy gate)
    cmp = None
    if prec == abi.F8_MIXED and not args.no_fp64_compare:
        cmp = fp64_compare(fns, w, pois, args.compare_steps or w.steps, value)
    adj = None
    if not args.no_adjoint:
        adj = adjoint_cost(fns, args.adjoint_steps, args.adjoint_every, args.adjoint_grid, args.adjoint_workload,
                           args.adjoint_mixed_prefix, args.adjoint_precision)
        if args.adjoint_precision == "mixed" and not args.adjoint_grid:
            # the same gradient in FP64 (the parity path), for its own ratio
            adj["fp64"] = adjoint_cost(fns, args.adjoint_steps, args.adjoint_every, None, args.adjoint_workload,
                                       0, "fp64")
        if args.adjoint_precision == "mixed" and not args.adjoint_grid and ws == 1 and not args.no_adjoint_large:
            # the mixed gradient of the 512 x 256 x 256 channel over a 100-step
            # window with a checkpoint every 10 steps (one GPU only: it holds
            # about 170 GB of tape and checkpoints)
            adj["large"] = adjoint_cost(fns, 100, 10, None, "c5_large", 0, "mixed")
    sb = state_bytes(st0)
    ncyl = len(w.cyls)
    e2e = {"value": cells * args.steps * ws / e2e_s / 1e6, "unit": "Mcell-steps/s", "repetitions": len(reps),
           "values": [cells * args.steps * ws / r / 1e6 for r in reps],
           "median_rep_ms": {"load": e2e_parts[0] * 1e3, "steps": e2e_parts[1] * 1e3, "store": e2e_parts[2] * 1e3},
           "h2d_bytes_per_step": int(sb / args.steps),
           "d2h_bytes_per_step": int(out_bytes / args.steps + ncyl * 3 * 8 + 8)}
    if rank != 0:
        return 0
    # roofline of the dominant kernel: the single-launch kernel of the mixed
    # step with the longest event-timed duration in the stage-timing pass
    per_step = stage_ms / max(nst, 1)
    names = abi.STAGE_NAMES
    if prec == abi.F8_FP64:
        stage_bytes = {k: v * 8 for k, v in FP64_STAGE_WORDS.items()}
    else:
        stage_bytes = MIXED_STAGE_BYTES
    hbm = peaks["hbm_gbs"]
    roof = {"stage_ms_per_step": {n: float(v) for n, v in zip(names, per_step)},
            "stage_hbm_frac": {n: (stage_bytes[n] * cells / (float(v) / 1e3) / 1e9 / hbm) if v > 0 else None
                               for n, v in zip(names, per_step)},
            "step_bytes": sum(stage_bytes.values()) * cells,
            "step_hbm_frac": sum(stage_bytes.values()) * cells / (ms / args.steps / 1e3) / 1e9 / hbm}
    if kern_ms is not None:
        prof = load_kernel_profiles()
        kms = {n: float(v) / max(kern_n, 1) for n, v in zip(abi.KERNEL_NAMES, kern_ms)}
        top = max(kms, key=kms.get)
        byts = MIXED_KERNEL_BYTES[top] * cells
        achieved = byts / (kms[top] / 1e3) / 1e9
        pk = prof.get(top, {})
        roof = {"bound": "hbm", "kernel": top, "achieved": achieved, "peak": hbm, "unit": "GB/s",
                "frac": achieved / hbm, "peak_kind": peak_kind, "traffic": pk.get("dram_bytes"),
                "algorithmic_bytes": byts, "kernel_ms": kms[top], "launches_timed": int(kern_n),
                "compute": {k: pk[k] for k in ("issue_active", "fma_pipe", "fp64_pipe", "bound") if k in pk},
                "kernels": {n: {"ms": v, "hbm_frac": MIXED_KERNEL_BYTES[n] * cells / (v / 1e3) / 1e9 / hbm if v > 0 else None,
                                **({"ncu_bound": prof[n]["bound"]} if n in prof and "bound" in prof[n] else {})}
                            for n, v in kms.items()},
                "profiles": "profiles/kernels_mixed_c3_channel.json (ncu per-kernel captures)",
                **roof}
    else:
        top = int(np.argmax(per_step))
        byts = stage_bytes[names[top]] * cells
        achieved = byts / (per_step[top] / 1e3) / 1e9
        roof = {"bound": "hbm", "kernel_stage": names[top], "achieved": achieved, "peak": hbm, "unit": "GB/s",
                "frac": achieved / hbm, "peak_kind": peak_kind, "traffic": load_traffic(args.precision).get(names[top]),
                "algorithmic_bytes": byts, **roof}
    line = {"metric": "Mcell-steps/s", "value": value, "unit": "Mcell-steps/s", "n_gpus": ws, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": ms / args.steps, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f64" if prec == abi.F8_FP64 else "f32+f64",
            "data": "synthetic (seeded Poiseuille + noise, C = I)",
            "config": {"workload": w.name, "grid": [w.grid.nx, w.grid.ny, w.grid.nz], "cylinders": ncyl,
                       "precision": args.precision, "poisson": pois_name,
                       "l2": "inputs larger than L2 (state %.2f GB)" % (sb / 1e9), "parallelism": f"replicas{ws}"},
            "status": int(status), "div_max": diag.div_max, "newton_iters_per_cell_step": diag.newton_iters / (cells * args.steps),
            "drag_last": drag[-1].tolist() if drag is not None else None,
            "gpu_launches": launches, "clocks": clocks, "roofline": roof, "e2e": e2e, "fp64_compare": cmp,
            "adjoint": adj}
    if not args.no_cpu_baseline:
        line["cpu_baseline"] = cpu_baseline(w)
    print(json.dumps(line))
    return 0


def fp64_compare(fns, w, pois, nsteps, mixed_value):
    """Mixed and FP64 runs from the same seeded state over nsteps steps: the
    drag histories (largest difference over all steps relative to the largest
    FP64 drag, per component x / y) and the relative L2 differences of the
    final u, v, w, p and trC over the interior cells.  The FP64 run is also
    the FP64-GPU speed (CUDA events of its f8_step calls)."""
    st0 = configs.initial_state(w)
    res = {}
    for name, prec in (("fp64", abi.F8_FP64), ("mixed", abi.F8_MIXED)):
        with Solver(fns, w.grid, w.phys, w.cyls, precision=prec, poisson=pois) as s:
            s.load(st0)
            s.timing_reset()
            drags = []
            done = 0
            while done < nsteps:
                n = min(500, nsteps - done)
                _, d = s.step(n)
                if d is not None:
                    drags.append(d)
                done += n
            tms, _, _ = s.timing()
            res[name] = (np.concatenate(drags) if drags else None, s.store(), tms)
    (d64, o64, t64), (dm, om, _) = res["fp64"], res["mixed"]

    def rel(a, b):
        return float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300))

    inner = (slice(1, -1), slice(1, -1), slice(1, -1))
    vel = ("u", "v", "w", "p") if w.grid.dim == 3 else ("u", "v", "p")
    errs = {f: rel(om[f][inner], o64[f][inner]) for f in vel}
    # trace of C: (xx, xy, xz, yy, yz, zz) in 3D, (xx, xy, yy) in 2D
    tq = (0, 3, 5) if w.grid.dim == 3 else (0, 2)
    tr = lambda o: sum(o["c"][inner][..., q] for q in tq)
    errs["trC"] = rel(tr(om), tr(o64))
    out = {"steps_compared": nsteps, "field_rel_l2": errs}
    if d64 is not None:
        scale = np.max(np.abs(d64[..., 0]))
        out["drag_rel_err_vs_fp64"] = float(np.max(np.abs(dm[..., 0] - d64[..., 0])) / scale)
        out["drag_rel_err_by_component"] = {
            c: float(np.max(np.abs(dm[..., q] - d64[..., q])) / np.max(np.abs(d64[..., q])))
            for q, c in ((0, "x"), (1, "y"))}
        tail = max(1, nsteps // 10)
        out["drag_rel_err_last_10pct"] = float(np.max(np.abs(dm[-tail:, :, 0] - d64[-tail:, :, 0])) / scale)
    v64 = w.cells * nsteps / (t64 / 1e3) / 1e6
    out.update({"fp64_value": v64, "fp64_ms_per_step": t64 / nsteps, "mixed_over_fp64": mixed_value / v64})
    return out


def adjoint_cost(fns, steps, every, grid=None, workload="c4_adjoint", mixed_prefix=0, precision="mixed"):
    """Cost of the gradient (f8_grad: forward pass with checkpoints, which on
    the mixed path also keeps the tapes of as many segments as fit in device
    memory, recomputation of the other segments, adjoint sweep) over that of
    the forward (f8_step) in the same precision.

    Default: the adjoint workload, a 128 x 64 x 64 channel with 2 cylinders,
    gradient of the time-averaged total drag w.r.t. Wi, beta, L^2 and the
    centres, in FP32-mixed precision.  With mixed_prefix > 0 the FP32-mixed
    step first advances the seeded state that many steps (timed), and the
    gradient window starts from its state.  The forward and the gradient are
    each timed by CUDA events on the default stream around one synchronous
    call, after a warm-up call of each."""
    import torch
    w = configs.WORKLOADS[workload]()
    if grid:
        w = configs.scaled(w, *grid)
    prec = {"fp64": abi.F8_FP64, "mixed": abi.F8_MIXED}[precision]
    st0 = configs.initial_state(w)
    step0 = 0
    pre = None
    if mixed_prefix > 0:
        with Solver(fns, w.grid, w.phys, w.cyls, precision=abi.F8_MIXED) as sm:
            sm.load(st0)
            sm.timing_reset()
            sm.step(mixed_prefix)
            tms, _, _ = sm.timing()
            st0 = sm.store()
        step0 = mixed_prefix
        pre = {"mixed_steps": mixed_prefix, "mixed_ms_per_step": tms / mixed_prefix,
               "mixed_value": w.cells * mixed_prefix / (tms / 1e3) / 1e6}

    def timed(fn):
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        torch.cuda.synchronize()
        e0.record()
        r = fn()
        e1.record()
        torch.cuda.synchronize()
        return r, e0.elapsed_time(e1)

    with Solver(fns, w.grid, w.phys, w.cyls, precision=prec) as s:
        s.load(st0, step0)
        s.step(2)
        # a warm-up gradient of the same horizon: its buffers and the CUDA
        # graphs of its tape slots are made before the timed call
        s.load(st0, step0)
        s.grad(steps, every)
        s.load(st0, step0)
        _, tf = timed(lambda: s.step(steps))
        s.load(st0, step0)
        (status, J, dp, _, _), tg = timed(lambda: s.grad(steps, every))
    out = {"workload": w.name, "grid": [w.grid.nx, w.grid.ny, w.grid.nz], "cylinders": len(w.cyls),
           "steps": steps, "checkpoint_every": every, "precision": precision, "step0": step0,
           "forward_ms_per_step": tf / steps, "grad_ms_per_step": tg / steps,
           "adjoint_over_forward": tg / tf, "J": J,
           "dJ_dparams": {"wi": dp[0], "beta": dp[1], "lp2": dp[2], "centres": dp[3:].tolist()},
           "status": int(status)}
    if pre:
        out["mixed_prefix"] = pre
        out["grad_over_mixed_forward"] = (tg / steps) / pre["mixed_ms_per_step"]
    elif precision == "mixed":
        out["grad_over_mixed_forward"] = tg / tf
    return out


# launches per step of each stage kernel of the mixed step (wall channel)
MIXED_STAGE_LAUNCHES = {
    "eigen": {"k_codes3_f": 1, "k_codes_ghost3_f": 1},
    "newton": {"k_update3_f": 1, "k_newton_fix_f": 1, "k_update_ghost3_f": 1, "k_bc_c_pet_xz_f": 1},
    "momentum": {"k_momentum3_f": 1, "k_extrap_ghost_f": 1},
    "ibm": {"k_ibm_interp_f": 1, "k_ibm_spread_f": 1, "k_drag_part": 1, "k_drag_final": 1},
    "helmholtz": {"k_xfwd_w": 3, "k_plane_walls_c": 3, "k_xinv_w": 3},
    "poisson": {"k_poisson_rhs_df": 1, "k_xfwd_w": 2, "k_plane_walls_c": 2, "k_xinv_w": 2, "k_defect_df": 1},
    "project": {"k_march_df": 1, "k_bc_set": 1},
}


def summarize_ncu(csv_path, traffic_out=None):
    """Launch list of an ncu --csv log (per kernel: launches, total time, share)
    and, when the log holds dram__bytes_{read,write}.sum, the DRAM bytes per
    step of each stage of the mixed step (written to traffic_out as JSON)."""
    import collections
    import csv
    import io
    import re
    txt = Path(csv_path).read_text()
    rows = list(csv.DictReader(io.StringIO(txt[txt.index('"ID"'):])))
    launches = collections.defaultdict(dict)
    for r in rows:
        launches[r["ID"]]["name"] = r["Kernel Name"]
        launches[r["ID"]]["grid"] = r["Grid Size"]
        launches[r["ID"]]["block"] = r["Block Size"]
        launches[r["ID"]][r["Metric Name"]] = float(r["Metric Value"].replace(",", ""))

    def base(n):
        n = re.sub(r"\(.*", "", n).replace("unnamed>::", "").replace("f8::", "").replace("void ", "")
        return re.sub(r"<.*", "", n).strip()

    agg = collections.defaultdict(lambda: [0, 0.0, 0.0])
    for L in launches.values():
        a = agg[base(L["name"])]
        a[0] += 1
        a[1] += L.get("gpu__time_duration.sum", 0.0) / 1e3
        a[2] += L.get("dram__bytes_read.sum", 0.0) + L.get("dram__bytes_write.sum", 0.0)
    tot = sum(v[1] for v in agg.values())
    print("| kernel | launches | total us | share | avg us | DRAM MB / launch |")
    print("|---|---|---|---|---|---|")
    for k, v in sorted(agg.items(), key=lambda kv: -kv[1][1]):
        print(f"| {k} | {v[0]} | {v[1]:.1f} | {100 * v[1] / max(tot, 1e-9):.1f}% | {v[1] / v[0]:.1f} | "
              f"{v[2] / v[0] / 1e6:.1f} |")
    print(f"total {tot:.1f} us over {sum(v[0] for v in agg.values())} launches")
    if traffic_out:
        per = {k: v[2] / v[0] for k, v in agg.items() if v[0]}
        out = {st: sum(per.get(k, 0.0) * n for k, n in ks.items()) for st, ks in MIXED_STAGE_LAUNCHES.items()}
        out["source"] = ("ncu dram__bytes_read.sum + dram__bytes_write.sum, mean per launch x launches per step "
                         f"({Path(csv_path).name})")
        Path(traffic_out).write_text(json.dumps(out, indent=1) + "\n")
        print("wrote", traffic_out)
    return 0


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=400)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--precision", default="auto", choices=["auto", "fp64", "mixed"])
    ap.add_argument("--workload", default="c3_channel", choices=sorted(configs.WORKLOADS))
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-fp64-compare", action="store_true")
    ap.add_argument("--compare-steps", type=int, default=0,
                    help="steps of the mixed-vs-FP64 comparison (default: the workload's horizon, 2000)")
    ap.add_argument("--no-adjoint", action="store_true", help="skip the adjoint/forward cost measurement")
    ap.add_argument("--no-adjoint-large", action="store_true",
                    help="skip the gradient of the 512 x 256 x 256 channel in the adjoint measurement")
    ap.add_argument("--adjoint-steps", type=int, default=400)
    ap.add_argument("--adjoint-every", type=int, default=20, help="checkpoint interval of the adjoint run")
    ap.add_argument("--adjoint-only", action="store_true",
                    help="print only the adjoint/forward cost measurement (JSON)")
    ap.add_argument("--adjoint-grid", type=int, nargs=3, metavar=("NX", "NY", "NZ"),
                    help="scale the adjoint workload (small cases for profiling)")
    ap.add_argument("--adjoint-workload", default="c4_adjoint", choices=sorted(configs.WORKLOADS))
    ap.add_argument("--adjoint-mixed-prefix", type=int, default=0,
                    help="FP32-mixed steps before the adjoint window (with --adjoint-only)")
    ap.add_argument("--adjoint-precision", default="mixed", choices=["mixed", "fp64"],
                    help="precision of the gradient whose cost is measured")
    ap.add_argument("--poisson", default="fft", choices=["fft", "sor"],
                    help="pressure solver: FFT + tridiagonal (default) or red-black SOR")
    ap.add_argument("--grid", type=int, nargs=3, metavar=("NX", "NY", "NZ"),
                    help="scale the workload to this grid (small cases for profiling)")
    ap.add_argument("--summarize-ncu", metavar="CSV", help="summarise an ncu --csv log instead of running")
    ap.add_argument("--traffic-out", metavar="JSON", help="with --summarize-ncu: write per-stage DRAM bytes")
    args = ap.parse_args()
    if args.summarize_ncu:
        return summarize_ncu(args.summarize_ncu, args.traffic_out)
    if args.precision == "auto":
        args.precision = "mixed"
    w = configs.WORKLOADS[args.workload]()
    if args.grid:
        w = configs.scaled(w, *args.grid)
    if args.impl == "reference":
        return run_reference(args, w)
    if args.adjoint_only:
        import torch
        from fortran8_gb300 import build as b, lib as flib
        b.build()
        torch.cuda.set_device(0)
        print(json.dumps(adjoint_cost(flib.functions(), args.adjoint_steps, args.adjoint_every, args.adjoint_grid,
                                      args.adjoint_workload, args.adjoint_mixed_prefix, args.adjoint_precision)))
        return 0
    return run_ours(args, w)


if __name__ == "__main__":
    sys.exit(main())
