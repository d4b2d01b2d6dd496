#!/usr/bin/env python
"""Benchmark of the Armon time step on GB300: cell-updates/s.

Workload (the single-domain drop-in case): circular Sod on [0,1]^2, 4096 x 4096 real cells, 5 ghost
layers, FP64, gamma 1.4, rho/p = 1/1 inside radius 0.2 and 0.125/0.1 outside, GAD acoustic fluxes
with the minmod limiter, second-order Euler remap, Sequential X/Y splitting, CFL 0.6, 200 cycles.
A step is one solver cycle (dt reduction + X pass + Y pass) over the whole grid.  The timed steps
are the last K cycles of the 200-cycle run (its most expensive part: the fronts are widest); the
whole run's rate is reported beside them.  The state (4 x 135 MB per buffer set) is larger than
L2, so no flush is needed between steps.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl gb300|reference]

One JSON line (rank 0).  Beside the headline it holds, at N = 1: `parity` (the GPU run against the
strict oracle, field by field and dt cycle by cycle), `e2e` (the whole solve through the C ABI
with host buffers; `e2e_cold` the same in a process that has not measured this geometry's tiling),
`cpu_baseline` (the reference's own sources, Release flags, OpenMP on the host cores), and compact
runs of the other configurations: `fp32` (8192^2 FP32 variant, with its accuracy), `batch` (the
256-domain mix, batched against the plain path) and `serve` (a Poisson request trace).

--impl reference times the reference's own time loop (its sources compiled against the project's
Kokkos API shim with its Release flags, OpenMP) on the host cores.  N > 1 runs N independent
replicas (one per GPU), weak scaling.
"""
from __future__ import annotations

import argparse
import ctypes as C
import json
import os
import re
import statistics
import subprocess
import sys
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(ROOT, "armon-kokkos_gb300"))
sys.path.insert(0, os.path.join(ROOT, "tests"))

METRIC = "cell-updates/s"
WORKLOAD = dict(test="Sod_circ", scheme="GAD", projection="euler_2nd", limiter="Minmod", splitting="Sequential",
                nghost=5, nx=4096, ny=4096, cfl=0.6, max_time=1e9, test_option=0.04)
BYTES_PER_CELL_UPDATE = 64          # read + write rho, u, v, E once per cycle (FP64)
PARITY_FIELDS = ("rho", "umat", "vmat", "Emat", "pmat")


def config(nx: int, ny: int, n: int, precision: int = 64, cycles: int = 200) -> dict:
    prec = "FP64" if precision == 64 else "FP32 storage and arithmetic, FP64 dt and conservation sums"
    esize = 8 if precision == 64 else 4
    return {"workload": f"Sod_circ {nx}x{ny} {prec}, GAD-minmod + euler_2nd, CFL 0.6, radius 0.2, "
                        f"Sequential splitting, {cycles} cycles",
            "nx": nx, "ny": ny, "nghost": 5, "gamma": 1.4, "scheme": "GAD", "limiter": "Minmod",
            "projection": "euler_2nd", "splitting": "Sequential", "cfl": 0.6, "radius": 0.2, "run_cycles": cycles,
            "step": "one solver cycle (dt_CFL + X pass + Y pass)",
            "l2": "inputs larger than L2 (state: 4 arrays x %d MB per buffer set)" % ((nx + 10) * (ny + 10) * esize // 2**20),
            "parallelism": f"replicas x{n}" if n > 1 else "single domain"}


def measured_peaks() -> tuple[float, str]:
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            return float(json.load(f)["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


def profiled(key: str, precision: int = 64) -> float | None:
    """A per-cell figure from the committed ncu summary (profiles/sweep_f64_sod_circ.md or
    profiles/sweep_f32_sod_circ.md)."""
    path = os.path.join(ROOT, "profiles", "sweep_f%d_sod_circ.md" % precision)
    try:
        txt = open(path).read()
    except OSError:
        return None
    m = re.search(r"(?m)^" + re.escape(key) + r":\s*([0-9.eE+-]+)", txt)
    return float(m.group(1)) if m else None


class ClockSampler:
    """nvidia-smi clocks / throttle reasons sampled every 200 ms during the timed region."""
    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
         "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
         "clocks_event_reasons.sw_power_cap")

    def __init__(self):
        self.proc = None
        self.lines: list[str] = []

    def start(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", f"--query-gpu={self.Q}", "--format=csv,noheader,nounits",
                                          "-lms", "200"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except Exception:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self) -> dict:
        if not self.proc:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        rows = [[x.strip() for x in ln.split(",")] for ln in self.lines]
        rows = [r for r in rows if len(r) >= 9]
        if not rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["no samples"]}
        # the busiest GPU (highest power) is ours
        by_gpu: dict[str, list] = {}
        for r in rows:
            by_gpu.setdefault(r[0], []).append(r)

        def med_power(g):
            ps = [float(r[3]) for r in by_gpu[g] if r[3] not in ("", "[N/A]")]
            return statistics.median(ps) if ps else 0.0

        gpu = max(by_gpu, key=med_power)
        rs = by_gpu[gpu]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[k] for r in rs for k in range(4) if r[5 + k].lower() == "active"})
        return {"sm_mhz": statistics.median(float(r[1]) for r in rs), "sm_max_mhz": float(rs[0][2]),
                "reasons": reasons, "samples": len(rs), "power_w_median": med_power(gpu)}


def sampled(fn):
    """Runs fn() with the clock sampler on; returns (fn's result, clocks)."""
    smp = ClockSampler().start()
    time.sleep(0.2)
    try:
        out = fn()
    finally:
        clocks = smp.stop()
    return out, clocks


def max_over_ranks(x: float, world: int, device: str = "cuda") -> float:
    """The largest of every rank's x (the slowest rank's time); the identity on one rank."""
    import torch

    t = torch.tensor([x], dtype=torch.float64, device=device)
    if world > 1:
        torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
    return float(t.item())


def whole_job_rate(units_per_rank: float, world: int, seconds_max: float) -> float:
    """Units all ranks processed (each rank a replica of the same workload) over the slowest time."""
    return units_per_rank * world / seconds_max


def dist_info() -> tuple[int, int, int]:
    return int(os.environ.get("RANK", 0)), int(os.environ.get("WORLD_SIZE", 1)), int(os.environ.get("LOCAL_RANK", 0))


def l1_rel(a, b) -> float:
    """sum |a - b| / sum |b| (b the reference result)."""
    import numpy as np

    return float(np.abs(a - b).sum() / np.abs(b).sum())


def max_rel(a, b) -> float:
    """max |a - b| / |b| over the cells where b != 0, and max |a - b| where b == 0."""
    import numpy as np

    d = np.abs(a - b)
    nz = b != 0
    m1 = float((d[nz] / np.abs(b[nz])).max()) if nz.any() else 0.0
    m0 = float(d[~nz].max()) if (~nz).any() else 0.0
    return max(m1, m0)


# ---------------------------------------------------------------- the reference's CPU path
def reference_driver() -> str | None:
    """oracle/_ref/fast/ref_driver: the reference's own sources (staged in baseline/_ref) with its
    Release flags, built on this machine on first use; None when the tree is not there."""
    exe = os.path.join(ROOT, "oracle", "_ref", "fast", "ref_driver")
    if not os.path.exists(exe):
        if not os.path.isdir(os.path.join(ROOT, "baseline", "_ref", "src", "kernels")):
            return None
        r = subprocess.run(["make", "-C", os.path.join(ROOT, "oracle"), "ref-fast", f"-j{os.cpu_count() or 4}"],
                           capture_output=True, text=True)
        if r.returncode != 0 or not os.path.exists(exe):
            return None
    return exe


def cpu_model() -> str:
    try:
        m = re.search(r"Model name:\s*(.+)", subprocess.run(["lscpu"], capture_output=True, text=True).stdout)
        return m.group(1).strip() if m else ""
    except OSError:
        return ""


def reference_cpu(nx: int, ny: int, cycles: int, warmup: int) -> dict:
    """The reference's time_loop (src/armon_2D.cpp:327-386) on the host cores: `warmup` cycles, then
    `cycles` timed by the reference itself; the rate is its grind time's inverse
    (src/armon_2D.cpp:374-382)."""
    exe = reference_driver()
    if exe is None:
        raise RuntimeError("the reference tree is not staged (make -C oracle stage)")
    threads = os.cpu_count() or 1
    env = dict(os.environ, OMP_NUM_THREADS=str(threads), OMP_PROC_BIND="close", OMP_PLACES="cores")
    args = [exe, "-", "test=Sod_circ", "scheme=GAD", "projection=euler_2nd", "limiter=Minmod",
            "splitting=Sequential", "nghost=5", f"nx={nx}", f"ny={ny}", "cfl=0.6", "max_time=1e9",
            "radius2=0.04", f"bench_cycles={cycles}", f"bench_warmup={warmup}"]
    r = subprocess.run(args, capture_output=True, text=True, env=env, check=True)
    kv = dict(tok.split("=") for tok in r.stdout.strip().splitlines()[-1].split()[1:])
    grind_us = float(kv["grind_us"])
    return {"value": 1e6 / grind_us, "unit": METRIC, "cores": int(kv["threads"]), "kind": "reference",
            "sample": f"{kv['cycles']} cycles of the {nx}x{ny} workload after {warmup} warm-up cycles: the reference's "
                      "own time_loop and grind time (its src/ and src/kernels/ compiled unchanged against the "
                      "project's Kokkos API shim, -O3 -funroll-loops -ffast-math, OpenMP static schedule)",
            "seconds": float(kv["seconds"]), "grind_us_per_cell_cycle": grind_us, "cpu": cpu_model(),
            "omp": "OMP_PROC_BIND=close OMP_PLACES=cores"}


def port_cpu(nx: int, ny: int, cycles: int) -> dict:
    """The oracle (the project's C restatement of the reference) built with the reference's Release
    flags, OpenMP on the host cores, `cycles` cycles after init."""
    import oracle_lib as O

    L = O.lib(fast=True)
    case = O.Case(**WORKLOAD)
    case.nx, case.ny = nx, ny
    p = O.make_params(case, L)
    st = O.OracleState(p)
    L.o_init_test_p(C.byref(p), C.byref(st.data), 0)
    p.cycle, p.time, p.current_cycle_dt, p.next_cycle_dt = 0, 0.0, 0.0, 0.0
    L.o_update_axis(C.byref(p), 0)
    L.o_update_EOS(C.byref(p), C.byref(st.data))
    t0 = time.perf_counter()
    for _ in range(cycles):
        assert L.o_solver_cycle(C.byref(p), C.byref(st.data)) == 0
        p.time += p.current_cycle_dt
        p.cycle += 1
    secs = time.perf_counter() - t0
    return {"value": nx * ny * cycles / secs, "unit": METRIC, "cores": L.o_num_threads(), "kind": "port",
            "sample": f"{cycles} cycles of the {nx}x{ny} workload after init (oracle/armon_oracle.c, -O3 -ffast-math, "
                      "OpenMP)", "seconds": secs}


def run_reference(args) -> None:
    rank, world, _ = dist_info()
    if rank != 0:
        return
    nx = ny = args.size
    try:
        cb = reference_cpu(nx, ny, args.steps, args.warmup)
    except Exception as e:
        cb = dict(port_cpu(nx, ny, args.steps), note=f"reference build unavailable here ({e}); the oracle port instead")
    value = cb["value"]
    out = {"metric": METRIC, "value": value, "unit": METRIC, "impl": "reference", "n_gpus": args.gpus,
           "steps": args.steps, "warmup": args.warmup, "ms_per_step": nx * ny / value * 1e3,
           "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
           "config": config(nx, ny, 1), "cpu_baseline": cb,
           "e2e": {"value": value, "unit": METRIC, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(out), flush=True)


# ---------------------------------------------------------------- parity against the oracle
def parity(A, case, cycles: int, precision: int = 64) -> dict:
    """The GPU solver (default options: measured tiling, longest-first dispatch, split passes, reuse)
    against the strict oracle, cycle by cycle: max and L1 relative error per field after `cycles`
    cycles, and the largest relative difference of (current dt, next dt, time) over every cycle."""
    import numpy as np

    import oracle_lib as O

    L = O.lib()
    c = O.Case(**{**case.__dict__, "max_cycles": cycles})
    p = O.make_params(c, L)
    st = O.OracleState(p)
    L.o_init_test_p(C.byref(p), C.byref(st.data), 0)
    p.cycle, p.time, p.current_cycle_dt, p.next_cycle_dt = 0, 0.0, 0.0, 0.0
    L.o_update_axis(C.byref(p), 0)
    L.o_update_EOS(C.byref(p), C.byref(st.data))
    t0 = time.perf_counter()
    ref_steps = []
    for _ in range(cycles):
        assert L.o_solver_cycle(C.byref(p), C.byref(st.data)) == 0
        p.time += p.current_cycle_dt
        p.cycle += 1
        ref_steps.append((p.current_cycle_dt, p.next_cycle_dt, p.time))
    oracle_s = time.perf_counter() - t0
    ref = {k: O.real_cells(p, st[k]).copy() for k in PARITY_FIELDS}
    del st
    gcase = A.Case(**{**case.__dict__, "max_cycles": cycles})
    steps = []
    with A.Solver(gcase, precision=precision) as s:
        s.init_test()
        for _ in range(cycles):
            s.enqueue_cycles(1)
            q, status = s.state()
            assert status == 0
            steps.append((q.current_cycle_dt, q.next_cycle_dt, q.time))
        s.run()
        got = {k: A.real_cells(s.params, s.download(k)) for k in PARITY_FIELDS}
    dt_err = max(abs(a - b) / abs(b) for sa, sb in zip(steps, ref_steps) for a, b in zip(sa, sb))
    fields = {k: {"max_rel": max_rel(got[k], ref[k]), "l1_rel": l1_rel(got[k], ref[k]),
                  "bitwise_equal": bool(np.array_equal(got[k].view(np.int64), ref[k].view(np.int64)))}
              for k in PARITY_FIELDS}
    return {"cycles": cycles, "size": f"{case.nx}x{case.ny}", "fields": fields, "dt_time_max_rel": dt_err,
            "cycles_equal": len(steps) == len(ref_steps),
            "against": "the oracle (strict IEEE build of the project's C restatement, pinned bit for bit to the "
                       "reference's own code by tests/golden), cycle by cycle; tolerance 1e-10 relative on fields, "
                       "1e-12 on dt (the tests assert bit equality)",
            "oracle_seconds": oracle_s}


# ---------------------------------------------------------------- the single-domain path
def single_run(A, args, nx: int, prec: int, K: int, W: int, run_cycles: int, stream, world: int) -> dict:
    """One domain: the timed K cycles are the last of a `run_cycles` run (at least 80 cycles precede
    the W warm-up cycles; the first of them measure the tiling when this process has not).  Returns
    the timings and the solver."""
    import torch

    total = max(run_cycles, W + K + 80)
    case = A.Case(**{**WORKLOAD, "nx": nx, "ny": nx, "max_cycles": total})
    s = A.Solver(case, precision=prec, stream=stream.cuda_stream, cycles_per_graph=args.graph, seg_len=args.seg_len,
                 block_lines=args.block_lines, split_pass=args.split_pass, reuse=args.reuse)
    s.init_test()
    ev = [torch.cuda.Event(enable_timing=True) for _ in range(3)]
    torch.cuda.synchronize()
    s.enqueue_cycles(total - W - K)
    s.enqueue_cycles(W)
    torch.cuda.synchronize()
    tuning_left = s.tuning()
    if world > 1:
        torch.distributed.barrier()
    torch.cuda.synchronize()
    launches0 = s.kernel_launches
    measured0 = s.measurement_cycles()

    def timed():
        ev[1].record(stream)
        s.enqueue_cycles(K)
        ev[2].record(stream)
        if world > 1:
            torch.distributed.barrier()
        torch.cuda.synchronize()
        return ev[1].elapsed_time(ev[2])

    ms, clocks = sampled(timed)
    launches = s.kernel_launches - launches0
    measured_in_window = s.measurement_cycles() - measured0
    p, status = s.state()
    if status != 0 or p.cycle != total:
        raise RuntimeError(f"solver state after the timed region: status {status}, cycle {p.cycle}")
    tiling, blocks = s.tiling()
    return {"ms": ms, "total": total, "clocks": clocks, "launches": launches,
            "tiling": tiling, "blocks": blocks, "block_lines": s.block_lines(), "tuning_left": tuning_left,
            "measured_in_window": measured_in_window, "measurement_cycles": s.measurement_cycles(),
            "split": s.split_pass(), "solver": s}


def e2e_run(A, args, nx: int, prec: int, cycles: int, stream, ins: dict, outs: dict,
            cold: bool) -> tuple[float, int, float]:
    """The whole solve through the C ABI with host buffers: upload of rho, u, v, E from pinned
    memory, begin_loop, `cycles` cycles, download of rho, u, v, E, p into pinned memory (wall
    clock).  cold: the process forgets its measured tilings first, so the solve measures its own.
    Also returns the device time of its time loop (CUDA events around begin_loop and the cycles)."""
    import torch

    case = A.Case(**{**WORKLOAD, "nx": nx, "ny": nx, "max_cycles": cycles})
    se = A.Solver(case, precision=prec, stream=stream.cuda_stream, cycles_per_graph=args.graph,
                  seg_len=args.seg_len, block_lines=args.block_lines, split_pass=args.split_pass, reuse=args.reuse)
    se.init_test()
    L = A.lib()
    if cold:
        A.tiling_cache_clear()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for name in ("rho", "umat", "vmat", "Emat"):
        A.check(L.armon_solver_upload(se._h, A.ARRAYS.index(name), ins[name].data_ptr()))
    e0.record(stream)
    se.begin_loop()
    se.run()
    e1.record(stream)
    for name in ("rho", "umat", "vmat", "Emat", "pmat"):
        A.check(L.armon_solver_download(se._h, A.ARRAYS.index(name), outs[name].data_ptr()))
    torch.cuda.synchronize()
    secs = time.perf_counter() - t0
    pe, st_e = se.state()
    assert st_e == 0 and pe.cycle == cycles
    nb = se.params.nb_cells
    se.close()
    return secs, nb, e0.elapsed_time(e1)


def roofline(prec: int, cells: int, ms_per_cycle: float, split: bool) -> dict:
    peak, peak_kind = measured_peaks()
    t_pass = ms_per_cycle / 1e3 / 2
    bpc = BYTES_PER_CELL_UPDATE if prec == 64 else BYTES_PER_CELL_UPDATE // 2
    achieved = bpc / 2 * cells / t_pass / 1e9
    tname = "double" if prec == 64 else "float"
    kernel = ("armon::sweep_faces_kernel<%s,1,2,*> + armon::sweep_cells_kernel<%s,1,2,*> (one axis pass = a face "
              "launch and a cell launch)" % (tname, tname) if split else
              "armon::sweep_kernel<%s,1,2,*> (one launch = one axis pass)" % tname)
    key = ("split_" if split else "fused_") + "traffic_bytes_per_cell_per_pass"
    tr = profiled(key, prec)
    return {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
            "peak_source": peak_kind + " (MEASURED_PEAKS.json hbm_gbs, a STREAM-style copy)",
            "traffic": (tr * cells if tr else None), "traffic_bytes_per_cell_per_pass": tr,
            "kernel": kernel, "algorithmic_bytes_per_pass": bpc / 2 * cells,
            "per_unit": f"{bpc // 2} B per cell and axis pass (read and write rho, u, v, E once per cycle: "
                        f"{bpc} B per cell-update), over the mean axis-pass time of the timed cycles"}


def run_gpu(args) -> None:
    import torch

    import armon_gb300 as A

    rank, world, local = dist_info()
    torch.cuda.set_device(local)
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl", device_id=torch.device("cuda", local))
    nx = args.size
    K, W, prec = args.steps, args.warmup, args.precision
    run_cycles = args.run_cycles or (200 if prec == 64 else 100)
    # a dedicated stream: the solver launches on it and the CUDA events are recorded on it
    stream = torch.cuda.Stream()
    torch.cuda.set_stream(stream)
    r = single_run(A, args, nx, prec, K, W, run_cycles, stream, world)
    r.pop("solver").close()
    cells = nx * nx
    ms_max = max_over_ranks(r["ms"], world)
    value = whole_job_rate(cells * K, world, ms_max / 1e3)
    # end to end, from the run's initial state (init_test of a fresh solver) in pinned host memory,
    # the results into pinned buffers allocated and written once before, as those of an application
    # that reuses them
    with A.Solver(A.Case(**{**WORKLOAD, "nx": nx, "ny": nx, "max_cycles": 1}), precision=prec) as s0:
        s0.init_test()
        ins = {k: torch.from_numpy(s0.download(k)).pin_memory() for k in ("rho", "umat", "vmat", "Emat")}
        outs = {k: torch.empty(s0.params.nb_cells, dtype=torch.float64).pin_memory()
                for k in ("rho", "umat", "vmat", "Emat", "pmat")}
        for k, buf in outs.items():
            A.check(A.lib().armon_solver_download(s0._h, A.ARRAYS.index(k), buf.data_ptr()))
    e2e_s, nb, loop_ms = e2e_run(A, args, nx, prec, run_cycles, stream, ins, outs, cold=False)
    e2e_value = whole_job_rate(cells * run_cycles, world, max_over_ranks(e2e_s, world))
    whole = whole_job_rate(cells * run_cycles, world, max_over_ranks(loop_ms, world) / 1e3)
    cold_s, _, cold_loop_ms = e2e_run(A, args, nx, prec, run_cycles, stream, ins, outs, cold=True)
    cold_value = whole_job_rate(cells * run_cycles, world, max_over_ranks(cold_s, world))

    if rank == 0:
        out = {"metric": METRIC, "value": value, "unit": METRIC, "n_gpus": world, "steps": K, "warmup": W,
               "ms_per_step": ms_max / K, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
               "dtype": "f64" if prec == 64 else "f32", "data": "synthetic",
               "config": dict(config(nx, nx, world, prec, r["total"]), seg_len=list(r["tiling"]),
                              blocks=list(r["blocks"]), block_lines=r["block_lines"], split_pass=r["split"],
                              reuse=args.reuse == 0, timed_cycles=[r["total"] - K, r["total"]],
                              tiling_measured_before_timing=not r["tuning_left"],
                              tiling_measurement_cycles=r["measurement_cycles"],
                              tiling_measurement_cycles_timed=r["measured_in_window"]),
               "whole_run": {"value": whole, "unit": METRIC, "cycles": run_cycles,
                             "note": "every cycle of the whole run, from the initial state, on the device (CUDA events "
                                     "around begin_loop and the time loop of the e2e solve)"},
               "roofline": roofline(prec, cells, ms_max / K, r["split"]),
               "e2e": {"value": e2e_value, "unit": METRIC, "cycles": run_cycles,
                       "h2d_bytes_per_step": 4 * nb * 8 / run_cycles, "d2h_bytes_per_step": 5 * nb * 8 / run_cycles,
                       "seconds": e2e_s, "host_arrays": "FP64 (converted to the solver's precision inside the call)",
                       "path": f"armon_solver_upload x4 (pinned) + begin_loop + {run_cycles} cycles + "
                               "armon_solver_download x5 (into pinned buffers allocated and written once "
                               "before); tiling already measured in this process"},
               "e2e_cold": {"value": cold_value, "unit": METRIC, "seconds": cold_s, "cycles": run_cycles,
                            "loop_value": cells * run_cycles / (cold_loop_ms / 1e3),
                            "path": "the same after armon_tiling_cache_clear(): the solve measures its tiling on "
                                    "its own cycles"},
               "gpu_launches": r["launches"], "clocks": r["clocks"]}
        if world == 1 and args.parity_cycles > 0 and prec == 64:
            out["parity"] = parity(A, A.Case(**{**WORKLOAD, "nx": nx, "ny": nx}), min(args.parity_cycles, run_cycles))
        if world == 1 and not args.no_cpu and prec == 64:
            try:
                out["cpu_baseline"] = reference_cpu(nx, nx, args.cpu_cycles, 1)
            except Exception as e:
                out["cpu_baseline"] = dict(port_cpu(nx, nx, args.cpu_cycles), note=f"reference build unavailable ({e})")
            out["cpu_baseline_port"] = port_cpu(nx, nx, args.cpu_cycles)
        if world == 1 and prec == 32 and args.accuracy_cycles > 0:
            out["accuracy"] = fp32_accuracy(A, nx, args.accuracy_cycles, args.graph)
        if world == 1 and prec == 64 and not args.no_extra:
            out["fp32"] = fp32_line(A, args, stream)
            out["batch"] = batch_line(args, compact=True)
            out["serve"] = serve_line(args, compact=True)
        print(json.dumps(out), flush=True)
    if world > 1:
        torch.distributed.destroy_process_group()


# ---------------------------------------------------------------- configuration 5: the FP32 variant
def fp32_accuracy(A, nx: int, cycles: int, graph: int) -> dict:
    """The FP32 variant against the FP64 solve of the same workload and cycles (the FP64 solver
    equals the oracle bit for bit: tests/test_scale_parity_gpu.py): L1 relative error of rho and E,
    and the relative drift of the FP64 mass and energy sums over the run."""
    res = {}
    for prec in (64, 32):
        case = A.Case(**{**WORKLOAD, "nx": nx, "ny": nx, "max_cycles": cycles})
        with A.Solver(case, precision=prec, cycles_per_graph=graph) as s:
            s.init_test()
            m0, e0 = s.conservation()
            s.run()
            p, status = s.state()
            m1, e1 = s.conservation()
            res[prec] = ({k: A.real_cells(s.params, s.download(k)) for k in ("rho", "Emat")},
                         (m1 - m0) / m0, (e1 - e0) / e0, p.cycle, status)
    f64, f32 = res[64], res[32]
    return {"cycles": f32[3], "l1_rho": l1_rel(f32[0]["rho"], f64[0]["rho"]),
            "l1_E": l1_rel(f32[0]["Emat"], f64[0]["Emat"]),
            "mass_drift": {"f32": f32[1], "f64": f64[1]}, "energy_drift": {"f32": f32[2], "f64": f64[2]},
            "against": "the FP64 solve of the same workload and cycles (equal to the FP64 oracle bit for bit)"}


def fp32_line(A, args, stream) -> dict:
    """Configuration 5 compact: 8192^2 FP32, the last K cycles of a 100-cycle run timed, and the
    accuracy of the 100-cycle run against FP64."""
    nx, K, W = 8192, args.steps, args.warmup
    r = single_run(A, argparse.Namespace(**{**vars(args), "split_pass": 0}), nx, 32, K, W, 100, stream, 1)
    r.pop("solver").close()
    cells = nx * nx
    return {"value": cells * K / (r["ms"] / 1e3), "unit": METRIC, "ms_per_step": r["ms"] / K, "steps": K, "warmup": W,
            "config": dict(config(nx, nx, 1, 32, r["total"]), seg_len=list(r["tiling"]), block_lines=r["block_lines"],
                           split_pass=r["split"], timed_cycles=[r["total"] - K, r["total"]],
                           tiling_measurement_cycles=r["measurement_cycles"],
                           tiling_measurement_cycles_timed=r["measured_in_window"]),
            "roofline": roofline(32, cells, r["ms"] / K, r["split"]),
            "accuracy": fp32_accuracy(A, nx, 100, args.graph) if args.accuracy_cycles > 0 else None,
            "gpu_launches": r["launches"], "clocks": r["clocks"]}


# ---------------------------------------------------------------- configuration 3: batches
def plain_solve(A, spec, precision: int, graph: int, block_lines: int = 0, reuse: int = 0) -> tuple[float, int]:
    """One domain on the plain single-domain path (its own solver: init, upload of the initial
    fields, time loop); returns the seconds of its time loop and its cell-updates."""
    import torch

    with A.Solver(spec.params(), precision=precision, cycles_per_graph=graph, block_lines=block_lines,
                  reuse=reuse) as s:
        s.init_test()
        for k, a in spec.initial_state().items():
            s.upload(k, a)
        s.begin_loop()
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        s.run()
        secs = time.perf_counter() - t0
        p, st = s.state()
        assert st == 0
        return secs, spec.nx * spec.ny * p.cycle


def stratified(items: list, key, n: int) -> list:
    """n items spread evenly over the list sorted by key (one from each of n equal slices)."""
    if n >= len(items):
        return list(items)
    srt = sorted(items, key=key)
    step = len(srt) / n
    return [srt[int(i * step + step / 2)] for i in range(n)]


def batch_line(args, compact: bool) -> dict:
    """Configuration 3: 256 uneven domains (seeded), FP64, each to t = 0.15, all in one batch (one
    launch per pass half over every domain, CUDA graphs), against the plain single-domain path (one
    solver per domain, one after another) on the same domains, or on a stratified sample of them."""
    import torch

    import armon_gb300 as A
    from armon_gb300 import workloads as W

    specs = W.mixed_domains(args.domains, seed=2024)
    torch.cuda.set_device(0)
    n_plain = args.plain_domains or (32 if compact else len(specs))
    sample = stratified(specs, lambda sp: sp.nx * sp.ny, n_plain)
    plain_solve(A, sample[0], 64, args.graph, args.block_lines, args.reuse)   # warm-up
    plain_secs, plain_work = 0.0, 0
    for sp in sample:
        s_, w_ = plain_solve(A, sp, 64, args.graph, args.block_lines, args.reuse)
        plain_secs += s_
        plain_work += w_
    with A.Batch(precision=64, cycles_per_graph=8, block_lines=args.block_lines or 128, reuse=args.reuse,
                 split_pass=args.split_pass) as b:
        ids = [b.add_sod(sp.params(), sp.sod_interface()) for sp in specs]
        b.poll()
        launches0 = b.kernel_launches

        def go():
            t0 = time.perf_counter()
            assert b.run() == 0
            return time.perf_counter() - t0

        secs, clocks = sampled(go)
        launches = b.kernel_launches - launches0
        waves, _ = b.schedule()
        work = 0
        for i, sp in zip(ids, specs):
            p, st = b.state(i)
            assert st == 0
            work += sp.nx * sp.ny * p.cycle
    value = work / secs
    plain_value = plain_work / plain_secs
    return {"metric": METRIC, "value": value, "unit": METRIC, "seconds": secs, "dtype": "f64",
            "config": {"workload": f"{len(specs)} uneven Sod-interface domains (seed 2024), sides in {{64..1024}}, "
                                   "GAD-minmod + euler_2nd, CFL 0.6, each to t = 0.15",
                       "domains": len(specs), "cells": sum(sp.nx * sp.ny for sp in specs), "cell_updates": work,
                       "step": "the whole batch run to completion (one launch per pass half over every domain, "
                               "8-cycle CUDA graphs)"},
            "plain": {"value": plain_value, "seconds": plain_secs, "domains": len(sample),
                      "sample": ("a stratified sample by domain size (one domain from each of %d equal slices of the "
                                 "%d sorted by cells)" % (len(sample), len(specs))) if len(sample) < len(specs) else "all",
                      "path": "one Solver per domain, one after another (time loops only)"},
            "batched_over_plain": value / plain_value,
            "schedule": {"waves": waves, "how": "autotuned online (CUDA-event timing of one graph batch per candidate)"},
            "gpu_launches": launches, "clocks": clocks}


# ---------------------------------------------------------------- configuration 4: serving
def serve_line(args, compact: bool) -> dict:
    """Configuration 4: Poisson arrivals of Sod-interface solves (side lognormal(6, 0.6) clipped to
    [128, 2048], FP64 or FP32 with p = 1/2, t_end ~ U(0.05, 0.2)) replayed in real time through the
    server with a 150 GB state budget; p50/p99 time-to-solution and cell-updates/s, against the plain
    path on a stratified sample of the same requests."""
    import torch

    import armon_gb300 as A
    from armon_gb300 import serving as S
    from armon_gb300 import workloads as W

    n = args.serve_requests_compact if compact else args.requests
    trace = W.serving_trace(n=n, rate=args.rate, seed=7)
    torch.cuda.set_device(0)
    with A.Server(cycles_per_step=args.serve_cycles) as srv:      # warm-up: the kernels of both precisions
        S.replay(srv, W.serving_trace(n=4, rate=1000.0, seed=1, side_range=(128, 128)))
    with A.Server(memory_budget=150_000_000_000, cycles_per_step=args.serve_cycles,
                  max_inflight_cells=args.max_inflight, waves=args.serve_waves) as srv:
        (served, wall), clocks = sampled(lambda: S.replay(srv, trace))
        launches = srv.kernel_launches
    assert all(r.status == A.REQ_DONE for r in served)
    work = sum(r.cells * r.cycles for r in served)
    tts = [r.tts for r in served]
    by_prec = {}
    for prec in (64, 32):
        t = [r.tts for r in served if r.precision == prec]
        by_prec[str(prec)] = {"requests": len(t), "tts_p50_s": S.percentile(t, 0.5), "tts_p99_s": S.percentile(t, 0.99)}
    sample = stratified(trace, lambda r: r.spec.nx * r.spec.ny, min(args.plain_sample, len(trace)))
    p_secs, p_work = 0.0, 0
    for r in sample:
        s_, w_ = plain_solve(A, r.spec, r.spec.precision, args.graph, reuse=args.reuse)
        p_secs += s_
        p_work += w_
    value = work / wall
    return {"metric": METRIC, "value": value, "unit": METRIC, "seconds": wall, "dtype": "f64+f32",
            "config": {"workload": f"{len(trace)} requests, Poisson arrivals at {args.rate}/s (seed 7), side "
                                   "lognormal(6, 0.6) clipped to [128, 2048], FP64 or FP32 (p = 1/2), "
                                   "t_end ~ U(0.05, 0.2), 150 GB state budget",
                       "requests": len(trace), "cycles_per_round": args.serve_cycles, "cell_updates": work,
                       "max_inflight_cells": args.max_inflight},
            "tts_p50_s": S.percentile(tts, 0.5), "tts_p99_s": S.percentile(tts, 0.99), "by_precision": by_prec,
            "plain": {"value": p_work / p_secs, "seconds": p_secs, "requests": len(sample),
                      "sample": "a stratified sample of the same requests by size (one from each of n equal slices "
                                "sorted by cells)",
                      "path": "one Solver per request, one after another (time loops only)"},
            "served_over_plain": value / (p_work / p_secs),
            "gpu_launches": launches, "clocks": clocks}


def run_batch(args) -> None:
    out = batch_line(args, compact=False)
    out.update({"n_gpus": 1, "steps": 1, "warmup": 1, "ms_per_step": out["seconds"] * 1e3, "higher_is_better": True,
                "scaling": "weak", "vs_baseline": None, "data": "synthetic"})
    print(json.dumps(out), flush=True)


def run_serve(args) -> None:
    out = serve_line(args, compact=False)
    out.update({"n_gpus": 1, "steps": 1, "warmup": 1, "ms_per_step": out["seconds"] * 1e3, "higher_is_better": True,
                "scaling": "weak", "vs_baseline": None, "data": "synthetic"})
    print(json.dumps(out), flush=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--size", type=int, default=0, help="cells per side (default 4096; 8192 for --precision 32)")
    ap.add_argument("--precision", type=int, default=64, choices=[64, 32])
    ap.add_argument("--run-cycles", type=int, default=0,
                    help="cycles of the run whose last --steps cycles are timed (default 200; 100 for --precision 32)")
    ap.add_argument("--graph", type=int, default=16, help="cycles per CUDA graph")
    ap.add_argument("--seg-len", type=int, default=0, help="cells per thread along the sweep axis (0 = automatic)")
    ap.add_argument("--block-lines", type=int, default=0, help="threads (lines) per block of the axis pass (0 = automatic)")
    ap.add_argument("--split-pass", type=int, default=0, choices=[-1, 0, 1],
                    help="1: each axis pass as a face launch and a cell launch; -1: one fused launch; "
                         "0: the solver's default (measured)")
    ap.add_argument("--reuse", type=int, default=0, choices=[-1, 0],
                    help="0: positions whose input window repeats the previous one reuse its results (exact); "
                         "-1: every position computed")
    ap.add_argument("--parity-cycles", type=int, default=200, help="cycles compared with the oracle (0 = skip)")
    ap.add_argument("--cpu-cycles", type=int, default=10, help="cycles of the CPU baseline sample")
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--no-extra", action="store_true", help="skip the compact fp32 / batch / serve runs")
    ap.add_argument("--accuracy-cycles", type=int, default=100, help="FP32 accuracy run's cycles (0 = skip)")
    ap.add_argument("--workload", default="single", choices=["single", "batch", "serve"],
                    help="single: the 4096^2 drop-in case (default); batch: 256 mixed domains; serve: a request trace")
    ap.add_argument("--domains", type=int, default=256, help="batch: domains")
    ap.add_argument("--plain-domains", type=int, default=0,
                    help="batch: domains timed on the plain path, a stratified sample (0 = 32 in the default line, "
                         "all with --workload batch)")
    ap.add_argument("--requests", type=int, default=10000, help="--workload serve: requests of the trace")
    ap.add_argument("--serve-requests-compact", type=int, default=600, help="serve in the default line: requests")
    ap.add_argument("--rate", type=float, default=50.0,
                    help="serve: arrivals per second (50 offers more than one GB300 serves, so the served rate "
                         "is the server's capacity)")
    ap.add_argument("--serve-cycles", type=int, default=8, help="serve: cycles per round")
    ap.add_argument("--serve-waves", type=int, default=0,
                    help="serve: block waves the batches' schedules aim for (0 = autotuned)")
    ap.add_argument("--plain-sample", type=int, default=40, help="serve: requests timed on the plain path")
    ap.add_argument("--max-inflight", type=int, default=None,
                    help="serve: real cells running at once per batch (0 = no limit; default: the server's)")
    args = ap.parse_args()
    if args.warmup < 3:
        args.warmup = 3
    if args.size <= 0:
        args.size = 4096 if args.precision == 64 else 8192
    if args.impl == "reference":
        run_reference(args)
    elif args.workload == "batch":
        run_batch(args)
    elif args.workload == "serve":
        run_serve(args)
    else:
        run_gpu(args)


if __name__ == "__main__":
    main()
