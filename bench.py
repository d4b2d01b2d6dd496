#!/usr/bin/env python
"""Benchmark of the Armon time step on GB300: cell-updates/s of the fused FP64 solver.

Workload (the single-domain drop-in case): circular Sod on [0,1]^2, 4096 x 4096 real cells, 5 ghost
layers, FP64, gamma 1.4, rho/p = 1/1 inside radius 0.2 and 0.125/0.1 outside, GAD acoustic fluxes
with the minmod limiter, second-order Euler remap, Sequential X/Y splitting, CFL 0.6.  A step is one
solver cycle (dt reduction + X pass + Y pass) over the whole grid; the state (4 x 135 MB per buffer
set) is larger than L2, so no flush is needed between steps.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl gb300|reference]

--impl reference times the reference's CPU path (the oracle's OpenMP build with the reference's
Release flags) on the host cores.  N > 1 runs N independent replicas (one per GPU), weak scaling.
Prints one JSON line (rank 0).
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


def config(nx: int, ny: int, n: int, precision: int = 64) -> dict:
    prec = "FP64" if precision == 64 else "FP32 storage and arithmetic, FP64 dt and conservation sums"
    esize = 8 if precision == 64 else 4
    return {"workload": f"Sod_circ {nx}x{ny} {prec}, GAD-minmod + euler_2nd, CFL 0.6, radius 0.2, Sequential splitting",
            "nx": nx, "ny": ny, "nghost": 5, "gamma": 1.4, "scheme": "GAD", "limiter": "Minmod",
            "projection": "euler_2nd", "splitting": "Sequential", "cfl": 0.6, "radius": 0.2,
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


def profiled_traffic(precision: int = 64, prefix: str = "") -> float | None:
    """DRAM bytes per cell and axis pass (scaled to the workload by the caller); prefix "fused_" /
    "split_" selects the figure of the pass form that is not the precision's default."""
    return profiled(prefix + "traffic_bytes_per_cell_per_pass", precision)


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
        rows = []
        for ln in self.lines:
            parts = [x.strip() for x in ln.split(",")]
            if len(parts) >= 9:
                try:
                    rows.append(parts)
                except Exception:
                    pass
        if not rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["no samples"]}
        # the busiest GPU (highest power) is ours
        by_gpu: dict[str, list] = {}
        for r in rows:
            by_gpu.setdefault(r[0], []).append(r)
        gpu = max(by_gpu, key=lambda g: statistics.median(float(r[3]) for r in by_gpu[g] if r[3] not in ("", "[N/A]")))
        rs = by_gpu[gpu]
        sm = [float(r[1]) for r in rs]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[k] for r in rs for k in range(4) if r[5 + k].lower() == "active"})
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": float(rs[0][2]), "reasons": reasons,
                "samples": len(rs), "power_w_median": statistics.median(float(r[3]) for r in rs)}


def fp64_roofline(cells: int, s_per_cycle: float, clocks: dict | None, prefix: str = "") -> dict | None:
    """The FP64 pipe as the bound: FP64 operations per cell and axis pass (ncu's DADD + DMUL + DFMA
    counts, profiles/) over the pipe's peak, 2 per SM per cycle (ncu's peak_sustained) at the SM
    clock sampled during the timed region."""
    import torch

    ops = profiled(prefix + "fp64_ops_per_cell_per_pass")
    if not ops:
        return None
    sms = torch.cuda.get_device_properties(0).multi_processor_count
    mhz = (clocks or {}).get("sm_mhz") or 2070.0
    peak = 2.0 * sms * mhz * 1e6
    achieved = ops * cells * 2 / s_per_cycle
    return {"bound": "fp64", "achieved": achieved / 1e9, "peak": peak / 1e9, "unit": "G FP64 op/s",
            "frac": achieved / peak, "ops_per_cell_per_pass": ops,
            "note": "divisions, square roots and compares run on the integer pipes (exact), so only "
                    "additions and multiplications count here"}


def l1_rel(a, b) -> float:
    """sum |a - b| / sum |b| (b the FP64 result)."""
    import numpy as np

    return float(np.abs(a - b).sum() / np.abs(b).sum())


def fp32_accuracy(A, case, graph: int) -> dict:
    """The FP32 variant against the FP64 solve of the same case and cycles (the FP64 solver is
    bit-identical to the FP64 oracle): L1 relative error of rho and E, and the relative drift of the
    mass and energy sums (FP64 sums in both) over the run."""
    res = {}
    for prec in (64, 32):
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
            "against": "the FP64 solve of the same workload and cycles (bit-identical to the FP64 oracle)"}


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


def cpu_port_throughput(nx: int, ny: int, budget_s: float, max_cycles: int) -> dict:
    """The oracle's OpenMP build with the reference's Release flags, on the host cores."""
    import oracle_lib as O

    L = O.lib(fast=True)
    case = O.Case(**{k: v for k, v in WORKLOAD.items()})
    case.nx, case.ny = nx, ny
    p = O.make_params(case, L)
    st = O.OracleState(p)
    L.o_init_test_p(C.byref(p), C.byref(st.data), 0)
    p.cycle, p.time, p.current_cycle_dt, p.next_cycle_dt = 0, 0.0, 0.0, 0.0
    L.o_update_axis(C.byref(p), 0)
    L.o_update_EOS(C.byref(p), C.byref(st.data))
    t0 = time.perf_counter()
    n = 0
    while n < max_cycles:
        if L.o_solver_cycle(C.byref(p), C.byref(st.data)) != 0:
            break
        p.time += p.current_cycle_dt
        p.cycle += 1
        n += 1
        if time.perf_counter() - t0 >= budget_s:
            break
    secs = time.perf_counter() - t0
    return {"value": nx * ny * n / secs, "unit": METRIC, "cores": L.o_num_threads(), "kind": "port",
            "sample": f"{n} cycles of the {nx}x{ny} workload after init (oracle/armon_oracle.c, -O3 -ffast-math, OpenMP)",
            "seconds": secs, "cycles": n}


def run_reference(args) -> None:
    rank, world, _ = dist_info()
    if rank != 0:
        return
    nx = ny = args.size
    os.environ.setdefault("OMP_PROC_BIND", "close")
    os.environ.setdefault("OMP_PLACES", "cores")
    # W untimed cycles are included in the same run as warm-up of caches and page faults
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

    def cycle():
        assert L.o_solver_cycle(C.byref(p), C.byref(st.data)) == 0
        p.time += p.current_cycle_dt
        p.cycle += 1

    for _ in range(args.warmup):
        cycle()
    t0 = time.perf_counter()
    for _ in range(args.steps):
        cycle()
    secs = time.perf_counter() - t0
    value = nx * ny * args.steps / secs
    out = {"metric": METRIC, "value": value, "unit": METRIC, "impl": "reference", "n_gpus": args.gpus,
           "steps": args.steps, "warmup": args.warmup, "ms_per_step": secs * 1e3 / args.steps,
           "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
           "config": config(nx, ny, 1),
           "cpu_baseline": {"value": value, "unit": METRIC, "cores": L.o_num_threads(), "kind": "port",
                            "sample": f"{args.steps} timed cycles of the {nx}x{ny} workload on the host cores "
                                      "(oracle/armon_oracle.c: the reference's unfused stage sequence, OpenMP, "
                                      "-O3 -funroll-loops -ffast-math)"},
           "e2e": {"value": value, "unit": METRIC, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(out), flush=True)


def run_gpu(args) -> None:
    import numpy as np
    import torch

    import armon_gb300 as A

    rank, world, local = dist_info()
    torch.cuda.set_device(local)
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl", device_id=torch.device("cuda", local))
    nx = ny = args.size
    K, W = args.steps, args.warmup
    case = A.Case(**WORKLOAD)
    case.nx, case.ny = nx, ny
    case.max_cycles = W + K
    prec = args.precision
    # a dedicated stream: the solver launches on it and the CUDA events are recorded on it
    stream = torch.cuda.Stream()
    torch.cuda.set_stream(stream)
    s = A.Solver(case, precision=prec, stream=stream.cuda_stream, cycles_per_graph=args.graph, seg_len=args.seg_len,
                 block_lines=args.block_lines, split_pass=args.split_pass, reuse=args.reuse)
    s.init_test()
    s.enqueue_cycles(W)
    torch.cuda.synchronize()

    def barrier():
        if world > 1:
            torch.distributed.barrier()
        torch.cuda.synchronize()

    barrier()
    launches0 = s.kernel_launches
    tiling = s.tiling()
    block_lines = s.block_lines()
    sampler = ClockSampler() if rank == 0 else None
    if sampler:
        sampler.start()
        time.sleep(0.25)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    s.enqueue_cycles(K)
    e1.record(stream)
    barrier()
    clocks = sampler.stop() if sampler else None
    ms = e0.elapsed_time(e1)
    launches = s.kernel_launches - launches0
    p, status = s.state()
    if status != 0 or p.cycle != W + K:
        raise RuntimeError(f"solver state after the timed region: status {status}, cycle {p.cycle}")
    ms_max = max_over_ranks(ms, world)
    cells = nx * ny
    value = whole_job_rate(cells * K, world, ms_max / 1e3)

    # end to end through the C ABI with host buffers: H2D of the initial fields from pinned memory,
    # the time loop, D2H of rho, u, v, E, p (every step of it inside the timed region)
    ins = {k: torch.from_numpy(s.download(k)).pin_memory() for k in ("rho", "umat", "vmat", "Emat")}
    s.close()
    case_e2e = A.Case(**WORKLOAD)
    case_e2e.nx, case_e2e.ny = nx, ny
    case_e2e.max_cycles = K
    se = A.Solver(case_e2e, precision=prec, stream=stream.cuda_stream, cycles_per_graph=args.graph,
                  seg_len=args.seg_len, block_lines=args.block_lines, split_pass=args.split_pass, reuse=args.reuse)
    se.init_test()
    outs = {k: torch.empty(se.params.nb_cells, dtype=torch.float64).pin_memory()
            for k in ("rho", "umat", "vmat", "Emat", "pmat")}
    L = A.lib()
    barrier()
    t0 = time.perf_counter()
    for k, name in enumerate(("rho", "umat", "vmat", "Emat")):
        A.check(L.armon_solver_upload(se._h, A.ARRAYS.index(name), ins[name].data_ptr()))
    se.begin_loop()
    se.run()
    for name in ("rho", "umat", "vmat", "Emat", "pmat"):
        A.check(L.armon_solver_download(se._h, A.ARRAYS.index(name), outs[name].data_ptr()))
    barrier()
    e2e_s = time.perf_counter() - t0
    pe, st_e = se.state()
    assert st_e == 0 and pe.cycle == K
    se.close()
    nb = se.params.nb_cells if hasattr(se, "params") else (nx + 10) * (ny + 10)
    e2e_value = whole_job_rate(cells * K, world, max_over_ranks(e2e_s, world))

    if rank == 0:
        peak, peak_kind = measured_peaks()
        t_launch = ms_max / 1e3 / (K * 2)
        bpc = BYTES_PER_CELL_UPDATE if prec == 64 else BYTES_PER_CELL_UPDATE // 2
        achieved = bpc / 2 * cells / t_launch / 1e9
        split = args.split_pass == 1 or (args.split_pass == 0 and prec == 64)
        prefix = "" if split == (prec == 64) else ("fused_" if prec == 64 else "split_")
        tr = profiled_traffic(prec, prefix)
        tname = "double" if prec == 64 else "float"
        kernel = ("armon::sweep_faces_kernel<%s,1,*> + armon::sweep_cells_kernel<%s,1,2,*> (one axis pass = a face "
                  "launch and a cell launch)" % (tname, tname) if split else
                  "armon::sweep_kernel<%s,1,2,*> (one launch = one axis pass)" % tname)
        out = {"metric": METRIC, "value": value, "unit": METRIC, "n_gpus": world, "steps": K, "warmup": W,
               "ms_per_step": ms_max / K, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
               "dtype": "f64" if prec == 64 else "f32", "data": "synthetic",
               "config": dict(config(nx, ny, world, prec), seg_len=list(tiling[0]), blocks=list(tiling[1]),
                             block_lines=block_lines),
               "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                            "frac": achieved / peak, "peak_source": peak_kind,
                            "traffic": (tr * cells if tr else None),
                            "kernel": kernel,
                            "algorithmic_bytes_per_pass": bpc / 2 * cells,
                            "note": ("not HBM-bound: the FP64 pipe and integer latency bound the pass (fp64_roofline, profiles/)"
                                     if prec == 64 else
                                     "not HBM-bound: instruction latency bounds the pass (12 warps per SM; profiles/)")},
               "fp64_roofline": fp64_roofline(cells, ms_max / 1e3 / K, clocks, prefix) if prec == 64 else None,
               "e2e": {"value": e2e_value, "unit": METRIC, "h2d_bytes_per_step": 4 * nb * 8 / K,
                       "d2h_bytes_per_step": 5 * nb * 8 / K, "seconds": e2e_s,
                       "host_arrays": "FP64 (converted to the solver's precision inside the call)",
                       "path": "armon_solver_upload x4 (pinned) + begin_loop + run + armon_solver_download x5"},
               "gpu_launches": launches, "clocks": clocks}
        if world == 1 and not args.no_cpu and prec == 64:
            out["cpu_baseline"] = cpu_port_throughput(nx, ny, args.cpu_seconds, 200)
        if world == 1 and prec == 32 and args.accuracy_cycles > 0:
            acc_case = A.Case(**WORKLOAD)
            acc_case.nx, acc_case.ny = nx, ny
            acc_case.max_cycles = args.accuracy_cycles
            out["accuracy"] = fp32_accuracy(A, acc_case, args.graph)
        print(json.dumps(out), flush=True)
    if world > 1:
        torch.distributed.destroy_process_group()


def plain_solve(A, spec, precision: int, graph: int, block_lines: int = 0) -> tuple[float, int]:
    """One domain on the plain single-domain path (its own solver: init, upload of the initial
    fields, time loop); returns the seconds of its time loop and its cell-updates."""
    import torch

    with A.Solver(spec.params(), precision=precision, cycles_per_graph=graph, block_lines=block_lines) as s:
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


def run_batch(args) -> None:
    """Configuration 3: 256 uneven domains (seeded), FP64, each to t = 0.15 -- all of them in one
    batch (one fused launch per pass, CUDA graphs) against the same domains one after another on the
    plain single-domain path."""
    import torch

    import armon_gb300 as A
    from armon_gb300 import workloads as W

    specs = W.mixed_domains(args.domains, seed=2024)
    torch.cuda.set_device(0)
    # plain path (domains one at a time; the first is a warm-up)
    plain_secs, plain_work = 0.0, 0
    plain_solve(A, specs[0], 64, args.graph, args.block_lines)
    for sp in specs:
        s_, w_ = plain_solve(A, sp, 64, args.graph, args.block_lines)
        plain_secs += s_
        plain_work += w_
    # batched
    with A.Batch(precision=64, cycles_per_graph=8, block_lines=args.block_lines or 128) as b:
        ids = [b.add_sod(sp.params(), sp.sod_interface()) for sp in specs]
        b.poll()
        launches0 = b.kernel_launches
        sampler = ClockSampler()
        sampler.start()
        t0 = time.perf_counter()
        assert b.run() == 0
        secs = time.perf_counter() - t0
        clocks = sampler.stop()
        launches = b.kernel_launches - launches0
        waves, _ = b.schedule()
        work = 0
        for i, sp in zip(ids, specs):
            p, st = b.state(i)
            assert st == 0
            work += sp.nx * sp.ny * p.cycle
    assert work == plain_work
    value = work / secs
    cells = sum(sp.nx * sp.ny for sp in specs)
    out = {"metric": METRIC, "value": value, "unit": METRIC, "n_gpus": 1, "steps": 1, "warmup": 1,
           "ms_per_step": secs * 1e3, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
           "dtype": "f64", "data": "synthetic",
           "config": {"workload": f"{len(specs)} uneven Sod-interface domains (seed 2024), sides in "
                                  "{64..1024}, GAD-minmod + euler_2nd, CFL 0.6, each to t = 0.15",
                      "domains": len(specs), "cells": cells, "cell_updates": work,
                      "step": "the whole batch run to completion (one fused launch per pass, 8-cycle CUDA graphs)"},
           "plain": {"value": plain_work / plain_secs, "seconds": plain_secs,
                     "path": "one Solver per domain, one after another (time loops only)"},
           "batched_over_plain": value / (plain_work / plain_secs),
           "schedule": {"waves": waves, "how": "autotuned online (CUDA-event timing of one graph batch per candidate)"},
           "gpu_launches": launches, "clocks": clocks}
    print(json.dumps(out), flush=True)


def run_serve(args) -> None:
    """Configuration 4: Poisson arrivals of Sod-interface solves (side lognormal(6, 0.6) clipped to
    [128, 2048], FP64 or FP32 with p = 1/2, t_end ~ U(0.05, 0.2)) replayed in real time through the
    server with a 150 GB state budget; p50/p99 time-to-solution and cell-updates/s."""
    import torch

    import armon_gb300 as A
    from armon_gb300 import serving as S
    from armon_gb300 import workloads as W

    trace = W.serving_trace(n=args.requests, rate=args.rate, seed=7)
    torch.cuda.set_device(0)
    # warm-up: the kernels of both precisions
    with A.Server(cycles_per_step=args.serve_cycles) as srv:
        S.replay(srv, W.serving_trace(n=4, rate=1000.0, seed=1, side_range=(128, 128)))
    with A.Server(memory_budget=150_000_000_000, cycles_per_step=args.serve_cycles,
                  max_inflight_cells=args.max_inflight, waves=args.serve_waves) as srv:
        sampler = ClockSampler()
        sampler.start()
        served, wall = S.replay(srv, trace)
        clocks = sampler.stop()
        launches = srv.kernel_launches
    assert all(r.status == A.REQ_DONE for r in served)
    work = sum(r.cells * r.cycles for r in served)
    tts = [r.tts for r in served]
    by_prec = {}
    for prec in (64, 32):
        t = [r.tts for r in served if r.precision == prec]
        by_prec[str(prec)] = {"requests": len(t), "tts_p50_s": S.percentile(t, 0.5), "tts_p99_s": S.percentile(t, 0.99)}
    # the plain path on a sample of the same requests, one solve at a time
    sample = trace[:args.plain_sample]
    p_secs, p_work = 0.0, 0
    for r in sample:
        s_, w_ = plain_solve(A, r.spec, r.spec.precision, args.graph)
        p_secs += s_
        p_work += w_
    # FP32 requests against the same solve in FP64 (served results equal solo ones bit for bit)
    l1 = []
    for r in [r for r in trace if r.spec.precision == 32][:args.accuracy_sample]:
        fields = {}
        for prec in (64, 32):
            with A.Solver(r.spec.params(), precision=prec) as s:
                s.init_test()
                for k, a in r.spec.initial_state().items():
                    s.upload(k, a)
                s.begin_loop()
                s.run()
                fields[prec] = {k: A.real_cells(s.params, s.download(k)) for k in ("rho", "Emat")}
        l1.append((l1_rel(fields[32]["rho"], fields[64]["rho"]), l1_rel(fields[32]["Emat"], fields[64]["Emat"])))
    value = work / wall
    out = {"metric": METRIC, "value": value, "unit": METRIC, "n_gpus": 1, "steps": 1, "warmup": 1,
           "ms_per_step": wall * 1e3, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
           "dtype": "f64+f32", "data": "synthetic",
           "fp32_accuracy": {"requests": len(l1), "l1_rho_max": max((a for a, _ in l1), default=None),
                             "l1_E_max": max((b for _, b in l1), default=None),
                             "against": "each request solved alone in FP64 (to its own t_end; cycle counts may differ)"},
           "config": {"workload": f"{len(trace)} requests, Poisson arrivals at {args.rate}/s (seed 7), side "
                                  "lognormal(6, 0.6) clipped to [128, 2048], FP64 or FP32 (p = 1/2), t_end ~ U(0.05, 0.2), "
                                  "150 GB state budget",
                      "requests": len(trace), "cycles_per_round": args.serve_cycles, "cell_updates": work,
                      "max_inflight_cells": args.max_inflight},
           "tts_p50_s": S.percentile(tts, 0.5), "tts_p99_s": S.percentile(tts, 0.99), "by_precision": by_prec,
           "plain": ({"value": p_work / p_secs, "seconds": p_secs, "sample": f"the first {len(sample)} requests",
                      "path": "one Solver per request, one after another (time loops only)"} if sample else None),
           "served_over_plain": value / (p_work / p_secs) if sample else None,
           "gpu_launches": launches, "clocks": clocks}
    print(json.dumps(out), flush=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--size", type=int, default=0, help="cells per side (default 4096; 8192 for --precision 32)")
    ap.add_argument("--precision", type=int, default=64, choices=[64, 32])
    ap.add_argument("--graph", type=int, default=16, help="cycles per CUDA graph")
    ap.add_argument("--seg-len", type=int, default=0, help="cells per thread along the sweep axis (0 = automatic)")
    ap.add_argument("--block-lines", type=int, default=0, help="threads (lines) per block of the axis pass (0 = automatic)")
    ap.add_argument("--split-pass", type=int, default=0, choices=[-1, 0, 1],
                    help="1: each axis pass as a face launch and a cell launch; -1: one fused launch; "
                         "0: the solver's default (split in FP64)")
    ap.add_argument("--reuse", type=int, default=0, choices=[-1, 0],
                    help="0: positions whose input window repeats the previous one reuse its results (exact); "
                         "-1: every position computed")
    ap.add_argument("--cpu-seconds", type=float, default=12.0)
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--accuracy-cycles", type=int, default=100,
                    help="--precision 32: cycles of the FP32-vs-FP64 accuracy run (0 = skip)")
    ap.add_argument("--workload", default="single", choices=["single", "batch", "serve"],
                    help="single: the 4096^2 drop-in case (default); batch: 256 mixed domains; serve: a request trace")
    ap.add_argument("--domains", type=int, default=256, help="--workload batch: domains")
    ap.add_argument("--requests", type=int, default=2000, help="--workload serve: requests of the trace")
    ap.add_argument("--rate", type=float, default=50.0, help="--workload serve: arrivals per second")
    ap.add_argument("--serve-cycles", type=int, default=8, help="--workload serve: cycles per round")
    ap.add_argument("--serve-waves", type=int, default=0,
                    help="--workload serve: block waves the batches' schedules aim for (0 = autotuned)")
    ap.add_argument("--plain-sample", type=int, default=100, help="--workload serve: requests timed on the plain path")
    ap.add_argument("--accuracy-sample", type=int, default=5, help="--workload serve: FP32 requests checked against FP64")
    ap.add_argument("--max-inflight", type=int, default=None,
                    help="--workload serve: real cells running at once per batch (0 = no limit; default: the server's)")
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
