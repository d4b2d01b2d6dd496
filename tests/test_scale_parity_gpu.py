"""Parity at the benchmark configurations, against the strict oracle.

* Circular Sod at 4096 x 4096 (radius 0.2, GAD-minmod, second-order remap, CFL 0.6, FP64) run the way
  the benchmark runs it: default options, so the tiling and pass form are measured on the loop's
  own cycles, units are dispatched longest first and runs of identical inputs reuse their results.  Every cycle's dt and time equal the oracle's as doubles and the final rho, u, v, E, p, c
  hash the same, for a cycle-by-cycle run and for a run in CUDA-graph batches.  The same at 2048^2
  over 120 cycles, where the fronts have moved some 60 cells.
* The FP32 variant at 8192 x 8192 against the FP64 oracle: L1 relative error of rho and E, and the
  drift of the FP64 mass and energy sums.
* A seeded sample of the 256-domain mix (sides 64..1024, planar and circular Sod interfaces, each to
  t = 0.15), including its largest domains, run together in one batch: each equals the oracle.

The tolerances are those of the reference's comparison (tests/armon_2D_tests.cpp:278-346 compares
every field and the final dt; src/io.h:14-17): here every FP64 field and dt bit for bit, and the
FP32 variant within 1e-5 L1.
"""
import ctypes as C
import hashlib

import numpy as np
import pytest

import armon_gb300 as A
import oracle_lib as O
from armon_gb300 import workloads as W

pytestmark = pytest.mark.gpu

FIELDS = ("rho", "umat", "vmat", "Emat", "pmat", "cmat")


def sha(a):
    return hashlib.sha256(np.ascontiguousarray(a).tobytes()).hexdigest()


def sod_circ(n, cycles):
    return A.Case(test="Sod_circ", scheme="GAD", projection="euler_2nd", limiter="Minmod", splitting="Sequential",
                  nghost=5, nx=n, ny=n, cfl=0.6, max_cycles=cycles, max_time=1e9, test_option=0.04)


def oracle_cycles(case):
    """The oracle's time loop, one solver_cycle at a time (src/armon_2D.cpp:327-386): per cycle
    (current dt, next dt, time), and the final state."""
    L = O.lib()
    p = O.make_params(O.Case(**case.__dict__), L)
    st = O.OracleState(p)
    L.o_init_test_p(C.byref(p), C.byref(st.data), 0)
    p.cycle, p.time, p.current_cycle_dt, p.next_cycle_dt = 0, 0.0, 0.0, 0.0
    L.o_update_axis(C.byref(p), 0)
    L.o_update_EOS(C.byref(p), C.byref(st.data))
    steps = []
    while p.time < p.max_time and p.cycle < p.max_cycles:
        assert L.o_solver_cycle(C.byref(p), C.byref(st.data)) == 0
        p.time += p.current_cycle_dt
        p.cycle += 1
        steps.append((p.current_cycle_dt, p.next_cycle_dt, p.time))
    return p, steps, {k: sha(O.real_cells(p, st[k])) for k in FIELDS}


@pytest.mark.parametrize("n,cycles", [(4096, 24), (2048, 120)])
def test_benchmark_configuration_matches_oracle_every_cycle(n, cycles):
    case = sod_circ(n, cycles)
    po, steps, ref = oracle_cycles(case)
    assert len(steps) == cycles
    # cycle by cycle: dt and time of every cycle
    with A.Solver(case) as s:
        s.init_test()
        seg, _ = s.tiling()
        got_steps = []
        for c in range(cycles):
            s.enqueue_cycles(1)
            p, st = s.state()
            assert st == 0 and p.cycle == c + 1
            got_steps.append((p.current_cycle_dt, p.next_cycle_dt, p.time))
        s.run()
        got = {k: sha(A.real_cells(s.params, s.download(k))) for k in FIELDS}
    for c, (a, b) in enumerate(zip(got_steps, steps)):
        assert a == b, f"cycle {c + 1}: (current dt, next dt, time) {a} != oracle {b}"
    assert got == ref, [k for k in FIELDS if got[k] != ref[k]]
    # in CUDA-graph batches, as the benchmark issues them
    with A.Solver(case, cycles_per_graph=16) as s:
        s.init_test()
        s.run()
        p, st = s.state()
        assert st == 0 and p.cycle == cycles and (p.current_cycle_dt, p.next_cycle_dt, p.time) == steps[-1]
        got = {k: sha(A.real_cells(s.params, s.download(k))) for k in FIELDS}
    assert got == ref, [k for k in FIELDS if got[k] != ref[k]]


def test_fp32_variant_at_8192_against_fp64_oracle():
    cycles = 30
    case = sod_circ(8192, cycles)
    L = O.lib()
    po = O.make_params(O.Case(**case.__dict__), L)
    st = O.OracleState(po)
    L.o_init_test_p(C.byref(po), C.byref(st.data), 0)
    m0, e0 = C.c_double(), C.c_double()
    L.o_conservation_vars_p(C.byref(po), C.byref(st.data), C.byref(m0), C.byref(e0))
    status = C.c_int()
    L.o_time_loop(C.byref(po), C.byref(st.data), C.byref(status))
    assert status.value == 0 and po.cycle == cycles
    ref = {k: O.real_cells(po, st[k]).copy() for k in ("rho", "Emat")}
    del st
    with A.Solver(case, precision=32) as s:
        s.init_test()
        m32_0, e32_0 = s.conservation()
        s.run()
        p, status = s.state()
        m32, e32 = s.conservation()
        got = {k: A.real_cells(s.params, s.download(k)) for k in ("rho", "Emat")}
    assert status == 0 and p.cycle == cycles
    for k in ("rho", "Emat"):
        l1 = np.abs(got[k] - ref[k]).sum() / np.abs(ref[k]).sum()
        assert l1 <= 1e-5, (k, l1)
    # FP64 sums of the FP32 state: the drift stays far below the FP32 rounding of one cell
    assert abs(m32 - m32_0) / m32_0 < 1e-6 and abs(e32 - e32_0) / e32_0 < 1e-6
    assert abs(dt_rel := (p.next_cycle_dt - po.next_cycle_dt) / po.next_cycle_dt) < 1e-5, dt_rel


def batch_sample():
    """8 domains of the 256-domain mix (seed 2024): its two largest and six others, seeded."""
    specs = W.mixed_domains(256, seed=2024)
    by_size = sorted(range(len(specs)), key=lambda i: -specs[i].nx * specs[i].ny)
    rng = np.random.default_rng(99)
    rest = [i for i in rng.permutation(len(specs)) if i not in by_size[:2]][:6]
    return [specs[i] for i in by_size[:2] + rest]


def test_batch_sample_of_the_mix_matches_oracle():
    sample = batch_sample()
    assert max(max(s.nx, s.ny) for s in sample) == 1024
    with A.Batch() as b:
        ids = [b.add_sod(sp.params(), sp.sod_interface()) for sp in sample]
        assert b.run() == 0
        res = []
        for i in ids:
            p, st = b.state(i)
            assert st == 0
            res.append((p, {k: sha(A.real_cells(b.params[i], b.download(i, k))) for k in FIELDS}))
    L = O.lib()
    for sp, (p, got) in zip(sample, res):
        po = O.make_params(O.Case(**sp.case().__dict__), L)
        st = O.OracleState(po)
        L.o_init_test_p(C.byref(po), C.byref(st.data), 0)
        for k, a in sp.initial_state().items():
            st[k][:] = a
        status = C.c_int()
        L.o_time_loop(C.byref(po), C.byref(st.data), C.byref(status))
        assert status.value == 0
        assert p.cycle == po.cycle and p.next_cycle_dt == po.next_cycle_dt and p.time == po.time, sp
        ref = {k: sha(O.real_cells(po, st[k])) for k in FIELDS}
        assert got == ref, (sp, [k for k in FIELDS if got[k] != ref[k]])
