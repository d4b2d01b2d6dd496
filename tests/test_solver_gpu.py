"""The fused GPU solver against the reference: bit-for-bit on FP64 (golden fixtures made by the
reference's own code, and the oracle on further cases), by tolerance for the FP32 variant."""
import ctypes as C
import hashlib
import json
import os

import numpy as np
import pytest

import armon_gb300 as A
import oracle_lib as O

pytestmark = pytest.mark.gpu

GOLDEN = json.load(open(os.path.join(os.path.dirname(__file__), "golden", "golden.json")))
FIELDS = ["rho", "umat", "vmat", "Emat", "pmat", "cmat"]
FUSED = [k for k, v in GOLDEN["cases"].items() if v["case"]["test"] != "Bizarrium"]


def sha(a):
    return hashlib.sha256(np.ascontiguousarray(a).tobytes()).hexdigest()


def run_solver(case, **kw):
    s = A.Solver(case, **kw)
    s.init_test()
    s.run()
    p, status = s.state()
    return s, p, status


@pytest.mark.parametrize("name", FUSED)
def test_fused_solver_matches_reference_bitwise(name):
    g = GOLDEN["cases"][name]
    s, p, status = run_solver(A.Case(**g["case"]))
    with s:
        assert status == 0
        assert p.cycle == g["cycles"]
        assert p.next_cycle_dt == float.fromhex(g["next_cycle_dt"])
        assert p.current_cycle_dt == float.fromhex(g["current_cycle_dt"])
        assert p.time == float.fromhex(g["time"])
        got = {k: sha(A.real_cells(s.params, s.download(k))) for k in FIELDS}
        bad = [k for k in FIELDS if got[k] != g["hashes"][k]]
        assert not bad, f"{name}: {bad} differ from the reference"
        m, e = s.conservation()
        # the GPU sums the same positive terms in another order: the two sums differ by at most the
        # rounding error bound of summation, 2 n u of the total (n terms, u = 2^-53)
        tol = 2 * g["case"]["nx"] * g["case"]["ny"] * 2.0 ** -53
        assert abs(m - float.fromhex(g["mass"])) <= tol * abs(m)
        assert abs(e - float.fromhex(g["energy"])) <= tol * abs(e)
        assert s.kernel_launches > 0


def _oracle_fields(case):
    p, st, status, _ = O.run(O.Case(**case.__dict__))
    assert status == 0
    return p, {k: O.real_cells(p, st[k]).copy() for k in FIELDS}


EXTRA = [
    # the benchmark's circular Sod at radius 0.2 (squared radius 0.04), a shrunken configuration 2
    A.Case(test="Sod_circ", scheme="GAD", projection="euler_2nd", nghost=5, nx=160, ny=96, cfl=0.6,
           max_cycles=12, max_time=1e9, test_option=0.04),
    A.Case(test="Sedov", scheme="GAD", projection="euler_2nd", limiter="Superbee", splitting="SequentialSym",
           nghost=4, nx=75, ny=52, max_cycles=15),
    A.Case(test="Sod_y", scheme="Godunov", projection="euler_2nd", splitting="Strang", nghost=3, nx=41, ny=67,
           max_cycles=12, max_time=1.0),
    A.Case(test="Sod", scheme="GAD", projection="euler", nghost=3, nx=5, ny=4, max_cycles=20, max_time=1.0),
]


@pytest.mark.parametrize("case", EXTRA, ids=lambda c: f"{c.test}-{c.scheme}-{c.projection}-{c.nx}x{c.ny}")
@pytest.mark.parametrize("seg_len,graph,eos_every_pass", [(0, 16, -1), (16, 0, 1), (23, 3, 0), (40, 0, -1)])
def test_fused_solver_matches_oracle_bitwise(case, seg_len, graph, eos_every_pass):
    # p, c, g written on every pass, on the last pass of each cycle, or computed from the last pass's
    # input when they are read: the same final arrays
    po, ref = _oracle_fields(case)
    s, p, status = run_solver(case, seg_len=seg_len, cycles_per_graph=graph, materialize_eos=eos_every_pass)
    with s:
        assert status == 0 and p.cycle == po.cycle
        assert p.next_cycle_dt == po.next_cycle_dt and p.time == po.time
        for k in FIELDS:
            got = A.real_cells(s.params, s.download(k))
            assert np.array_equal(got.view(np.int64), ref[k].view(np.int64)), k


def test_cycle_limit_and_resume_are_bitwise():
    case = A.Case(test="Sod_circ", scheme="GAD", projection="euler_2nd", nghost=5, nx=64, ny=48,
                  max_cycles=25, max_time=1e9)
    po, ref = _oracle_fields(case)
    s = A.Solver(case, cycles_per_graph=4)
    with s:
        s.init_test()
        s.run(cycle_limit=7)
        p, _ = s.state()
        assert p.cycle == 7
        s.run(cycle_limit=5)
        s.run()
        p, status = s.state()
        assert status == 0 and p.cycle == 25 and p.next_cycle_dt == po.next_cycle_dt
        for k in FIELDS:
            assert np.array_equal(A.real_cells(s.params, s.download(k)), ref[k]), k


def test_solve_host_end_to_end():
    """armon_solve_host: host buffers in, host buffers out (the reference-facing call)."""
    case = A.Case(test="Sod", scheme="Godunov", projection="euler", splitting="SequentialSym", nx=100, ny=100,
                  cfl=0.6, max_time=0.2, max_cycles=100000)
    g = GOLDEN["cases"]["cfg1_sod_godunov_100_symsplit"]
    final, outs = A.solve_host(case)
    assert final.cycle == g["cycles"] and final.next_cycle_dt == float.fromhex(g["next_cycle_dt"])
    p = A.make_params(case)
    for k in ("rho", "umat", "vmat", "Emat", "pmat"):
        assert sha(A.real_cells(p, outs[k])) == g["hashes"][k], k


def test_solve_host_with_uploaded_state_matches_oracle():
    """A non-test-case initial state given from the host (random smooth perturbation)."""
    case = A.Case(test="Sod_circ", scheme="GAD", projection="euler_2nd", nghost=5, nx=48, ny=40, max_cycles=10,
                  max_time=1e9)
    oc = O.Case(**case.__dict__)
    L = O.lib()
    po = O.make_params(oc)
    st = O.OracleState(po)
    L.o_init_test_p(C.byref(po), C.byref(st.data), 0)
    rng = np.random.default_rng(7)
    # relative perturbations keep rho and E positive (a NaN state is not bit-portable across CPUs/GPUs)
    for k, amp in (("rho", 0.05), ("Emat", 0.1)):
        st[k][:] = st[k] * (1 + amp * rng.uniform(-1, 1, st[k].size))
    for k in ("umat", "vmat"):
        st[k][:] = 0.02 * rng.uniform(-1, 1, st[k].size)
    inputs = {k: st[k].copy() for k in ("rho", "umat", "vmat", "Emat")}
    status = C.c_int()
    L.o_time_loop(C.byref(po), C.byref(st.data), C.byref(status))
    final, outs = A.solve_host(case, inputs=inputs)
    assert final.cycle == po.cycle and final.next_cycle_dt == po.next_cycle_dt
    p = A.make_params(case)
    for k in ("rho", "umat", "vmat", "Emat", "pmat"):
        assert np.array_equal(A.real_cells(p, outs[k]), O.real_cells(po, st[k])), k


def test_fp32_variant_close_to_fp64_oracle():
    case = A.Case(test="Sod_circ", scheme="GAD", projection="euler_2nd", nghost=5, nx=128, ny=128, cfl=0.6,
                  max_cycles=40, max_time=1e9, test_option=0.04)
    po, ref = _oracle_fields(case)
    s, p, status = run_solver(case, precision=32)
    with s:
        assert status == 0 and p.cycle == 40
        # dt is reduced in FP64 from FP32 fields: same cycle count, dt close
        assert abs(p.next_cycle_dt - po.next_cycle_dt) <= 1e-5 * po.next_cycle_dt
        for k in ("rho", "Emat"):
            got = A.real_cells(s.params, s.download(k))
            l1 = np.abs(got - ref[k]).sum() / np.abs(ref[k]).sum()
            assert l1 <= 1e-5, (k, l1)
        m, e = s.conservation()
        assert np.isfinite(m) and np.isfinite(e)


def test_invalid_dt_is_reported_not_fatal():
    """A state that gives dt <= 0 stops the loop with ARMON_ERR_INVALID_DT (the reference exits)."""
    case = A.Case(test="Sod", scheme="GAD", projection="euler_2nd", nghost=5, nx=32, ny=32, max_cycles=10)
    s = A.Solver(case)
    with s:
        s.init_test()
        E = s.download("Emat")
        p = s.params
        g, R = p.nb_ghosts, p.row_length
        E.reshape(p.col_length, R)[g + 3, g + 3] = np.inf   # c = inf there, so dt_CFL == 0
        s.upload("Emat", E)
        s.begin_loop()
        with pytest.raises(A.ArmonError) as ei:
            s.run()
        assert ei.value.code == A.ERR_INVALID_DT
        _, status = s.state()
        assert status == 1


def test_measured_tiling_keeps_results():
    # a domain large enough for the solver to time candidate tilings on its cycles (here only 4,
    # before the measurement starts); whatever it runs, the cycles give the same bits as fixed tilings
    case = A.Case(test="Sod_circ", scheme="GAD", projection="euler_2nd", nghost=5, nx=1024, ny=1024, cfl=0.6,
                  max_cycles=4, max_time=1e9, test_option=0.04)
    out = []
    for seg in (0, 64, 1024):
        s, p, status = run_solver(case, seg_len=seg)
        with s:
            assert status == 0 and p.cycle == 4
            (sx, sy), (bx, by) = s.tiling()
            assert sx > 0 and sy > 0 and bx > 0 and by > 0
            if seg:
                assert (sx, sy) == (seg, seg)
            out.append({k: s.download(k) for k in FIELDS})
    for other in out[1:]:
        for k in FIELDS:
            assert np.array_equal(out[0][k].view(np.int64), other[k].view(np.int64)), k



@pytest.mark.parametrize("precision", [64, 32])
def test_longest_first_dispatch_keeps_results(precision):
    # blocks launched in the order of the previous cycle's unit costs give the same bits as blocks
    # in index order, for 128- and 32-thread blocks and an alternating splitting
    case = A.Case(test="Sod_circ", scheme="GAD", projection="euler_2nd", nghost=5, nx=384, ny=320, cfl=0.6,
                  max_cycles=40, max_time=1e9, test_option=0.04, splitting="SequentialSym")
    ref = None
    for block, order in ((128, -1), (128, 0), (32, 0), (64, 0)):
        s, p, status = run_solver(case, precision=precision, block_lines=block, seg_len=24, unit_order=order,
                                  cycles_per_graph=8)
        with s:
            assert status == 0 and p.cycle == 40
            fields = {k: s.download(k) for k in FIELDS}
        if ref is None:
            ref = fields
            continue
        for k in FIELDS:
            assert np.array_equal(ref[k].view(np.int64), fields[k].view(np.int64)), (block, order, k)


@pytest.mark.parametrize("precision", [64, 32])
def test_tiling_measured_on_the_loops_own_cycles(precision):
    # a domain of 2^20 cells or more times its candidate tilings (and, in FP64, pass forms) on the
    # cycles of its own time loop: the results equal a fixed tiling's, the choice is cached for the
    # geometry, and a loop that ends while measuring keeps the model's tiling and caches nothing
    case = A.Case(test="Sod_circ", scheme="GAD", projection="euler_2nd", nghost=5, nx=1024, ny=1040, cfl=0.6,
                  max_cycles=120, max_time=1e9, test_option=0.04)
    A.tiling_cache_clear()
    with A.Solver(case, precision=precision) as s:
        s.init_test()
        assert s.tuning()
        s.run()
        p, status = s.state()
        assert status == 0 and p.cycle == 120 and not s.tuning()
        assert s.measurement_cycles() > 0 and s.measurement_cycles() % 2 == 0
        got = ({k: s.download(k) for k in FIELDS}, p.time, p.current_cycle_dt)
    with A.Solver(case, precision=precision) as s:
        s.init_test()
        assert not s.tuning()           # the cached choice
        s.run(cycle_limit=30)
        assert s.measurement_cycles() == 0
    with A.Solver(case, precision=precision, seg_len=128) as s:
        s.init_test()
        assert not s.tuning()
        s.run()
        p, status = s.state()
        assert s.measurement_cycles() == 0
        ref = ({k: s.download(k) for k in FIELDS}, p.time, p.current_cycle_dt)
    assert got[1:] == ref[1:]
    for k in FIELDS:
        assert np.array_equal(got[0][k].view(np.int64), ref[0][k].view(np.int64)), k
    # 20 cycles: the measurement starts after 16 and needs at least two per candidate
    A.tiling_cache_clear()
    short = A.Case(**{**case.__dict__, "max_cycles": 20})
    with A.Solver(short, precision=precision) as s:
        s.init_test()
        s.run()
        p, status = s.state()
        assert status == 0 and p.cycle == 20 and not s.tuning()
    with A.Solver(short, precision=precision) as s:
        s.init_test()
        assert s.tuning()               # nothing was cached


SPLIT_CASES = [
    dict(test="Sod_circ", scheme="GAD", projection="euler_2nd", splitting="Sequential"),
    dict(test="Sod_circ", scheme="GAD", projection="euler", splitting="SequentialSym"),
    dict(test="Sod", scheme="Godunov", projection="euler_2nd", splitting="Strang"),
    dict(test="Sedov", scheme="Godunov", projection="euler", splitting="Sequential"),
    dict(test="Sod_y", scheme="GAD", projection="euler", splitting="Sequential"),
]


@pytest.mark.parametrize("precision", [64, 32])
@pytest.mark.parametrize("kw", SPLIT_CASES, ids=lambda k: f"{k['test']}-{k['scheme']}-{k['projection']}-{k['splitting']}")
def test_split_pass_gives_the_fused_bits(kw, precision):
    # the pass as two launches (face fluxes through a face buffer, then the cell update) computes
    # the same operations on the same operands as the fused pass
    # the fewest ghosts the solver accepts for the scheme (2 + GAD + second order), so that the face
    # half's reads at the domain edges run right up to the end of the ghost band
    nghost = 2 + (kw["scheme"] == "GAD") + (kw["projection"] == "euler_2nd")
    case = A.Case(nghost=nghost, nx=200, ny=136, cfl=0.6, max_cycles=30, max_time=1e9, **kw)
    out = []
    for split in (-1, 1):
        s, p, status = run_solver(case, precision=precision, split_pass=split, seg_len=40)
        with s:
            assert status == 0 and p.cycle == 30
            out.append(({k: s.download(k) for k in FIELDS}, p.time, p.current_cycle_dt))
    (a, ta, da), (b, tb, db) = out
    assert ta == tb and da == db
    for k in FIELDS:
        assert np.array_equal(a[k].view(np.int64), b[k].view(np.int64)), k


@pytest.mark.parametrize("precision", [64, 32])
def test_eos_computed_when_read_matches_eos_written_by_the_passes(precision):
    # materialize_eos -1 (default): p, c, g are computed from the last pass's input when they are
    # downloaded or their device pointer taken, between cycles issued with enqueue_cycles, and give
    # what the passes write in mode 0 (last pass of each cycle), cycle count after cycle count
    case = A.Case(test="Sod_circ", scheme="GAD", projection="euler_2nd", nghost=5, nx=160, ny=96, cfl=0.6,
                  max_cycles=40, max_time=1e9, test_option=0.04)
    got = {}
    for mode in (-1, 0):
        with A.Solver(case, precision=precision, split_pass=-1, materialize_eos=mode) as s:
            s.init_test()
            out = []
            for n in (3, 8, 12):
                s.enqueue_cycles(n)
                out.append({k: s.download(k) for k in ("pmat", "cmat", "gmat", "rho")})
                if precision == 64:
                    ptr = A.lib().armon_solver_device_array(s._h, A.ARRAYS.index("cmat"))
                    assert ptr
            got[mode] = out
    for a, b in zip(got[-1], got[0]):
        for k in a:
            assert np.array_equal(a[k].view(np.int64), b[k].view(np.int64)), k
