"""Exact reuse over runs of identical inputs (armon_solver_opts.reuse, SweepArgs::reuse): a position
whose whole input window repeats the previous position's bit for bit stores the previous results.

These states are built to exercise the thresholds: every line is a sequence of runs of identical
cells whose lengths cover 1..16 (below, at and above each march's threshold), drawn from a small
palette of states at rest and in motion, along both axes.  With reuse on, every field must be the
same bits as with reuse off, for the fused pass and both halves of the split pass, in FP64 and FP32,
for several segment lengths, and in a batch; and FP64 must equal the oracle."""
import ctypes as C

import numpy as np
import pytest

import armon_gb300 as A
import oracle_lib as O

pytestmark = pytest.mark.gpu

FIELDS = ("rho", "umat", "vmat", "Emat", "pmat", "cmat")


def run_labels(n, rng):
    """Labels of n positions forming runs of random lengths 1..16 (consecutive runs differ)."""
    out, lab = [], 0
    while len(out) < n:
        lab += int(rng.integers(1, 4))
        out += [lab] * int(rng.integers(1, 17))
    return np.array(out[:n])


def runs_state(case, seed):
    """rho, umat, vmat, Emat over all nb_cells cells: palette state (lx + 3 ly) mod P at cell (x, y)."""
    rng = np.random.default_rng(seed)
    p = A.make_params(case)
    R, Cl = p.row_length, p.col_length
    lx, ly = run_labels(R, rng), run_labels(Cl, rng)
    P = 7
    rho = rng.uniform(0.5, 2.0, P)
    pr = rng.uniform(0.3, 2.0, P)
    u = np.where(np.arange(P) % 2 == 0, 0.0, rng.uniform(-0.3, 0.3, P))   # half of them at rest
    v = np.where(np.arange(P) % 3 == 0, 0.0, rng.uniform(-0.3, 0.3, P))
    idx = (lx[None, :] + 3 * ly[:, None]) % P
    E = pr / (0.4 * rho) + 0.5 * (u * u + v * v)
    return {"rho": rho[idx].ravel(), "umat": u[idx].ravel(), "vmat": v[idx].ravel(), "Emat": E[idx].ravel()}


def solve(case, state, **kw):
    with A.Solver(case, **kw) as s:
        s.init_test()
        for k, a in state.items():
            s.upload(k, a)
        s.begin_loop()
        s.run()
        p, st = s.state()
        assert st == 0
        return p, {k: A.real_cells(s.params, s.download(k)) for k in FIELDS}


def oracle(case, state):
    L = O.lib()
    p = O.make_params(O.Case(**case.__dict__))
    st = O.OracleState(p)
    L.o_init_test_p(C.byref(p), C.byref(st.data), 0)
    for k, a in state.items():
        st[k][:] = a
    status = C.c_int()
    L.o_time_loop(C.byref(p), C.byref(st.data), C.byref(status))
    assert status.value == 0
    return p, {k: O.real_cells(p, st[k]) for k in FIELDS}


CASES = [
    A.Case(test="Sod_circ", scheme="GAD", projection="euler_2nd", nghost=5, nx=203, ny=157, cfl=0.6,
           max_cycles=10, max_time=1e9),
    A.Case(test="Sod", scheme="GAD", projection="euler", splitting="SequentialSym", nghost=4, nx=170, ny=96,
           cfl=0.6, max_cycles=9, max_time=1e9),
    A.Case(test="Sod_y", scheme="Godunov", projection="euler_2nd", splitting="Strang", nghost=4, nx=120, ny=131,
           cfl=0.5, max_cycles=8, max_time=1e9),
]


def same_bits(a, b):
    return np.array_equal(np.asarray(a).view(np.uint64 if a.dtype == np.float64 else np.uint32),
                          np.asarray(b).view(np.uint64 if b.dtype == np.float64 else np.uint32))


@pytest.mark.parametrize("case", CASES, ids=lambda c: f"{c.test}-{c.scheme}-{c.projection}-{c.splitting}")
@pytest.mark.parametrize("precision", [64, 32])
@pytest.mark.parametrize("split_pass", [1, -1])
def test_reuse_is_bit_identical_to_full_computation(case, precision, split_pass):
    state = runs_state(case, seed=hash((case.nx, case.ny)) % 1000)
    for seg_len in (0, 23, 400):
        kw = dict(precision=precision, split_pass=split_pass, seg_len=seg_len)
        p0, ref = solve(case, state, reuse=-1, **kw)
        p1, got = solve(case, state, reuse=0, **kw)
        assert p0.cycle == p1.cycle == case.max_cycles
        assert p0.next_cycle_dt == p1.next_cycle_dt and p0.time == p1.time
        for k in FIELDS:
            assert same_bits(got[k], ref[k]), (seg_len, k)


@pytest.mark.parametrize("case", CASES[:2], ids=lambda c: f"{c.test}-{c.projection}")
def test_reuse_matches_oracle(case):
    state = runs_state(case, seed=5)
    po, ref = oracle(case, state)
    for split_pass in (1, -1):
        p, got = solve(case, state, split_pass=split_pass)
        assert p.cycle == po.cycle and p.next_cycle_dt == po.next_cycle_dt and p.time == po.time
        for k in FIELDS:
            assert same_bits(got[k], ref[k]), (split_pass, k)


@pytest.mark.parametrize("precision", [64, 32])
def test_batch_reuse_is_bit_identical(precision):
    # the batch kernels' streaming (FP32: batches of eight cells in a loop of their own) against every
    # position computed, and each domain against its solo solver
    cases = [CASES[0], A.Case(**{**CASES[0].__dict__, "nx": 64, "ny": 300}),
             A.Case(**{**CASES[0].__dict__, "nx": 333, "ny": 41})]
    states = [runs_state(c, seed=k) for k, c in enumerate(cases)]
    results = {}
    for reuse in (-1, 0):
        with A.Batch(precision=precision, cycles_per_graph=4, reuse=reuse) as b:
            ids = [b.add(A.make_params(c), st) for c, st in zip(cases, states)]
            assert b.run() == 0
            results[reuse] = [{k: A.real_cells(b.params[i], b.download(i, k)) for k in FIELDS} for i in ids]
    for a, r in zip(results[0], results[-1]):
        for k in FIELDS:
            assert same_bits(a[k], r[k]), k
    for c, st, a in zip(cases, states, results[0]):
        _, solo = solve(c, st, precision=precision)
        for k in FIELDS:
            assert same_bits(a[k], solo[k]), k
