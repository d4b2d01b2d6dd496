"""The serving loop (armon_server_*): requests admitted in order against a memory budget and advanced
together in shared batches (continuous batching), each giving the same result as the same solve run
alone -- bit for bit, in FP64 and in FP32."""
import numpy as np
import pytest

import armon_gb300 as A
from armon_gb300 import serving as S
from armon_gb300 import workloads as W
from test_batch_gpu import FIELDS, solo

pytestmark = pytest.mark.gpu


def small_trace(n, seed, rate=400.0):
    tr = W.serving_trace(n=n, rate=rate, seed=seed, mu=3.9, sigma=0.5, side_range=(24, 96))
    for r in tr:
        r.spec.t_end *= 0.25          # short solves: 10 to 60 cycles
    return tr


@pytest.mark.parametrize("precision", [64, 32])
def test_device_interface_init_matches_host_state(precision):
    specs = W.mixed_domains(6, seed=5, sides=(16, 40, 64))
    with A.Batch(precision=precision) as b:
        for spec in specs:
            i = b.add_sod(spec.params(), spec.sod_interface())
            j = b.add(spec.params(), spec.initial_state())
            host = spec.initial_state()
            for k in ("rho", "umat", "vmat", "Emat"):
                got = b.download(i, k)
                assert np.array_equal(got, b.download(j, k)), (spec, k)
                want = host[k] if precision == 64 else host[k].astype(np.float32).astype(np.float64)
                assert np.array_equal(got, want), (spec, k)


def test_served_requests_match_solo_runs():
    trace = small_trace(12, seed=3)
    assert {r.spec.precision for r in trace} == {32, 64}
    results = {}

    with A.Server(cycles_per_step=4) as srv:
        def keep(rid, k, info):
            results[k] = {f: A.real_cells(srv.params[rid], srv.download(rid, f)) for f in FIELDS}

        served, wall = S.replay(srv, trace, on_done=keep)
        assert srv.bytes_in_use == 0
    assert len(served) == len(trace) and wall > 0
    for rec in served:
        spec = trace[rec.index].spec
        assert rec.status == A.REQ_DONE and rec.done >= rec.admitted >= rec.arrival - 1e-3
        p, st, ref = solo(spec, precision=spec.precision)
        assert st == 0 and rec.cycles == p.cycle
        for f in FIELDS:
            assert np.array_equal(results[rec.index][f], ref[f]), (rec.index, spec.precision, f)


def test_admission_is_in_order_and_within_budget():
    specs = W.mixed_domains(7, seed=8, sides=(32, 64, 96))
    for s in specs:
        s.t_end = 0.03
    need = [A.domain_bytes(s.params(), 64) for s in specs]
    budget = sorted(need)[-1] + sorted(need)[-2]        # two of the largest at once, at most
    with A.Server(memory_budget=budget, cycles_per_step=2) as srv:
        ids = [srv.submit(s.params(), 64, s.sod_interface()) for s in specs]
        peak = 0
        finished = []
        for _ in range(10_000):
            running, queued = srv.step()
            peak = max(peak, srv.bytes_in_use)
            assert srv.bytes_in_use <= budget
            while (r := srv.next_done()) is not None:
                finished.append(r)
                srv.release(r)
            if running == 0 and queued == 0:
                break
        assert sorted(finished) == ids
        infos = [srv.info(r) for r in ids]
        assert all(i.status == A.REQ_DONE for i in infos)
        admits = [i.t_admit for i in infos]
        assert admits == sorted(admits)                   # first come, first served
        assert peak > max(need)                           # solves did overlap


def test_unsupported_request_fails_alone():
    specs = W.mixed_domains(3, seed=9, sides=(32,))
    with A.Server() as srv:
        good = [srv.submit(s.params(), 64, s.sod_interface()) for s in specs]
        bad = srv.submit(A.Case(test="Bizarrium", scheme="GAD", projection="euler_2nd", limiter="Minmod",
                                nghost=5, nx=32, ny=32, max_cycles=5), 64)
        done = {}
        for _ in range(10_000):
            running, queued = srv.step()
            while (r := srv.next_done()) is not None:
                done[r] = srv.info(r).status
            if running == 0 and queued == 0:
                break
        assert done[bad] == A.REQ_FAILED
        assert all(done[g] == A.REQ_DONE for g in good)


def test_cell_limit_keeps_batches_under_it_in_order():
    specs = W.mixed_domains(10, seed=12, sides=(32, 48, 64))
    for k, s in enumerate(specs):
        s.t_end = 0.03
        s.precision = 64 if k % 2 == 0 else 32
    cap = 2 * 64 * 64
    with A.Server(cycles_per_step=2, max_inflight_cells=cap) as srv:
        ids = [srv.submit(s.params(), s.precision, s.sod_interface()) for s in specs]
        for _ in range(10_000):
            running, queued = srv.step()
            for prec in (64, 32):
                run = [i for i in ids if srv.info(i).status == A.REQ_RUNNING and srv.info(i).precision == prec]
                cells = sum(srv.info(i).nx * srv.info(i).ny for i in run)
                assert cells <= cap or len(run) == 1
            while (r := srv.next_done()) is not None:
                srv.release(r)
            if running == 0 and queued == 0:
                break
        infos = [srv.info(i) for i in ids]
        assert all(i.status == A.REQ_DONE for i in infos)
        for prec in (64, 32):
            admits = [i.t_admit for i in infos if i.precision == prec]
            assert admits == sorted(admits)            # first come, first served within a batch

