"""The batched multi-domain step (armon_batch_*): every domain of a batch must give what it gives
alone, bit for bit in FP64, and what the oracle gives for the same initial state."""
import ctypes as C

import numpy as np
import pytest

import armon_gb300 as A
import oracle_lib as O
from armon_gb300 import workloads as W

pytestmark = pytest.mark.gpu

FIELDS = ("rho", "umat", "vmat", "Emat", "pmat")


def small_domains(n, seed, sides=(16, 24, 40, 64, 96), t_end=0.15):
    ds = W.mixed_domains(n, seed=seed, sides=sides)
    for k, d in enumerate(ds):
        d.t_end = t_end * (0.5 + 0.5 * (k % 3) / 2)   # different end times: domains finish apart
    return ds


def solo(spec, precision=64, seg_len=0):
    with A.Solver(spec.params(), precision=precision, seg_len=seg_len) as s:
        s.init_test()
        for k, a in spec.initial_state().items():
            s.upload(k, a)
        s.begin_loop()
        s.run()
        p, st = s.state()
        return p, st, {k: A.real_cells(s.params, s.download(k)) for k in FIELDS}


def oracle(spec):
    L = O.lib()
    p = O.make_params(O.Case(**spec.case().__dict__))
    st = O.OracleState(p)
    L.o_init_test_p(C.byref(p), C.byref(st.data), 0)
    for k, a in spec.initial_state().items():
        st[k][:] = a
    status = C.c_int()
    L.o_time_loop(C.byref(p), C.byref(st.data), C.byref(status))
    assert status.value == 0
    return p, {k: O.real_cells(p, st[k]) for k in FIELDS}


def test_batch_domains_match_solo_runs_bitwise():
    specs = small_domains(14, seed=11)
    with A.Batch(cycles_per_graph=4) as b:
        ids = [b.add(s.params(), s.initial_state()) for s in specs]
        assert b.run() == 0
        for i, spec in zip(ids, specs):
            pb, stb = b.state(i)
            ps, sts, ref = solo(spec)
            assert stb == 0 and sts == 0
            assert pb.cycle == ps.cycle and pb.time == ps.time and pb.next_cycle_dt == ps.next_cycle_dt
            for k in FIELDS:
                got = A.real_cells(b.params[i], b.download(i, k))
                assert np.array_equal(got.view(np.int64), ref[k].view(np.int64)), (spec, k)
        assert b.kernel_launches > 0


def test_batch_domain_matches_oracle():
    spec = small_domains(3, seed=5, sides=(48, 80))[2]
    po, ref = oracle(spec)
    with A.Batch() as b:
        i = b.add(spec.params(), spec.initial_state())
        b.run()
        pb, st = b.state(i)
        assert st == 0 and pb.cycle == po.cycle and pb.next_cycle_dt == po.next_cycle_dt
        for k in FIELDS:
            assert np.array_equal(A.real_cells(b.params[i], b.download(i, k)), ref[k]), k


def test_batch_admission_removal_and_budget():
    specs = small_domains(6, seed=3)
    per = [A.domain_bytes(s.params()) for s in specs]
    budget = sum(per[:3]) + per[3] // 2
    with A.Batch(memory_budget=budget) as b:
        ids = [b.add(s.params(), s.initial_state()) for s in specs[:3]]
        with pytest.raises(A.ArmonError) as ei:
            b.add(specs[3].params(), specs[3].initial_state())
        assert ei.value.code == A.ERR_NOMEM
        b.run(cycle_limit=5)
        b.remove(ids[1])                      # frees a slot and its memory
        assert b.bytes_in_use == per[0] + per[2]
        j = b.add(specs[4].params(), specs[4].initial_state())   # admitted while others are mid-run
        assert j == ids[1]                    # slot reused
        assert b.run() == 0
        for i, spec in ((ids[0], specs[0]), (ids[2], specs[2]), (j, specs[4])):
            ps, _, ref = solo(spec)
            pb, _ = b.state(i)
            assert pb.cycle == ps.cycle
            for k in FIELDS:
                assert np.array_equal(A.real_cells(b.params[i], b.download(i, k)), ref[k]), k


def test_batch_fp32_identical_to_solo_fp32():
    specs = small_domains(5, seed=21)
    with A.Batch(precision=32) as b:
        ids = [b.add(s.params(), s.initial_state()) for s in specs]
        b.run()
        for i, spec in zip(ids, specs):
            ps, _, ref = solo(spec, precision=32)
            pb, _ = b.state(i)
            assert pb.cycle == ps.cycle
            for k in FIELDS:
                got = A.real_cells(b.params[i], b.download(i, k))
                assert np.array_equal(got, ref[k]), k


def test_batch_segment_choice_does_not_change_results():
    spec = small_domains(1, seed=9, sides=(96,))[0]
    _, _, ref = solo(spec)
    with A.Batch() as b:
        i = b.add(spec.params(), spec.initial_state())
        b.set_seg_len(i, 17)
        b.run()
        for k in FIELDS:
            assert np.array_equal(A.real_cells(b.params[i], b.download(i, k)), ref[k]), k


def test_autotuned_schedule_keeps_results():
    # enough cells for the tuner to time its candidates (one 8-cycle graph batch each)
    specs = W.mixed_domains(6, seed=31, sides=(512, 768, 1024))
    for s in specs:
        s.t_end = 1.0
    out = []
    for waves in (0, 2):
        with A.Batch(cycles_per_graph=8, waves=waves) as b:
            ids = [b.add_sod(s.params(), s.sod_interface()) for s in specs]
            b.run(cycle_limit=56)
            w, blocks = b.schedule()
            if waves == 0:
                assert w in (2, 4, 8, 16, 64) and blocks > 0
            else:
                assert w == 2
            out.append([{k: b.download(i, k) for k in FIELDS} for i in ids])
            for i in ids:
                assert b.state(i)[0].cycle == 56
    for a, c in zip(*out):
        for k in FIELDS:
            assert np.array_equal(a[k], c[k]), k


@pytest.mark.parametrize("splitting", ["SequentialSym", "Strang"])
def test_late_joiners_with_parity_dependent_axes_match_solo(splitting):
    # with these splittings a pass's axis depends on each domain's own cycle parity, so domains that
    # join after an odd number of cycles sweep the other axis in the same launches
    specs = small_domains(4, seed=41, sides=(24, 40, 64), t_end=0.1)
    for s in specs:
        s.splitting = splitting
    with A.Batch(cycles_per_graph=4) as b:
        ids = [b.add(s.params(), s.initial_state()) for s in specs[:2]]
        b.run(cycle_limit=3)
        ids += [b.add(s.params(), s.initial_state()) for s in specs[2:]]
        assert b.run() == 0
        for i, spec in zip(ids, specs):
            pb, stb = b.state(i)
            ps, sts, ref = solo(spec)
            assert stb == 0 and sts == 0 and pb.cycle == ps.cycle and pb.time == ps.time
            for k in FIELDS:
                got = A.real_cells(b.params[i], b.download(i, k))
                assert np.array_equal(got.view(np.int64), ref[k].view(np.int64)), (splitting, k)



def test_split_and_fused_batch_passes_agree_bitwise():
    # the batch's passes as face + cell launches (the FP64 default) and as one fused launch
    specs = small_domains(10, seed=23, sides=(24, 40, 64, 96, 130))
    out = []
    for split in (1, -1):
        with A.Batch(cycles_per_graph=4, split_pass=split) as b:
            ids = [b.add(s.params(), s.initial_state()) for s in specs]
            assert b.run() == 0
            out.append([(b.state(i)[0].cycle, b.state(i)[0].time,
                         {k: b.download(i, k) for k in FIELDS}) for i in ids])
    for (ca, ta, fa), (cb, tb, fb) in zip(*out):
        assert ca == cb and ta == tb
        for k in FIELDS:
            assert np.array_equal(fa[k].view(np.int64), fb[k].view(np.int64)), k


@pytest.mark.parametrize("precision", [64, 32])
def test_longest_first_batch_dispatch_keeps_results(precision):
    # the blocks of all domains launched by the previous cycle's costs or in index order
    specs = small_domains(9, seed=31, sides=(24, 40, 64, 96, 130))
    out = []
    for order in (0, -1):
        with A.Batch(precision=precision, cycles_per_graph=4, unit_order=order) as b:
            ids = [b.add(s.params(), s.initial_state()) for s in specs]
            assert b.run() == 0
            out.append([(b.state(i)[0].cycle, b.state(i)[0].time, {k: b.download(i, k) for k in FIELDS})
                        for i in ids])
    for (ca, ta, fa), (cb, tb, fb) in zip(*out):
        assert ca == cb and ta == tb
        for k in FIELDS:
            assert np.array_equal(fa[k].view(np.int64), fb[k].view(np.int64)), k
