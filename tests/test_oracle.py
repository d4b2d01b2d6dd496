"""The oracle against the reference: golden fixtures made by the reference's own code
(tests/golden/make_golden.py), plus the reference's in-tree known answers
(tests/armon_2D_tests.cpp in the reference)."""
import ctypes as C
import hashlib
import json
import os

import numpy as np
import pytest

import oracle_lib as O

GOLDEN = json.load(open(os.path.join(os.path.dirname(__file__), "golden", "golden.json")))
FIELDS = ["rho", "umat", "vmat", "Emat", "pmat", "cmat"]


def sha(a):
    return hashlib.sha256(np.ascontiguousarray(a).tobytes()).hexdigest()


def case_of(d):
    return O.Case(**d)


FAST_CASES = [k for k, v in GOLDEN["cases"].items()
              if v["case"]["nx"] * v["case"]["ny"] * v["cycles"] <= 2_000_000]
SLOW_CASES = [k for k in GOLDEN["cases"] if k not in FAST_CASES]


def _check_case(name):
    g = GOLDEN["cases"][name]
    p, st, status, _ = O.run(case_of(g["case"]))
    assert status == 0
    assert p.cycle == g["cycles"]
    assert p.next_cycle_dt == float.fromhex(g["next_cycle_dt"])
    assert p.current_cycle_dt == float.fromhex(g["current_cycle_dt"])
    assert p.time == float.fromhex(g["time"])
    got = {k: sha(O.real_cells(p, st[k])) for k in FIELDS}
    assert got == g["hashes"], f"{name}: fields differ from the reference"
    m, e = C.c_double(), C.c_double()
    O.lib().o_conservation_vars_p(C.byref(p), C.byref(st.data), C.byref(m), C.byref(e))
    assert m.value == float.fromhex(g["mass"]) and e.value == float.fromhex(g["energy"])


@pytest.mark.parametrize("name", FAST_CASES)
def test_oracle_matches_reference_bitwise(name):
    _check_case(name)


@pytest.mark.parametrize("name", SLOW_CASES)
def test_oracle_matches_reference_bitwise_long(name):
    _check_case(name)


@pytest.mark.parametrize("name,expected", [("ref_Sod", 45), ("ref_Sod_y", 45), ("ref_Sod_circ", 43),
                                           ("ref_Bizarrium", 76), ("ref_Sedov", 568)])
def test_reference_cycle_counts(name, expected):
    # tests/armon_2D_tests.cpp:238-242
    assert GOLDEN["cases"][name]["cycles"] == expected


@pytest.mark.parametrize("test", ["Sod", "Sod_y", "Sod_circ", "Sedov"])
def test_conservation(test):
    # tests/armon_2D_tests.cpp:246-275: mass and energy conserved to 1e-12 over 400 cycles
    g = GOLDEN["cases"][f"conservation_{test}"]
    L = O.lib()
    p = O.make_params(case_of(g["case"]))
    st = O.OracleState(p)
    L.o_init_test_p(C.byref(p), C.byref(st.data), 0)
    m0, e0 = C.c_double(), C.c_double()
    L.o_conservation_vars_p(C.byref(p), C.byref(st.data), C.byref(m0), C.byref(e0))
    status = C.c_int()
    L.o_time_loop(C.byref(p), C.byref(st.data), C.byref(status))
    m1, e1 = C.c_double(), C.c_double()
    L.o_conservation_vars_p(C.byref(p), C.byref(st.data), C.byref(m1), C.byref(e1))
    assert p.cycle == 400
    assert abs(m1.value - m0.value) <= 1e-12 * max(abs(m0.value), abs(m1.value))
    assert abs(e1.value - e0.value) <= 1e-12 * max(abs(e0.value), abs(e1.value))


def test_stage_sequence_matches_reference():
    """Every stage of the first two cycles (the reference's step_checkpoint list,
    src/armon_2D.cpp:255-324), all 16 arrays including ghosts."""
    L = O.lib()
    s = GOLDEN["stages"]
    p = O.make_params(case_of(s["case"]))
    st = O.OracleState(p)
    recs = iter(s["records"])

    def check(tag):
        r = next(recs)
        assert r["tag"] == tag
        got = {k: sha(st[k]) for k in O.ARRAY_NAMES}
        bad = [k for k in O.ARRAY_NAMES if got[k] != r["hashes"][k]]
        assert not bad, f"{tag} cycle {p.cycle}: {bad}"
        assert p.current_cycle_dt == float.fromhex(r["current_cycle_dt"])
        assert p.next_cycle_dt == float.fromhex(r["next_cycle_dt"])

    L.o_init_test_p(C.byref(p), C.byref(st.data), 0)
    check("init_test")
    p.cycle, p.time, p.current_cycle_dt, p.next_cycle_dt = 0, 0.0, 0.0, 0.0
    L.o_update_axis(C.byref(p), 0)
    L.o_update_EOS(C.byref(p), C.byref(st.data))
    check("EOS_init")
    while p.time < p.max_time and p.cycle < p.max_cycles:
        assert L.o_time_step(C.byref(p), C.byref(st.data)) == 0
        check("time_step")
        axes = (C.c_int32 * 3)()
        facs = (C.c_double * 3)()
        n = L.o_split_axes(C.byref(p), axes, facs)
        for k in range(n):
            L.o_update_axis(C.byref(p), axes[k])
            p.cycle_dt = p.current_cycle_dt * facs[k]
            for fn, tag in ((L.o_update_EOS, "EOS"), (L.o_boundary_conditions_p, "boundary_conditions"),
                            (L.o_numerical_fluxes, "numerical_fluxes"), (L.o_cell_update_p, "cell_update"),
                            (L.o_projection_remap, "projection_remap")):
                fn(C.byref(p), C.byref(st.data))
                check(tag)
        p.time += p.current_cycle_dt
        p.cycle += 1
    check("final")


def _default_params():
    # tests/armon_2D_tests.cpp:61-80
    return O.make_params(O.Case(test="Sod", scheme="GAD", projection="euler_2nd", limiter="Minmod",
                                nghost=5, nx=100, ny=5, max_cycles=100))


def _dom(d):
    return (d.col_start, d.col_step, d.col_end, d.row_start, d.row_step, d.row_end)


def test_indexing_known_answers():
    # tests/armon_2D_tests.cpp:83-189
    L = O.lib()
    p = _default_params()
    P = C.byref(p)
    assert L.o_params_check(P)
    assert _dom(L.o_real_domain(P)) == (555, 110, 995, 0, 1, 99)
    assert _dom(L.o_domain_fluxes(P)) == (555, 110, 995, -2, 1, 102)
    assert _dom(L.o_domain_advection(P)) == (555, 110, 995, 0, 1, 100)
    assert _dom(L.o_complete_domain(P)) == (5, 110, 1545, -5, 1, 104)
    for fn, length, rl, cl, b, e in ((L.o_real_domain, 500, 100, 5, 555, 1094),
                                     (L.o_domain_fluxes, 525, 105, 5, 553, 1097),
                                     (L.o_domain_advection, 505, 101, 5, 555, 1095),
                                     (L.o_complete_domain, 1650, 110, 15, 0, 1649)):
        d = fn(P)
        assert L.o_domain_length(d) == length
        assert L.o_domain_row_length(d) == rl
        assert L.o_domain_col_length(d) == cl
        assert L.o_domain_begin(d) == b
        assert L.o_domain_end(d) == e
    r, i1 = O.ORange(), O.OInner1D()
    L.o_domain_iter1D(L.o_real_domain(P), C.byref(r), C.byref(i1))
    assert (r.start, r.end, i1.start) == (0, 540, 555)
    r2, i2 = O.ORange(), O.OInner2D()
    L.o_domain_iter2D(L.o_real_domain(P), C.byref(r2), C.byref(i2))
    assert (r2.start, r2.end) == (0, 500)
    assert (i2.main_range_start, i2.main_range_step, i2.row_range_start, i2.row_range_length) == (555, 110, 0, 100)
    assert L.o_scale_index_2d(i2, 0) == 555 and L.o_scale_index_2d(i2, 499) == 1094
    assert L.o_scale_index_2d(i2, 100) == 555 + 110 and L.o_scale_index_2d(i2, 200) == 555 + 220
    for side, (b, e, n, disp) in enumerate([(554, 994, 5, 1), (655, 1095, 5, -1),
                                            (1105, 1204, 100, -110), (445, 544, 100, 110)]):
        dd = C.c_int32()
        d = L.o_boundary_conditions_domain(P, side, C.byref(dd))
        assert (L.o_domain_begin(d), L.o_domain_end(d), L.o_domain_length(d), dd.value) == (b, e, n, disp)


def test_ghost_requirement_check():
    # src/parameters.cpp:102-106: a stencil wider than the ghost layer is an error
    L = O.lib()
    p = O.make_params(O.Case(test="Sod", scheme="GAD", projection="euler_2nd", nghost=3, nx=10, ny=10))
    assert p.stencil_width == 4 and not L.o_params_check(C.byref(p))
    p = O.make_params(O.Case(test="Sod", scheme="Godunov", projection="euler", nghost=3, nx=10, ny=10))
    assert p.stencil_width == 1 and L.o_params_check(C.byref(p))


BORDERS = GOLDEN["borders"]
BORDER_FIELDS = ("rho", "umat", "vmat", "pmat", "cmat", "gmat", "Emat")


def border_inputs(p):
    """The field values the reference's border records were made from: exact integers
    ((37 i + 1013 k) mod 65521) - 30000 for field k and linear cell index i."""
    i = np.arange(p.nb_cells, dtype=np.int64)
    return {name: ((37 * i + 1013 * k) % 65521 - 30000).astype(np.float64) for k, name in enumerate(BORDER_FIELDS)}


def test_border_arrays_match_reference():
    """read_border_array / write_border_array (src/kernels/halo_exchange.cpp:39-92) of the oracle
    against the reference's own output on the four borders (tests/golden/borders_20x12.npz)."""
    L = O.lib()
    p = O.make_params(O.Case(**BORDERS["case"]))
    f = border_inputs(p)
    ptr = lambda a: a.ctypes.data_as(C.POINTER(C.c_double))
    packed = []
    saved = np.load(os.path.join(os.path.dirname(__file__), "golden", "borders_20x12.npz"))
    for side in BORDERS["sides"]:
        r = O.ORange(*side["range"])
        ir = O.OInner2D(*side["inner"])
        va = np.full(7 * side["nghost"] * side["side_length"], np.nan)
        L.o_read_border_array(r, ir, side["side_length"], side["nghost"], *[ptr(f[k]) for k in BORDER_FIELDS], ptr(va))
        assert sha(va) == side["values"], side["tag"]
        assert np.array_equal(va, saved[side["tag"]]), side["tag"]
        packed.append(va)
    for side, va in zip(BORDERS["sides"], packed):
        va2 = 2 * va + 1
        L.o_write_border_array(O.ORange(*side["range"]), O.OInner2D(*side["inner"]), side["side_length"],
                               side["nghost"], *[ptr(f[k]) for k in BORDER_FIELDS], ptr(va2))
    for k in BORDER_FIELDS:
        assert sha(f[k]) == BORDERS["final_hashes"][k], k
