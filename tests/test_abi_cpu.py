"""CPU checks of the C ABI: the library loads, exports every entry point the headers declare,
and its host-side parameter logic agrees with the oracle's restatement of the reference."""
import ctypes as C
import os
import re
import subprocess

import pytest

import oracle_lib as O
import armon_gb300 as A

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_functions():
    names = set()
    for h in ("armon_gb300.h", "armon_kernels.h"):
        src = open(os.path.join(ROOT, "include", h)).read()
        src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
        for m in re.finditer(r"^[A-Za-z_][\w\s\*]*?\b([a-z_][a-zA-Z0-9_]*)\s*\(", src, flags=re.M):
            name = m.group(1)
            if name not in ("if", "for", "while", "sizeof", "return", "void", "int", "double", "bool"):
                names.add(name)
    names.add("raise_exception_handler")
    return sorted(names)


def test_library_exports_every_declared_symbol():
    L = A.lib()
    out = subprocess.run(["nm", "-D", "--defined-only", A.LIB_PATH], capture_output=True, text=True).stdout
    exported = {line.split()[-1] for line in out.splitlines() if line.strip()}
    missing = [n for n in declared_functions() if n not in exported]
    assert not missing, f"declared but not exported: {missing}"
    for n in declared_functions():
        getattr(L, n)  # resolvable through dlsym


def test_introspection():
    # src/kernels/utils.cpp:20-27 (64-bit indices, unsigned UIdx, double flt_t)
    L = A.lib()
    assert L.idx_size() == 8 and L.is_uidx_signed() is False and L.flt_size() == 8


def test_params_layout_matches_oracle():
    assert A.lib().armon_params_sizeof() == O.lib().o_params_sizeof() == C.sizeof(A.Params)
    assert [f[0] for f in A.Params._fields_] == [f[0] for f in O.OParams._fields_]
    for (n, t), (n2, t2) in zip(A.Params._fields_, O.OParams._fields_):
        assert getattr(A.Params, n).offset == getattr(O.OParams, n2).offset


CASES = [
    O.Case(test=t, scheme=s, projection=pr, nghost=g, nx=nx, ny=ny, stencil=sw, cfl=cfl)
    for t in ("Sod", "Sod_y", "Sod_circ", "Bizarrium", "Sedov")
    for s, pr in (("Godunov", "euler"), ("GAD", "euler_2nd"), ("GAD", "euler"))
    for g, nx, ny, sw, cfl in ((3, 10, 10, -1, 0.0), (5, 100, 5, -1, 0.6), (5, 37, 23, 5, 0.0))
]


@pytest.mark.parametrize("case", CASES, ids=lambda c: f"{c.test}-{c.scheme}-{c.projection}-{c.nx}x{c.ny}")
def test_params_init_and_check_match_oracle(case):
    pa = A.make_params(A.Case(**case.__dict__))
    po = O.make_params(case)
    for name, _ in A.Params._fields_:
        va, vo = getattr(pa, name), getattr(po, name)
        if hasattr(va, "__len__"):
            assert list(va) == list(vo), name
        else:
            assert va == vo or (va != va and vo != vo), name
    assert bool(A.lib().armon_params_check(C.byref(pa))) == bool(O.lib().o_params_check(C.byref(po)))
    assert A.lib().armon_min_ghosts(C.byref(pa)) == O.lib().o_min_ghosts(C.byref(po))


def test_boundary_factors_match_oracle():
    fa = A.lib().armon_boundary_factors
    fa.argtypes = [C.c_int, C.c_int, C.POINTER(C.c_double), C.POINTER(C.c_double)]
    for test in range(5):
        for side in range(4):
            a = (C.c_double(), C.c_double())
            o = (C.c_double(), C.c_double())
            fa(test, side, C.byref(a[0]), C.byref(a[1]))
            O.lib().o_boundary_factors(test, side, C.byref(o[0]), C.byref(o[1]))
            assert (a[0].value, a[1].value) == (o[0].value, o[1].value)


def _align256(n):
    return (n + 255) & ~255


@pytest.mark.parametrize("nx,ny", [(64, 64), (300, 128), (1024, 2048)])
def test_batch_domain_bytes_count_the_face_buffer_in_fp64(nx, ny):
    # a batch domain holds 11 state arrays and its dt partials; an FP64 domain (split passes by
    # default) also holds three face arrays of max((nx + 5) ny, (ny + 5) nx) values
    p = A.make_params(A.Case(test="Sod_circ", scheme="GAD", projection="euler_2nd", nghost=5, nx=nx, ny=ny))
    f64, f32 = A.domain_bytes(p, 64), A.domain_bytes(p, 32)
    arrays64, arrays32 = 11 * _align256(p.nb_cells * 8), 11 * _align256(p.nb_cells * 4)
    faces64 = 3 * _align256(max((nx + 5) * ny, (ny + 5) * nx) * 8)
    partials = f32 - arrays32
    assert 0 < partials < 1 << 24 and partials % 256 == 0
    assert f64 == arrays64 + partials + faces64


@pytest.mark.parametrize("gad", [0, 1])
@pytest.mark.parametrize("second_order", [0, 1])
def test_split_pass_positions_stay_inside_the_required_ghosts(gad, second_order):
    # the index ranges of csrc/sweep_split.cuh for a line of n cells cut into segments, against the
    # ghost depth the solver requires (2 + GAD + second order); a restatement of the kernel's
    # arithmetic, checked here before any GPU runs it
    reach = 2 + gad + second_order
    r = 2 if second_order else 1
    for n, seg in ((16, 16), (40, 7), (100, 33), (5, 1)):
        segments = [(a0, min(n, a0 + seg)) for a0 in range(0, n, seg)]
        written, lo, hi = set(), 10**9, -10**9
        for a0, b0 in segments:
            fs = -r if a0 == 0 else a0
            fe = n + r + 1 if b0 == n else b0
            assert not written & set(range(fs, fe))                  # each face has one writer
            written |= set(range(fs, fe))
            t0, t1 = (fs - 2, fe) if gad else (fs - 1, fe - 1)       # the face half's positions
            lo, hi = min(lo, t0), max(hi, t1)
        for a0, b0 in segments:
            t0, t1 = a0 - r, b0 + r                                  # the cell half's iterations
            assert set(range(t0, t1 + 1)) <= written                 # face t of each iteration
            lo, hi = min(lo, t0 - 1), max(hi, t1 - 1)                # cell t - 1 of each iteration
        assert written == set(range(-r, n + r + 1)) and -2 <= -r and n + r <= n + 2   # n + 5 faces a line
        assert -reach <= lo and hi <= n + reach - 1, (n, seg, lo, hi, reach)


def test_soft_addition_matches_ieee_addition_on_the_host():
    # csrc/softfp.cuh add_bits (the integer-pipe FP64 addition, compiled for the host here) against
    # the host's IEEE addition on generated operands: every bit class, cancellations, ties, every
    # exponent, overflow and underflow ranges, zeros
    L = A.lib()
    L.armon_selftest_add_host.argtypes = [C.c_uint64, C.c_int64, C.POINTER(C.c_uint64)]
    for seed in (0x9E3779B97F4A7C15, 0x0F1E2D3C4B5A6978):
        out = (C.c_uint64 * 4)()
        assert L.armon_selftest_add_host(seed, 10_000_000, out) == 0
        assert out[0] == 0, f"{out[0]} mismatches, first a=0x{out[2]:016x} b=0x{out[3]:016x}"
        assert out[1] > 9_900_000
