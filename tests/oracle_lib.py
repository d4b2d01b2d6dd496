"""ctypes access to the oracle (oracle/armon_oracle.c) for the tests and the bench's CPU leg.

The oracle is the checker: it restates the reference's time step on the CPU with the same
expression order, so a strict build reproduces the reference bit for bit.  Nothing in the
product imports this module.
"""
from __future__ import annotations

import ctypes as C
import math
import os
import subprocess
from dataclasses import dataclass

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
ORACLE_DIR = os.path.join(ROOT, "oracle")
BUILD_DIR = os.path.join(ORACLE_DIR, "_build")

TESTS = {"Sod": 0, "Sod_y": 1, "Sod_circ": 2, "Bizarrium": 3, "Sedov": 4}
SCHEMES = {"Godunov": 0, "GAD": 1}
PROJECTIONS = {"none": 0, "euler": 1, "euler_2nd": 2}
LIMITERS = {"None": 0, "Minmod": 1, "Superbee": 2}
SPLITTINGS = {"Sequential": 0, "SequentialSym": 1, "Strang": 2, "X_only": 3, "Y_only": 4}

ARRAY_NAMES = ["x", "y", "rho", "umat", "vmat", "Emat", "pmat", "cmat", "gmat", "ustar", "pstar",
               "work_array_1", "work_array_2", "work_array_3", "work_array_4", "domain_mask"]


class OParams(C.Structure):
    """Same layout as o_params (oracle) and armon_params (product)."""
    _fields_ = [(n, C.c_int32) for n in (
        "test", "scheme", "riemann", "projection", "limiter", "current_axis", "axis_splitting",
        "nb_ghosts", "nx", "ny", "stencil_width", "cst_dt", "dt_on_even_cycles",
        "row_length", "col_length", "nb_cells", "ideb", "ifin", "index_start", "idx_row", "idx_col", "s",
        "cycle", "max_cycles",
        "write_output", "write_ghosts", "write_throughput", "output_precision", "verbose", "compare")] + [
        ("dx", C.c_double), ("cfl", C.c_double), ("Dt", C.c_double),
        ("domain_size", C.c_double * 2), ("domain_origin", C.c_double * 2),
        ("cycle_dt", C.c_double), ("current_cycle_dt", C.c_double), ("next_cycle_dt", C.c_double),
        ("time", C.c_double), ("max_time", C.c_double), ("comparison_tolerance", C.c_double),
        ("test_option", C.c_double)]


class OData(C.Structure):
    _fields_ = [(n, C.POINTER(C.c_double)) for n in ARRAY_NAMES]


class ODomain(C.Structure):
    _fields_ = [(n, C.c_int64) for n in ("col_start", "col_step", "col_end", "row_start", "row_step", "row_end")]


class ORange(C.Structure):
    _fields_ = [("start", C.c_int64), ("end", C.c_int64)]


class OInner1D(C.Structure):
    _fields_ = [("start", C.c_int64), ("step", C.c_int64)]


class OInner2D(C.Structure):
    _fields_ = [("main_range_start", C.c_int64), ("main_range_step", C.c_int64),
                ("row_range_start", C.c_int64), ("row_range_length", C.c_uint64)]


def build(quiet: bool = True) -> None:
    """Compile the oracle (strict + fast builds) with its Makefile."""
    out = subprocess.run(["make", "-C", ORACLE_DIR, "-j4"], capture_output=True, text=True)
    if out.returncode != 0:
        raise RuntimeError("oracle build failed:\n" + out.stdout + out.stderr)


_LIBS: dict[str, C.CDLL] = {}


def lib(fast: bool = False) -> C.CDLL:
    name = "liboracle_fast.so" if fast else "liboracle.so"
    if name in _LIBS:
        return _LIBS[name]
    path = os.path.join(BUILD_DIR, name)
    if not os.path.exists(path):
        build()
    L = C.CDLL(path)
    P = C.POINTER(OParams)
    D = C.POINTER(OData)
    L.o_params_defaults.argtypes = [P]
    L.o_params_init.argtypes = [P]
    L.o_params_check.argtypes = [P]
    L.o_params_check.restype = C.c_int
    L.o_params_sizeof.restype = C.c_int
    L.o_num_threads.restype = C.c_int
    L.o_min_ghosts.argtypes = [P]
    L.o_min_ghosts.restype = C.c_int
    L.o_init_test_p.argtypes = [P, D, C.c_int]
    L.o_time_loop.argtypes = [P, D, C.POINTER(C.c_int)]
    L.o_time_loop.restype = C.c_double
    L.o_solver_cycle.argtypes = [P, D]
    L.o_solver_cycle.restype = C.c_int
    L.o_time_step.argtypes = [P, D]
    L.o_time_step.restype = C.c_int
    for fn in ("o_update_EOS", "o_boundary_conditions_p", "o_numerical_fluxes", "o_cell_update_p",
               "o_projection_remap"):
        getattr(L, fn).argtypes = [P, D]
    L.o_update_axis.argtypes = [P, C.c_int]
    L.o_conservation_vars_p.argtypes = [P, D, C.POINTER(C.c_double), C.POINTER(C.c_double)]
    L.o_split_axes.argtypes = [P, C.POINTER(C.c_int32), C.POINTER(C.c_double)]
    L.o_split_axes.restype = C.c_int
    for fn in ("o_real_domain", "o_domain_fluxes", "o_domain_cell_update", "o_domain_advection",
               "o_complete_domain"):
        getattr(L, fn).argtypes = [P]
        getattr(L, fn).restype = ODomain
    L.o_boundary_conditions_domain.argtypes = [P, C.c_int, C.POINTER(C.c_int32)]
    L.o_boundary_conditions_domain.restype = ODomain
    for fn in ("o_domain_length", "o_domain_row_length", "o_domain_col_length"):
        getattr(L, fn).argtypes = [ODomain]
        getattr(L, fn).restype = C.c_uint64
    for fn in ("o_domain_begin", "o_domain_end"):
        getattr(L, fn).argtypes = [ODomain]
        getattr(L, fn).restype = C.c_int64
    L.o_domain_iter1D.argtypes = [ODomain, C.POINTER(ORange), C.POINTER(OInner1D)]
    L.o_domain_direct_iter1D.argtypes = [ODomain, C.POINTER(ORange), C.POINTER(OInner1D)]
    L.o_domain_iter2D.argtypes = [ODomain, C.POINTER(ORange), C.POINTER(OInner2D)]
    L.o_scale_index_2d.argtypes = [OInner2D, C.c_uint64]
    L.o_scale_index_2d.restype = C.c_int64
    L.o_boundary_factors.argtypes = [C.c_int, C.c_int, C.POINTER(C.c_double), C.POINTER(C.c_double)]
    DP = C.POINTER(C.c_double)
    for fn in ("o_read_border_array", "o_write_border_array"):
        getattr(L, fn).argtypes = [ORange, OInner2D, C.c_int64, C.c_int64] + [DP] * 8
        getattr(L, fn).restype = None
    _LIBS[name] = L
    return L


@dataclass
class Case:
    """A solver configuration in the reference's own terms (CLI names, src/main_2D.cpp:9-38)."""
    test: str = "Sod"
    scheme: str = "GAD"
    projection: str = "euler"
    limiter: str = "Minmod"
    splitting: str = "Sequential"
    nghost: int = 3
    nx: int = 10
    ny: int = 10
    stencil: int = -1
    cfl: float = 0.0
    dt: float = 0.0
    cst_dt: int = 0
    dt_on_even_cycles: int = 0
    max_cycles: int = 100
    max_time: float = 0.0
    test_option: float = 0.0

    def driver_args(self) -> list[str]:
        a = [f"test={self.test}", f"scheme={self.scheme}", f"projection={self.projection}",
             f"limiter={self.limiter}", f"splitting={self.splitting}", f"nghost={self.nghost}",
             f"nx={self.nx}", f"ny={self.ny}", f"stencil={self.stencil}", f"cfl={self.cfl!r}",
             f"dt={self.dt!r}", f"cst_dt={self.cst_dt}", f"dt_on_even_cycles={self.dt_on_even_cycles}",
             f"max_cycles={self.max_cycles}", f"max_time={self.max_time!r}"]
        return a


def make_params(case: Case, L: C.CDLL | None = None) -> OParams:
    L = L or lib()
    p = OParams()
    L.o_params_defaults(C.byref(p))
    p.test = TESTS[case.test]
    p.scheme = SCHEMES[case.scheme]
    p.projection = PROJECTIONS[case.projection]
    p.limiter = LIMITERS[case.limiter]
    p.axis_splitting = SPLITTINGS[case.splitting]
    p.nb_ghosts = case.nghost
    p.nx, p.ny = case.nx, case.ny
    p.stencil_width = case.stencil
    p.cfl = case.cfl
    p.Dt = case.dt
    p.cst_dt = case.cst_dt
    p.dt_on_even_cycles = case.dt_on_even_cycles
    p.max_cycles = case.max_cycles
    p.max_time = case.max_time
    p.test_option = case.test_option
    L.o_params_init(C.byref(p))
    return p


class OracleState:
    """The 16 solver arrays as numpy buffers plus the ctypes view the oracle reads."""

    def __init__(self, p: OParams):
        n = p.nb_cells
        self.arrays = {name: np.zeros(n, dtype=np.float64) for name in ARRAY_NAMES}
        self.data = OData(*[a.ctypes.data_as(C.POINTER(C.c_double)) for a in self.arrays.values()])

    def __getitem__(self, k: str) -> np.ndarray:
        return self.arrays[k]


def run(case: Case, fast: bool = False, L: C.CDLL | None = None):
    """init_test + time_loop.  Returns (params, state, status, seconds)."""
    L = L or lib(fast)
    p = make_params(case, L)
    if not L.o_params_check(C.byref(p)):
        raise ValueError(f"invalid parameters for {case}")
    st = OracleState(p)
    L.o_init_test_p(C.byref(p), C.byref(st.data), 0)
    status = C.c_int(0)
    secs = L.o_time_loop(C.byref(p), C.byref(st.data), C.byref(status))
    return p, st, status.value, secs


def real_cells(p: OParams, a: np.ndarray) -> np.ndarray:
    """View of the real (non-ghost) cells of a flat array, shape (ny, nx)."""
    g, R = p.nb_ghosts, p.row_length
    return a.reshape(p.col_length, R)[g:g + p.ny, g:g + p.nx]


def read_ref_dump(path: str) -> list[dict]:
    """Records written by oracle/ref_driver (see its header for the layout)."""
    recs = []
    with open(path, "rb") as f:
        raw = f.read()
    off = 0
    while off < len(raw):
        tag = raw[off:off + 32].split(b"\0", 1)[0].decode()
        off += 32
        cycle, axis, n, status = np.frombuffer(raw, dtype=np.int32, count=4, offset=off)
        off += 16
        cur, nxt, t, cdt = np.frombuffer(raw, dtype=np.float64, count=4, offset=off)
        off += 32
        arrs = np.frombuffer(raw, dtype=np.float64, count=16 * int(n), offset=off).reshape(16, int(n))
        off += 16 * int(n) * 8
        rec = {"tag": tag, "cycle": int(cycle), "axis": int(axis), "status": int(status),
               "current_cycle_dt": float(cur), "next_cycle_dt": float(nxt), "time": float(t),
               "cycle_dt": float(cdt)}
        rec.update({name: arrs[k].copy() for k, name in enumerate(ARRAY_NAMES)})
        recs.append(rec)
    return recs
