"""Python access to libarmon_gb300.so (the GB300 Armon time step) through its C ABI.

This module is a thin ctypes layer over include/armon_gb300.h and include/armon_kernels.h: the
solver, the parameter block and the reference's kernel entry points.  All the compute runs in the
CUDA library; if the library is missing, importing the bindings raises.
"""
from __future__ import annotations

import ctypes as C
import os
from dataclasses import dataclass

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libarmon_gb300.so")

TESTS = {"Sod": 0, "Sod_y": 1, "Sod_circ": 2, "Bizarrium": 3, "Sedov": 4}
SCHEMES = {"Godunov": 0, "GAD": 1}
PROJECTIONS = {"none": 0, "euler": 1, "euler_2nd": 2}
LIMITERS = {"None": 0, "Minmod": 1, "Superbee": 2}
SPLITTINGS = {"Sequential": 0, "SequentialSym": 1, "Strang": 2, "X_only": 3, "Y_only": 4}
ARRAYS = ["x", "y", "rho", "umat", "vmat", "Emat", "pmat", "cmat", "gmat", "ustar", "pstar",
          "work_array_1", "work_array_2", "work_array_3", "work_array_4", "domain_mask"]

OK, ERR_INVALID_DT, ERR_PARAMS, ERR_CUDA, ERR_UNSUPPORTED, ERR_NOMEM, ERR_STATE = range(7)


class ArmonError(RuntimeError):
    def __init__(self, code: int, msg: str):
        super().__init__(f"armon error {code}: {msg}")
        self.code = code


class Params(C.Structure):
    """armon_params (include/armon_gb300.h): the reference's Params fields."""
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


class SolverOpts(C.Structure):
    _fields_ = [("precision", C.c_int32), ("cycles_per_graph", C.c_int32), ("seg_len", C.c_int32),
                ("block_lines", C.c_int32), ("materialize_eos", C.c_int32), ("unit_order", C.c_int32),
                ("split_pass", C.c_int32), ("reuse", C.c_int32)]


class BatchOpts(C.Structure):
    _fields_ = [("precision", C.c_int32), ("cycles_per_graph", C.c_int32), ("block_lines", C.c_int32),
                ("seg_len", C.c_int32), ("memory_budget", C.c_int64), ("waves", C.c_int32), ("unit_order", C.c_int32),
                ("split_pass", C.c_int32), ("reuse", C.c_int32)]


class SodInterface(C.Structure):
    """armon_sod_interface: a planar (shape 0) or circular (shape 1) Sod interface made on the device."""
    _fields_ = [("shape", C.c_int32), ("reserved", C.c_int32), ("cx", C.c_double), ("cy", C.c_double),
                ("nx", C.c_double), ("ny", C.c_double), ("offset", C.c_double), ("r2", C.c_double),
                ("rho_high", C.c_double), ("p_high", C.c_double), ("rho_low", C.c_double), ("p_low", C.c_double)]


class ServerOpts(C.Structure):
    _fields_ = [("memory_budget", C.c_int64), ("cycles_per_step", C.c_int32), ("block_lines", C.c_int32),
                ("max_inflight_cells", C.c_int64), ("waves", C.c_int32), ("reserved", C.c_int32)]


class RequestInfo(C.Structure):
    """armon_server_request."""
    _fields_ = [("status", C.c_int32), ("precision", C.c_int32), ("cycle", C.c_int32), ("nx", C.c_int32),
                ("ny", C.c_int32), ("pad", C.c_int32), ("time", C.c_double), ("t_submit", C.c_double),
                ("t_admit", C.c_double), ("t_done", C.c_double), ("bytes", C.c_int64)]


REQ_QUEUED, REQ_RUNNING, REQ_DONE, REQ_FAILED = 0, 1, 2, 3


class Range(C.Structure):
    _fields_ = [("start", C.c_int64), ("end", C.c_int64)]


class InnerRange1D(C.Structure):
    _fields_ = [("start", C.c_int64), ("step", C.c_int64)]


class InnerRange2D(C.Structure):
    _fields_ = [("main_range_start", C.c_int64), ("main_range_step", C.c_int64),
                ("row_range_start", C.c_int64), ("row_range_length", C.c_uint64)]


class View(C.Structure):
    """armon_view: a device array of doubles with an optional label."""
    _fields_ = [("data", C.c_void_p), ("size", C.c_int64), ("label", C.c_char_p)]


_lib: C.CDLL | None = None


def lib() -> C.CDLL:
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB_PATH):
        raise ImportError(f"{LIB_PATH} is missing: build it with armon-kokkos_gb300/build.py "
                          "(there is no CPU fallback)")
    L = C.CDLL(LIB_PATH)
    P, S = C.POINTER(Params), C.c_void_p
    L.armon_last_error.restype = C.c_char_p
    L.armon_params_defaults.argtypes = [P]
    L.armon_params_init.argtypes = [P]
    L.armon_params_check.argtypes = [P]
    L.armon_min_ghosts.argtypes = [P]
    L.armon_solver_opts_default.argtypes = [C.POINTER(SolverOpts)]
    L.armon_solver_create.argtypes = [P, C.POINTER(SolverOpts), C.c_void_p, C.POINTER(C.c_void_p)]
    L.armon_solver_destroy.argtypes = [S]
    L.armon_solver_destroy.restype = None
    for fn in ("armon_solver_init_test", "armon_solver_begin_loop"):
        getattr(L, fn).argtypes = [S]
    L.armon_solver_run.argtypes = [S, C.c_int]
    L.armon_solver_enqueue_cycles.argtypes = [S, C.c_int]
    L.armon_solver_sync_params.argtypes = [S, P, C.POINTER(C.c_int32)]
    L.armon_solver_download.argtypes = [S, C.c_int, C.c_void_p]
    L.armon_solver_upload.argtypes = [S, C.c_int, C.c_void_p]
    L.armon_solver_device_array.argtypes = [S, C.c_int]
    L.armon_solver_device_array.restype = C.c_void_p
    L.armon_solver_conservation.argtypes = [S, C.POINTER(C.c_double), C.POINTER(C.c_double)]
    L.armon_solver_kernel_launches.argtypes = [S]
    L.armon_solver_kernel_launches.restype = C.c_int64
    L.armon_solver_tiling.argtypes = [S, C.POINTER(C.c_int32), C.POINTER(C.c_int32)]
    L.armon_solver_block_lines.argtypes = [S]
    L.armon_solver_tuning.argtypes = [S]
    L.armon_solver_measurement_cycles.argtypes = [S]
    L.armon_solver_measurement_cycles.restype = C.c_int64
    L.armon_solver_split_pass.argtypes = [S]
    L.armon_tiling_cache_clear.argtypes = []
    L.armon_tiling_cache_clear.restype = None
    L.armon_solve_host.argtypes = [P, C.POINTER(SolverOpts), C.POINTER(C.c_void_p), C.POINTER(C.c_void_p), P]
    B = C.c_void_p
    L.armon_batch_opts_default.argtypes = [C.POINTER(BatchOpts)]
    L.armon_batch_create.argtypes = [C.POINTER(BatchOpts), C.c_void_p, C.POINTER(C.c_void_p)]
    L.armon_batch_destroy.argtypes = [B]
    L.armon_batch_destroy.restype = None
    L.armon_batch_domain_bytes.argtypes = [P, C.c_int32]
    L.armon_batch_domain_bytes.restype = C.c_int64
    L.armon_batch_add.argtypes = [B, P, C.POINTER(C.c_void_p), C.POINTER(C.c_int32)]
    L.armon_batch_add_sod.argtypes = [B, P, C.POINTER(SodInterface), C.POINTER(C.c_int32)]
    L.armon_batch_set_seg_len.argtypes = [B, C.c_int32, C.c_int32]
    L.armon_batch_enqueue_cycles.argtypes = [B, C.c_int32]
    L.armon_batch_run.argtypes = [B, C.c_int32, C.POINTER(C.c_int32)]
    L.armon_batch_poll.argtypes = [B, C.POINTER(C.c_int32)]
    L.armon_batch_domain_state.argtypes = [B, C.c_int32, P, C.POINTER(C.c_int32)]
    L.armon_batch_domain_done.argtypes = [B, C.c_int32]
    L.armon_batch_download.argtypes = [B, C.c_int32, C.c_int, C.c_void_p]
    L.armon_batch_remove.argtypes = [B, C.c_int32]
    L.armon_batch_schedule.argtypes = [B, C.POINTER(C.c_int32), C.POINTER(C.c_int32)]
    L.armon_batch_size.argtypes = [B]
    L.armon_batch_bytes_in_use.argtypes = [B]
    L.armon_batch_bytes_in_use.restype = C.c_int64
    L.armon_batch_kernel_launches.argtypes = [B]
    L.armon_batch_kernel_launches.restype = C.c_int64
    V = C.c_void_p
    L.armon_server_opts_default.argtypes = [C.POINTER(ServerOpts)]
    L.armon_server_opts_default.restype = None
    L.armon_server_create.argtypes = [C.POINTER(ServerOpts), C.POINTER(C.c_void_p)]
    L.armon_server_destroy.argtypes = [V]
    L.armon_server_destroy.restype = None
    L.armon_server_submit.argtypes = [V, P, C.c_int32, C.POINTER(SodInterface), C.POINTER(C.c_int64)]
    L.armon_server_step.argtypes = [V, C.POINTER(C.c_int32), C.POINTER(C.c_int32)]
    L.armon_server_next_done.argtypes = [V, C.POINTER(C.c_int64)]
    L.armon_server_request_info.argtypes = [V, C.c_int64, C.POINTER(RequestInfo)]
    L.armon_server_download.argtypes = [V, C.c_int64, C.c_int, C.c_void_p]
    L.armon_server_release.argtypes = [V, C.c_int64]
    L.armon_server_bytes_in_use.argtypes = [V]
    L.armon_server_bytes_in_use.restype = C.c_int64
    L.armon_server_kernel_launches.argtypes = [V]
    L.armon_server_kernel_launches.restype = C.c_int64
    L.dt_CFL.restype = C.c_double
    L.idx_size.restype = C.c_int
    L.is_uidx_signed.restype = C.c_bool
    L.flt_size.restype = C.c_int
    L.armon_kernels_set_stream.argtypes = [C.c_void_p]
    L.armon_kernels_set_stream.restype = None
    _lib = L
    return L


def check(rc: int) -> None:
    if rc != OK:
        raise ArmonError(rc, lib().armon_last_error().decode())


@dataclass
class Case:
    """A configuration in the reference's CLI vocabulary (src/main_2D.cpp:9-38)."""
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


def make_params(case: Case) -> Params:
    L = lib()
    p = Params()
    L.armon_params_defaults(C.byref(p))
    p.test = TESTS[case.test]
    p.scheme = SCHEMES[case.scheme]
    p.projection = PROJECTIONS[case.projection]
    p.limiter = LIMITERS[case.limiter]
    p.axis_splitting = SPLITTINGS[case.splitting]
    p.nb_ghosts, p.nx, p.ny = case.nghost, case.nx, case.ny
    p.stencil_width = case.stencil
    p.cfl, p.Dt = case.cfl, case.dt
    p.cst_dt, p.dt_on_even_cycles = case.cst_dt, case.dt_on_even_cycles
    p.max_cycles, p.max_time = case.max_cycles, case.max_time
    p.test_option = case.test_option
    L.armon_params_init(C.byref(p))
    return p


class Solver:
    """A domain resident in HBM with the fused time loop (armon_solver_* of include/armon_gb300.h)."""

    def __init__(self, params: Params | Case, precision: int = 64, stream: int | None = None,
                 cycles_per_graph: int = 16, seg_len: int = 0, block_lines: int = 0, materialize_eos: int = -1,
                 unit_order: int = 0, split_pass: int = 0, reuse: int = 0):
        L = lib()
        self.params = make_params(params) if isinstance(params, Case) else params
        o = SolverOpts()
        L.armon_solver_opts_default(C.byref(o))
        o.precision = precision
        o.cycles_per_graph = cycles_per_graph
        o.seg_len = seg_len
        o.block_lines = block_lines
        o.materialize_eos = materialize_eos
        o.unit_order = unit_order
        o.split_pass = split_pass
        o.reuse = reuse
        self.opts = o
        h = C.c_void_p()
        check(L.armon_solver_create(C.byref(self.params), C.byref(o), C.c_void_p(stream or 0), C.byref(h)))
        self._h = h

    def close(self) -> None:
        if getattr(self, "_h", None):
            lib().armon_solver_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def init_test(self) -> None:
        check(lib().armon_solver_init_test(self._h))

    def begin_loop(self) -> None:
        check(lib().armon_solver_begin_loop(self._h))

    def run(self, cycle_limit: int = 0) -> None:
        check(lib().armon_solver_run(self._h, cycle_limit))

    def enqueue_cycles(self, n: int) -> None:
        check(lib().armon_solver_enqueue_cycles(self._h, n))

    def state(self) -> tuple[Params, int]:
        p = Params()
        st = C.c_int32()
        check(lib().armon_solver_sync_params(self._h, C.byref(p), C.byref(st)))
        return p, st.value

    def download(self, name: str) -> np.ndarray:
        a = np.empty(self.params.nb_cells, dtype=np.float64)
        check(lib().armon_solver_download(self._h, ARRAYS.index(name), a.ctypes.data))
        return a

    def upload(self, name: str, a: np.ndarray) -> None:
        a = np.ascontiguousarray(a, dtype=np.float64)
        assert a.size == self.params.nb_cells
        check(lib().armon_solver_upload(self._h, ARRAYS.index(name), a.ctypes.data))

    def device_array(self, name: str) -> int:
        return lib().armon_solver_device_array(self._h, ARRAYS.index(name)) or 0

    def conservation(self) -> tuple[float, float]:
        m, e = C.c_double(), C.c_double()
        check(lib().armon_solver_conservation(self._h, C.byref(m), C.byref(e)))
        return m.value, e.value

    @property
    def kernel_launches(self) -> int:
        return int(lib().armon_solver_kernel_launches(self._h))

    def tiling(self) -> tuple[tuple[int, int], tuple[int, int]]:
        """((seg_len X, seg_len Y), (blocks X, blocks Y)) of the fused pass."""
        sl, nb = (C.c_int32 * 2)(), (C.c_int32 * 2)()
        check(lib().armon_solver_tiling(self._h, sl, nb))
        return (sl[0], sl[1]), (nb[0], nb[1])

    def block_lines(self) -> int:
        """Lines (threads) per block of the fused pass."""
        return int(lib().armon_solver_block_lines(self._h))

    def tuning(self) -> bool:
        """True while the time loop is still timing candidate tilings on its cycles."""
        return lib().armon_solver_tuning(self._h) == 1

    def measurement_cycles(self) -> int:
        """Cycles run so far with a candidate tiling of the tiling measurement."""
        return int(lib().armon_solver_measurement_cycles(self._h))

    def split_pass(self) -> bool:
        """True when the axis passes run split (face launch + cell launch), False when fused."""
        return lib().armon_solver_split_pass(self._h) == 1


def tiling_cache_clear() -> None:
    """Forgets the tilings measured so far in this process (armon_tiling_cache_clear)."""
    lib().armon_tiling_cache_clear()


def real_cells(p: Params, a: np.ndarray) -> np.ndarray:
    """(ny, nx) view of the real cells of a flat array in the reference's layout."""
    g, R = p.nb_ghosts, p.row_length
    return a.reshape(p.col_length, R)[g:g + p.ny, g:g + p.nx]


def solve_host(case: Case | Params, inputs: dict[str, np.ndarray] | None = None, precision: int = 64,
               cycles_per_graph: int = 16) -> tuple[Params, dict[str, np.ndarray]]:
    """armon_solve_host: the end-to-end call with host buffers (H2D, time loop, D2H)."""
    L = lib()
    p = make_params(case) if isinstance(case, Case) else case
    o = SolverOpts()
    L.armon_solver_opts_default(C.byref(o))
    o.precision = precision
    o.cycles_per_graph = cycles_per_graph
    ins = (C.c_void_p * 4)()
    keep = []
    if inputs:
        for k, name in enumerate(("rho", "umat", "vmat", "Emat")):
            if name in inputs:
                a = np.ascontiguousarray(inputs[name], dtype=np.float64)
                keep.append(a)
                ins[k] = a.ctypes.data
    outs = {name: np.empty(p.nb_cells, dtype=np.float64) for name in ("rho", "umat", "vmat", "Emat", "pmat")}
    outp = (C.c_void_p * 5)(*[outs[n].ctypes.data for n in ("rho", "umat", "vmat", "Emat", "pmat")])
    final = Params()
    check(L.armon_solve_host(C.byref(p), C.byref(o), ins if inputs else None, outp, C.byref(final)))
    return final, outs


class Batch:
    """Many independent domains advanced together (armon_batch_* of include/armon_gb300.h)."""

    def __init__(self, precision: int = 64, stream: int | None = None, cycles_per_graph: int = 8,
                 block_lines: int = 128, seg_len: int = 0, memory_budget: int = 0, waves: int = 0,
                 unit_order: int = 0, split_pass: int = 0, reuse: int = 0):
        L = lib()
        o = BatchOpts()
        L.armon_batch_opts_default(C.byref(o))
        o.precision, o.cycles_per_graph, o.block_lines = precision, cycles_per_graph, block_lines
        o.seg_len, o.memory_budget, o.waves, o.unit_order = seg_len, memory_budget, waves, unit_order
        o.split_pass = split_pass
        o.reuse = reuse
        h = C.c_void_p()
        check(L.armon_batch_create(C.byref(o), C.c_void_p(stream or 0), C.byref(h)))
        self._h = h
        self.precision = precision
        self.params: dict[int, Params] = {}

    def close(self) -> None:
        if getattr(self, "_h", None):
            lib().armon_batch_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def add(self, params: Params | Case, init: dict[str, np.ndarray] | None = None) -> int:
        p = make_params(params) if isinstance(params, Case) else params
        arr = None
        keep = []
        if init is not None:
            arr = (C.c_void_p * 4)()
            for k, name in enumerate(("rho", "umat", "vmat", "Emat")):
                a = np.ascontiguousarray(init[name], dtype=np.float64)
                assert a.size == p.nb_cells
                keep.append(a)
                arr[k] = a.ctypes.data
        i = C.c_int32()
        check(lib().armon_batch_add(self._h, C.byref(p), arr, C.byref(i)))
        self.params[i.value] = p
        return i.value

    def add_sod(self, params: Params | Case, sod: SodInterface) -> int:
        """Adds a domain initialised on the device with a Sod interface (armon_batch_add_sod)."""
        p = make_params(params) if isinstance(params, Case) else params
        i = C.c_int32()
        check(lib().armon_batch_add_sod(self._h, C.byref(p), C.byref(sod), C.byref(i)))
        self.params[i.value] = p
        return i.value

    def set_seg_len(self, i: int, seg_len: int) -> None:
        check(lib().armon_batch_set_seg_len(self._h, i, seg_len))

    def enqueue_cycles(self, n: int) -> None:
        check(lib().armon_batch_enqueue_cycles(self._h, n))

    def run(self, cycle_limit: int = 0) -> int:
        r = C.c_int32()
        check(lib().armon_batch_run(self._h, cycle_limit, C.byref(r)))
        return r.value

    def poll(self) -> int:
        r = C.c_int32()
        check(lib().armon_batch_poll(self._h, C.byref(r)))
        return r.value

    def state(self, i: int) -> tuple[Params, int]:
        p = Params()
        st = C.c_int32()
        check(lib().armon_batch_domain_state(self._h, i, C.byref(p), C.byref(st)))
        return p, st.value

    def done(self, i: int) -> bool:
        return lib().armon_batch_domain_done(self._h, i) == 1

    def download(self, i: int, name: str) -> np.ndarray:
        a = np.empty(self.params[i].nb_cells, dtype=np.float64)
        check(lib().armon_batch_download(self._h, i, ARRAYS.index(name), a.ctypes.data))
        return a

    def remove(self, i: int) -> None:
        check(lib().armon_batch_remove(self._h, i))
        self.params.pop(i, None)

    def schedule(self) -> tuple[int, int]:
        """(block waves per launch in use, blocks of the current launch table)."""
        w, n = C.c_int32(), C.c_int32()
        check(lib().armon_batch_schedule(self._h, C.byref(w), C.byref(n)))
        return w.value, n.value

    @property
    def bytes_in_use(self) -> int:
        return int(lib().armon_batch_bytes_in_use(self._h))

    @property
    def kernel_launches(self) -> int:
        return int(lib().armon_batch_kernel_launches(self._h))


def domain_bytes(params: Params, precision: int = 64) -> int:
    return int(lib().armon_batch_domain_bytes(C.byref(params), precision))


class Server:
    """The request loop over batches (armon_server_* of include/armon_gb300.h)."""

    def __init__(self, memory_budget: int = 150_000_000_000, cycles_per_step: int = 8, block_lines: int = 128,
                 max_inflight_cells: int | None = None, waves: int = 0):
        L = lib()
        o = ServerOpts()
        L.armon_server_opts_default(C.byref(o))
        o.memory_budget, o.cycles_per_step, o.block_lines = memory_budget, cycles_per_step, block_lines
        if max_inflight_cells is not None:
            o.max_inflight_cells = max_inflight_cells
        o.waves = waves
        h = C.c_void_p()
        check(L.armon_server_create(C.byref(o), C.byref(h)))
        self._h = h
        self.params: dict[int, Params] = {}

    def close(self) -> None:
        if getattr(self, "_h", None):
            lib().armon_server_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def submit(self, params: Params | Case, precision: int = 64, sod: SodInterface | None = None) -> int:
        p = make_params(params) if isinstance(params, Case) else params
        r = C.c_int64()
        check(lib().armon_server_submit(self._h, C.byref(p), precision, C.byref(sod) if sod is not None else None,
                                         C.byref(r)))
        self.params[r.value] = p
        return r.value

    def step(self) -> tuple[int, int]:
        """One round; returns (requests running, requests waiting)."""
        a, b = C.c_int32(), C.c_int32()
        check(lib().armon_server_step(self._h, C.byref(a), C.byref(b)))
        return a.value, b.value

    def next_done(self) -> int | None:
        r = C.c_int64()
        return r.value if lib().armon_server_next_done(self._h, C.byref(r)) == 1 else None

    def info(self, req: int) -> RequestInfo:
        i = RequestInfo()
        check(lib().armon_server_request_info(self._h, req, C.byref(i)))
        return i

    def download(self, req: int, name: str) -> np.ndarray:
        a = np.empty(self.params[req].nb_cells, dtype=np.float64)
        check(lib().armon_server_download(self._h, req, ARRAYS.index(name), a.ctypes.data))
        return a

    def release(self, req: int) -> None:
        check(lib().armon_server_release(self._h, req))

    @property
    def bytes_in_use(self) -> int:
        return int(lib().armon_server_bytes_in_use(self._h))

    @property
    def kernel_launches(self) -> int:
        return int(lib().armon_server_kernel_launches(self._h))

