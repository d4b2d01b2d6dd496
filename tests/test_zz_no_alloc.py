"""dt_CFL_no_alloc: the CFL time step for callers that may not allocate device memory (hosts
that hand the whole GPU to their own memory pool, or time-critical loops that cannot afford
cudaMalloc's device-wide synchronisation).  It keeps its reduction scratch in a fixed array of
the library's device module; these tests check it against dt_CFL, which allocates, on the same
device arrays, on consecutive calls and on ranges of different lengths, and check its size
limit.  The file is collected last so that a stop-at-first-failure run has run everything else.
"""
import ctypes as C
import os
import subprocess
import sys
import textwrap

import numpy as np
import pytest

import armon_gb300 as A

pytestmark = pytest.mark.gpu

SIG = [C.c_void_p, C.c_void_p, C.c_double, C.c_double] + [C.c_void_p] * 4
MAX_INDICES = 32768 * 4096


def _lib():
    L = A.lib()
    for fn in (L.dt_CFL, L.dt_CFL_no_alloc):
        fn.argtypes = SIG
        fn.restype = C.c_double
    return L


def _device_state():
    torch = pytest.importorskip("torch")
    # a state a few cycles into a circular Sod run, then copied to torch device arrays
    case = A.Case(test="Sod_circ", scheme="GAD", projection="euler_2nd", nghost=5, nx=300, ny=200, cfl=0.6,
                  max_cycles=6, max_time=1e9, test_option=0.04)
    with A.Solver(case) as s:
        s.init_test()
        s.run()
        host = {k: s.download(k) for k in ("umat", "vmat", "cmat", "domain_mask")}
        p = s.params
    dev = {k: torch.from_numpy(v).cuda() for k, v in host.items()}
    torch.cuda.synchronize()
    return p, dev


def _views(dev):
    return [A.View(dev[k].data_ptr(), dev[k].numel(), k.encode()) for k in ("umat", "vmat", "cmat", "domain_mask")]


def _ranges(p, rows):
    # real_domain(p).iter1D() over the first `rows` real rows (src/ranges.cpp:5-11, src/kernels/indexing.cpp:82-88)
    begin = p.index_start
    end = p.index_start + (rows - 1) * p.row_length + p.nx - 1
    return A.Range(0, end - begin + 1), A.InnerRange1D(begin, 1)


def test_no_alloc_dt_matches_dt_cfl_on_consecutive_calls():
    L = _lib()
    p, dev = _device_state()
    views = _views(dev)
    dx, dy = p.domain_size[0] / p.nx, p.domain_size[1] / p.ny
    for rows in (p.ny, 7, p.ny):         # long, short, long: the shared array keeps the last call's partials
        rg, ir = _ranges(p, rows)
        expected = L.dt_CFL(C.byref(rg), C.byref(ir), dx, dy, *[C.byref(v) for v in views])
        assert np.isfinite(expected) and expected > 0
        for _ in range(2):
            got = L.dt_CFL_no_alloc(C.byref(rg), C.byref(ir), dx, dy, *[C.byref(v) for v in views])
            assert got == expected          # a min reduction: exact, whatever the order


def test_no_alloc_dt_rejects_ranges_beyond_its_scratch():
    L = _lib()
    messages = []
    HANDLER = C.CFUNCTYPE(None, C.c_char_p, C.c_char_p)

    def record(kernel, msg):
        messages.append((kernel.decode(), msg.decode()))

    cb = HANDLER(record)
    slot = C.c_void_p.in_dll(L, "raise_exception_handler")
    saved = slot.value
    slot.value = C.cast(cb, C.c_void_p).value
    try:
        # never dereferenced: the length check comes before any launch
        tiny = A.View(None, 1, None)
        rg, ir = A.Range(0, MAX_INDICES + 1), A.InnerRange1D(0, 1)
        L.dt_CFL_no_alloc(C.byref(rg), C.byref(ir), 1.0, 1.0, *[C.byref(tiny)] * 4)
    finally:
        slot.value = saved
    assert messages and messages[0][0] == "dt_CFL_no_alloc"
    assert "static scratch limit" in messages[0][1] and str(MAX_INDICES) in messages[0][1]


def test_no_alloc_dt_leaves_device_memory_untouched():
    """The property the entry point exists for, in a fresh process where nothing else of the
    library has allocated a reduction buffer: after one warm-up call (which may load the module and
    so reserve its fixed array), more calls leave the device's free memory exactly as it was."""
    here = os.path.dirname(os.path.abspath(__file__))
    code = textwrap.dedent(f"""
        import ctypes as C, sys
        sys.path[:0] = [{here!r}, {os.path.dirname(here)!r}, {os.path.join(os.path.dirname(here), "armon-kokkos_gb300")!r}]
        import torch
        import test_zz_no_alloc as T
        L = T._lib()
        p, dev = T._device_state()
        views = T._views(dev)
        dx, dy = p.domain_size[0] / p.nx, p.domain_size[1] / p.ny
        rg, ir = T._ranges(p, p.ny)
        args = (C.byref(rg), C.byref(ir), dx, dy, *[C.byref(v) for v in views])
        first = L.dt_CFL_no_alloc(*args)
        torch.cuda.synchronize()
        free0 = torch.cuda.mem_get_info()[0]
        vals = [L.dt_CFL_no_alloc(*args) for _ in range(5)]
        torch.cuda.synchronize()
        free1 = torch.cuda.mem_get_info()[0]
        assert all(v == first for v in vals), (first, vals)
        assert free1 == free0, (free0, free1)
        print("free bytes unchanged:", free0)
    """)
    r = subprocess.run([sys.executable, "-c", code], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stdout + r.stderr
