"""The drop-in C++ step API and command line (armon-kokkos_gb300/csrc/armon_2D.cpp, main_2D.cpp):
the reference's flags, text output, --compare step checkpoints and the per-stage path."""
import ctypes as C
import hashlib
import json
import os
import subprocess

import numpy as np
import pytest

import armon_gb300 as A
import oracle_lib as O
import text_io

CLI = os.path.join(os.path.dirname(A.LIB_PATH), "armon_gb300_2D")
GOLDEN = json.load(open(os.path.join(os.path.dirname(__file__), "golden", "golden.json")))


def run_cli(args, cwd):
    return subprocess.run([CLI] + args, cwd=cwd, capture_output=True, text=True, timeout=600)


def sha(a):
    return hashlib.sha256(np.ascontiguousarray(a).tobytes()).hexdigest()


def test_cli_usage_and_errors(tmp_path):
    r = run_cli(["--help"], tmp_path)
    assert r.returncode == 0 and "--cells Nx,Ny" in r.stdout
    assert run_cli(["--bogus", "1"], tmp_path).returncode == 1
    # GAD + second order needs 4 ghosts: Params::check rejects 3 (src/parameters.cpp:102-106)
    r = run_cli(["-s", "GAD", "--projection", "euler_2nd", "--nghost", "3", "--stencil", "4", "--verbose", "3"],
                tmp_path)
    assert r.returncode == 1 and "stencil width cannot be bigger" in r.stderr


@pytest.mark.gpu
@pytest.mark.parametrize("name,args", [
    ("cfg1_sod_godunov_100_symsplit", ["-t", "Sod", "-s", "Godunov", "--projection", "euler", "--cells", "100,100",
                                       "--cfl", "0.6", "--time", "0.2", "--splitting", "SequentialSym",
                                       "--cycle", "100000"]),
    ("ref_Sod_circ", ["-t", "Sod_circ", "-s", "GAD", "--limiter", "Minmod", "--projection", "euler_2nd",
                      "--cells", "100,100", "--nghost", "5", "--cycle", "1000"]),
])
def test_cli_output_matches_reference(tmp_path, name, args):
    g = GOLDEN["cases"][name]
    r = run_cli(args + ["--write-output", "1", "--precision", "17", "--output", "out", "--verbose", "2"], tmp_path)
    assert r.returncode == 0, r.stdout + r.stderr
    assert f"Cycles:     {g['cycles']}" in r.stdout
    p = O.make_params(O.Case(**g["case"]))
    fields = text_io.read_output(tmp_path / "out", p)
    for k in ("rho", "umat", "vmat", "pmat"):
        assert sha(fields[k]) == g["hashes"][k], k


@pytest.mark.gpu
def test_cli_compare_mode_against_oracle_step_files(tmp_path):
    """--compare 1 replays the stage sequence and diffs every stage with files named
    <output>_<cycle>_<stage>_<axis> (src/armon_2D.cpp:255-284); here the oracle writes them."""
    case = O.Case(test="Sod_circ", scheme="GAD", projection="euler_2nd", nghost=5, nx=30, ny=20, max_cycles=2,
                  max_time=1.0)
    L = O.lib()
    p = O.make_params(case)
    st = O.OracleState(p)
    base = str(tmp_path / "ref")

    def dump(tag):
        name = f"{base}_{p.cycle:03d}_{tag}_{'X' if p.current_axis == 0 else 'Y'}"
        if tag == "time_step":
            open(name, "w").write(f"{p.current_cycle_dt!r}\n")
        else:
            text_io.write_output(name, p, st.arrays)

    L.o_init_test_p(C.byref(p), C.byref(st.data), 0)
    dump("init_test")
    p.cycle, p.time, p.current_cycle_dt, p.next_cycle_dt = 0, 0.0, 0.0, 0.0
    L.o_update_axis(C.byref(p), 0)
    L.o_update_EOS(C.byref(p), C.byref(st.data))
    dump("EOS_init")
    while p.time < p.max_time and p.cycle < p.max_cycles:
        L.o_time_step(C.byref(p), C.byref(st.data))
        dump("time_step")
        axes, facs = (C.c_int32 * 3)(), (C.c_double * 3)()
        for k in range(L.o_split_axes(C.byref(p), axes, facs)):
            L.o_update_axis(C.byref(p), axes[k])
            p.cycle_dt = p.current_cycle_dt * facs[k]
            for fn, tag in ((L.o_update_EOS, "EOS"), (L.o_boundary_conditions_p, "boundary_conditions"),
                            (L.o_numerical_fluxes, "numerical_fluxes"), (L.o_cell_update_p, "cell_update"),
                            (L.o_projection_remap, "projection_remap")):
                fn(C.byref(p), C.byref(st.data))
                dump(tag)
        p.time += p.current_cycle_dt
        p.cycle += 1
    r = run_cli(["-t", "Sod_circ", "-s", "GAD", "--projection", "euler_2nd", "--nghost", "5", "--cells", "30,20",
                 "--cycle", "2", "--time", "1.0", "--compare", "1", "--output", base, "--verbose", "3",
                 "--comparison-tolerance", "0"], tmp_path)
    assert r.returncode == 0, r.stdout + r.stderr
    assert "Difference" not in r.stdout and "differences" not in r.stdout, r.stdout[-2000:]
    assert not any(n.endswith("_diff") for n in os.listdir(tmp_path))


@pytest.mark.gpu
def test_cli_bizarrium_uses_stage_kernels(tmp_path):
    g = GOLDEN["cases"]["ref_Bizarrium"]
    r = run_cli(["-t", "Bizarrium", "-s", "GAD", "--projection", "euler_2nd", "--cells", "100,100", "--nghost", "5",
                 "--cycle", "1000", "--write-output", "1", "--precision", "17", "--output", "out", "--verbose", "3"],
                tmp_path)
    assert r.returncode == 0, r.stdout + r.stderr
    p = O.make_params(O.Case(**g["case"]))
    fields = text_io.read_output(tmp_path / "out", p)
    po, st, _, _ = O.run(O.Case(**g["case"]))
    assert po.cycle == g["cycles"]
    for k in ("rho", "pmat"):
        ref = O.real_cells(po, st[k])
        assert np.abs(fields[k] - ref).max() <= 1e-9 * np.abs(ref).max(), k


@pytest.mark.gpu
def test_cli_verbose_conservation_lines(tmp_path):
    # a square domain: the reference's conservation_vars uses ds = dx*dx of the current axis
    # (src/kernels/reductions.cpp:38), so on dx != dy its own |dM| line jumps by (dy/dx)^2
    r = run_cli(["-t", "Sod", "-s", "GAD", "--projection", "euler_2nd", "--nghost", "5", "--cells", "64,64",
                 "--cycle", "12", "--verbose", "1"], tmp_path)
    assert r.returncode == 0, r.stderr
    lines = [ln for ln in r.stdout.splitlines() if ln.startswith("Cycle =")]
    assert len(lines) == 12
    # |dM| stays at round-off (mass is conserved by the scheme)
    dm = [float(ln.split("|ΔM| =")[1].split("%")[0]) for ln in lines]
    assert max(dm) < 1e-10
