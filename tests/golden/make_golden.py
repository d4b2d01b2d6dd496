"""Generate the golden fixtures that pin the oracle to the reference.

Runs the reference's own armon_2D step API, compiled from its unchanged sources against the
project's Kokkos API shim (oracle/Makefile target `ref`, driver oracle/ref_driver.cpp), on the
cases below and writes:

  golden.json      per case: the solver parameters, cycle count, final dt / time (as exact hex
                   floats), the conservation sums, and a SHA-256 per field over the real cells
                   (rho, umat, vmat, Emat, pmat, cmat); for the stage case, one SHA-256 per array
                   (all cells, ghosts included) after every stage of the first two cycles;
  fields_*.npz     the real-cell fields of a few small cases, for readable diffs.

The reference tree is only needed to regenerate the fixtures: python tests/golden/make_golden.py
compiles the tree at $ARMON_REF, else the copy that `make -C oracle stage` puts in baseline/_ref.
The tests only read the fixtures.
"""
from __future__ import annotations

import hashlib
import json
import os
import subprocess
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, os.path.dirname(HERE))
import oracle_lib as O  # noqa: E402

FIELDS = ["rho", "umat", "vmat", "Emat", "pmat", "cmat"]


def ref_cases() -> dict[str, O.Case]:
    """name -> Case.  The reference parameters of tests/reference.cpp:33-64 and the option grid."""
    ref = dict(scheme="GAD", projection="euler_2nd", limiter="Minmod", splitting="Sequential",
               nghost=5, nx=100, ny=100, max_cycles=1000)
    cases = {
        # configuration 1 of the benchmark: Sod, Godunov + first-order remap, CFL 0.6, t = 0.2
        "cfg1_sod_godunov_100_symsplit": O.Case(test="Sod", scheme="Godunov", projection="euler",
                                                splitting="SequentialSym", nx=100, ny=100, cfl=0.6,
                                                max_time=0.2, max_cycles=100000),
        "cfg1_sod_godunov_100_seq": O.Case(test="Sod", scheme="Godunov", projection="euler",
                                           splitting="Sequential", nx=100, ny=100, cfl=0.6,
                                           max_time=0.2, max_cycles=100000),
        # tests/armon_2D_tests.cpp:205-243 (cycle counts 45 / 45 / 43 / 76 / 568)
        "ref_Sod": O.Case(test="Sod", **ref),
        "ref_Sod_y": O.Case(test="Sod_y", **ref),
        "ref_Sod_circ": O.Case(test="Sod_circ", **ref),
        "ref_Sedov": O.Case(test="Sedov", **ref),
        "ref_Bizarrium": O.Case(test="Bizarrium", **ref),
        # tests/armon_2D_tests.cpp:61-80: the rectangular default parameters
        "rect_sod_100x5": O.Case(test="Sod", scheme="GAD", projection="euler_2nd", limiter="Minmod",
                                 nghost=5, nx=100, ny=5, max_cycles=100),
        # option grid on ragged sizes
        "strang_superbee_37x23": O.Case(test="Sod_circ", scheme="GAD", projection="euler_2nd",
                                        limiter="Superbee", splitting="Strang", nghost=4, nx=37, ny=23,
                                        max_cycles=30, max_time=1.0),
        "symsplit_gad_euler1_48x31": O.Case(test="Sod_circ", scheme="GAD", projection="euler",
                                            splitting="SequentialSym", nghost=3, nx=48, ny=31,
                                            max_cycles=40, max_time=1.0),
        "nolimiter_xonly_64x8": O.Case(test="Sod", scheme="GAD", projection="euler_2nd", limiter="None",
                                       splitting="X_only", nghost=4, nx=64, ny=8, max_cycles=25),
        "yonly_sody_8x64": O.Case(test="Sod_y", scheme="GAD", projection="euler_2nd", splitting="Y_only",
                                  nghost=4, nx=8, ny=64, max_cycles=25),
        "godunov_euler2_33x33": O.Case(test="Sod_circ", scheme="Godunov", projection="euler_2nd",
                                       nghost=3, nx=33, ny=33, max_cycles=30, max_time=1.0),
        "cstdt_sedov_40x40": O.Case(test="Sedov", scheme="GAD", projection="euler_2nd", nghost=4,
                                    nx=40, ny=40, cst_dt=1, dt=0.002, max_cycles=30),
        "dt_even_sod_circ_50x30": O.Case(test="Sod_circ", scheme="GAD", projection="euler_2nd", nghost=5,
                                         nx=50, ny=30, dt_on_even_cycles=1, max_cycles=30, max_time=1.0),
        "wide_ghosts_stencil_sod_60x20": O.Case(test="Sod", scheme="GAD", projection="euler_2nd", nghost=7,
                                                stencil=6, nx=60, ny=20, max_cycles=30, max_time=1.0),
        "sod_circ_gad_256_cfl06": O.Case(test="Sod_circ", scheme="GAD", projection="euler_2nd", nghost=5,
                                         nx=256, ny=256, cfl=0.6, max_cycles=20, max_time=1e9),
    }
    # the benchmark's circular Sod at radius 0.2 (configuration 2 shrunk): the reference's init_test
    # hard-codes radius 0.3, so ref_driver re-labels the cells outside 0.2 (its radius2 option)
    for name, (nx, ny, cyc) in {"sod_circ_r02_gad_160x96": (160, 96, 12), "sod_circ_r02_gad_512": (512, 512, 30)}.items():
        cases[name] = O.Case(test="Sod_circ", scheme="GAD", projection="euler_2nd", nghost=5, nx=nx, ny=ny,
                             cfl=0.6, max_cycles=cyc, max_time=1e9, test_option=0.04)
    # tests/armon_2D_tests.cpp:246-275: 400 cycles, max_time 1e4, conservation to 1e-12
    for t in ("Sod", "Sod_y", "Sod_circ", "Sedov"):
        c = dict(ref)
        c.update(max_cycles=400, max_time=1e4)
        cases[f"conservation_{t}"] = O.Case(test=t, **c)
    return cases


STAGE_CASE = ("stages_sod_circ_24x16", O.Case(test="Sod_circ", scheme="GAD", projection="euler_2nd",
                                              limiter="Minmod", splitting="Sequential", nghost=5,
                                              nx=24, ny=16, max_cycles=2, max_time=1.0))
FIELD_CASES = ("rect_sod_100x5", "strang_superbee_37x23", "symsplit_gad_euler1_48x31")


def sha(a: np.ndarray) -> str:
    return hashlib.sha256(np.ascontiguousarray(a).tobytes()).hexdigest()


def field_hashes(p: O.OParams, rec: dict) -> dict[str, str]:
    return {k: sha(O.real_cells(p, rec[k])) for k in FIELDS}


def run_ref(case: O.Case, out: str, extra: list[str] | None = None) -> tuple[list[dict], str]:
    env = dict(os.environ, OMP_NUM_THREADS="1")
    if case.test == "Sod_circ" and case.test_option > 0:
        extra = (extra or []) + [f"radius2={case.test_option!r}"]
    r = subprocess.run([os.path.join(ROOT, "oracle", "_ref", "ref_driver"), out] + case.driver_args()
                       + (extra or []), check=True, capture_output=True, text=True, env=env)
    return O.read_ref_dump(out), r.stdout


BORDER_CASE = O.Case(test="Sod_circ", scheme="GAD", projection="euler_2nd", nghost=5, nx=20, ny=12)


def read_border_records(path: str) -> tuple[list[dict], dict]:
    """The border records of ref_driver's border_dump mode, then its final state record."""
    raw = open(path, "rb").read()
    off, sides = 0, []
    while raw[off:off + 32].split(b"\0", 1)[0].decode().startswith("border_"):
        tag = raw[off:off + 32].split(b"\0", 1)[0].decode()
        hdr = np.frombuffer(raw, dtype=np.int64, count=9, offset=off + 32)
        n = int(hdr[8])
        vals = np.frombuffer(raw, dtype=np.float64, count=n, offset=off + 32 + 72).copy()
        sides.append({"tag": tag, "range": [int(hdr[0]), int(hdr[1])],
                      "inner": [int(x) for x in hdr[2:6]], "side_length": int(hdr[6]), "nghost": int(hdr[7]),
                      "values": vals})
        off += 32 + 72 + 8 * n
    tmp = path + ".final"
    with open(tmp, "wb") as f:
        f.write(raw[off:])
    final = O.read_ref_dump(tmp)[0]
    os.remove(tmp)
    return sides, final


def border_fixture(tmp: str) -> dict:
    """read_border_array / write_border_array (src/kernels/halo_exchange.cpp:39-92) of the
    reference on the four borders of a 20x12 domain with 5 ghosts (ref_driver border_dump)."""
    subprocess.run([os.path.join(ROOT, "oracle", "_ref", "ref_driver"), tmp] + BORDER_CASE.driver_args()
                   + ["border_dump=1"], check=True, capture_output=True, text=True)
    sides, final = read_border_records(tmp)
    np.savez_compressed(os.path.join(HERE, "borders_20x12.npz"), **{s["tag"]: s["values"] for s in sides})
    return {"case": BORDER_CASE.__dict__,
            "sides": [{k: (sha(v) if k == "values" else v) for k, v in s.items()} for s in sides],
            "final_hashes": {k: sha(final[k]) for k in ("rho", "umat", "vmat", "pmat", "cmat", "gmat", "Emat")}}


def main() -> None:
    ref_dir = os.environ.get("ARMON_REF", os.path.join(ROOT, "baseline", "_ref"))
    if not os.path.isdir(os.path.join(ref_dir, "src", "kernels")):
        raise SystemExit(f"no reference tree at {ref_dir}: set ARMON_REF or run make -C oracle stage")
    subprocess.run(["make", "-C", os.path.join(ROOT, "oracle"), "ref", f"REF={ref_dir}", "-j8"],
                   check=True, capture_output=True)
    gold: dict = {"cases": {}, "stages": {}}
    tmp = os.path.join(ROOT, "oracle", "_ref", "golden_tmp.bin")
    for name, case in ref_cases().items():
        recs, stdout = run_ref(case, tmp)
        init, final = recs[0], recs[-1]
        p = O.make_params(case)
        kv = dict(tok.split("=") for tok in stdout.split())
        # The Sedov radius comes from libm's hypot on the host that made the fixtures; record it so
        # that the fixtures do not depend on another host's libm.
        topt = float.fromhex(kv["test_option"])
        if case.test == "Sedov" and case.test_option == 0:
            case.test_option = topt
        gold["cases"][name] = {
            "case": case.__dict__,
            "cycles": final["cycle"],
            "next_cycle_dt": final["next_cycle_dt"].hex(),
            "current_cycle_dt": final["current_cycle_dt"].hex(),
            "time": final["time"].hex(),
            "mass": float(kv["mass"]).hex(),
            "energy": float(kv["energy"]).hex(),
            "reference_test_option": topt.hex(),
            "init_hashes": field_hashes(p, init),
            "hashes": field_hashes(p, final),
        }
        if name in FIELD_CASES:
            np.savez_compressed(os.path.join(HERE, f"fields_{name}.npz"),
                                **{k: O.real_cells(p, final[k]) for k in FIELDS})
        print(name, final["cycle"], final["next_cycle_dt"])
    name, case = STAGE_CASE
    recs, _ = run_ref(case, tmp, ["stage_dump_cycles=2"])
    gold["stages"] = {"name": name, "case": case.__dict__, "records": [
        {"tag": r["tag"], "cycle": r["cycle"], "axis": r["axis"],
         "current_cycle_dt": r["current_cycle_dt"].hex(), "next_cycle_dt": r["next_cycle_dt"].hex(),
         "cycle_dt": r["cycle_dt"].hex(),
         "hashes": {k: sha(r[k]) for k in O.ARRAY_NAMES}} for r in recs]}
    gold["borders"] = border_fixture(tmp)
    os.remove(tmp)
    with open(os.path.join(HERE, "golden.json"), "w") as f:
        json.dump(gold, f, indent=1, sort_keys=True)


if __name__ == "__main__":
    main()
