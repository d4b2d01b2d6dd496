"""Build libarmon_gb300.so (CUDA for sm_103a) in-tree with nvcc, translation units in parallel.

    python armon-kokkos_gb300/build.py            # build (skips up-to-date objects)
    python armon-kokkos_gb300/build.py --clean    # rebuild everything

All units are compiled with --fmad=false (no contraction, IEEE div/sqrt are nvcc's defaults),
which is what makes the FP64 kernels bit-exact with the reference's strict build, and the FP32
kernels independent of how the compiler fuses a given kernel.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(HERE, "armon_gb300", "libarmon_gb300.so")
CLI = os.path.join(HERE, "armon_gb300", "armon_gb300_2D")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
COMMON = ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "--extended-lambda",
          "-I" + os.path.join(ROOT, "include"), "-I" + CSRC]
# extra nvcc flags for tuning builds (e.g. -DARMON_SWEEP_MIN_BLOCKS=3); rebuild with --clean
EXTRA = os.environ.get("ARMON_NVCC_FLAGS", "").split()

# (source, extra flags)
UNITS = [
    ("sweep_f64.cu", ["--fmad=false"]),
    ("sweep_f32.cu", ["--fmad=false"]),
    ("sweep_split.cu", ["--fmad=false"]),
    ("abi_kernels.cu", ["--fmad=false"]),
    ("solver.cu", ["--fmad=false"]),
    ("batch.cu", ["--fmad=false"]),
    ("selftest.cu", ["--fmad=false"]),
    ("params.cpp", []),
    ("server.cpp", []),
    ("armon_2D.cpp", []),
]
CLI_SRC = "main_2D.cpp"


def nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found")


def _newer(obj: str, deps: list[str]) -> bool:
    if not os.path.exists(obj):
        return False
    t = os.path.getmtime(obj)
    return all(os.path.getmtime(d) <= t for d in deps)


def _headers() -> list[str]:
    hs = [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".cuh", ".h"))]
    inc = os.path.join(ROOT, "include")
    hs += [os.path.join(inc, f) for f in os.listdir(inc) if f.endswith(".h")]
    return hs


def _compile(src: str, flags: list[str], verbose: bool) -> str:
    obj = os.path.join(BUILD, os.path.basename(src) + ".o")
    path = os.path.join(CSRC, src)
    if _newer(obj, [path] + _headers() + [os.path.abspath(__file__)]):
        return obj
    lang = ["-x", "cu"] if src.endswith(".cu") else ["-x", "c++"]
    cmd = [nvcc()] + ARCH + COMMON + EXTRA + flags + lang + ["-c", path, "-o", obj]
    if verbose:
        cmd += ["-Xptxas", "-v"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"nvcc failed on {src}:\n{r.stdout}\n{r.stderr}")
    if verbose and r.stderr:
        sys.stderr.write(r.stderr)
    return obj


def build(clean: bool = False, verbose: bool = False) -> str:
    if clean and os.path.isdir(BUILD):
        shutil.rmtree(BUILD)
    os.makedirs(BUILD, exist_ok=True)
    with cf.ThreadPoolExecutor(max_workers=len(UNITS)) as ex:
        objs = list(ex.map(lambda u: _compile(u[0], u[1], verbose), UNITS))
    if not _newer(LIB, objs):
        cmd = [nvcc()] + ARCH + ["-shared", "-o", LIB] + objs + ["-lcudart_static", "-lrt", "-ldl", "-lpthread"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"link failed:\n{r.stdout}\n{r.stderr}")
    # the command line of the reference, linked against the library
    cli_obj = _compile(CLI_SRC, [], verbose)
    if not _newer(CLI, [cli_obj, LIB]):
        cmd = [nvcc()] + ARCH + ["-o", CLI, cli_obj, "-L" + os.path.dirname(LIB), "-larmon_gb300",
                                 "-Xlinker", "-rpath=$ORIGIN", "-lcudart_static", "-lrt", "-ldl", "-lpthread"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"link of {CLI_SRC} failed:\n{r.stdout}\n{r.stderr}")
    return LIB


if __name__ == "__main__":
    print(build(clean="--clean" in sys.argv, verbose="-v" in sys.argv))
