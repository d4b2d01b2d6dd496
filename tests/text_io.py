"""The reference's text dump format (src/io.cpp:10-74) for the tests: x, y, rho, umat, vmat, pmat
per cell, `precision` significant digits in scientific notation, one row of cells per block."""
import numpy as np

MAIN_VARS = ["x", "y", "rho", "umat", "vmat", "pmat"]


def write_output(path, p, arrays, precision=17, ghosts=False):
    g = p.nb_ghosts
    j0, j1 = (-g, p.ny + g) if ghosts else (0, p.ny)
    i0, i1 = (-g, p.nx + g) if ghosts else (0, p.nx)
    w = precision + 7
    with open(path, "w") as f:
        for j in range(j0, j1):
            for i in range(i0, i1):
                idx = p.index_start + j * p.row_length + i
                f.write(", ".join(f"{arrays[k][idx]:>{w}.{precision}e}" for k in MAIN_VARS) + "\n")
            f.write("\n")


def read_output(path, p):
    """(ny, nx) arrays of the six written fields (real cells)."""
    rows = [ln for ln in open(path).read().splitlines() if ln.strip()]
    vals = np.array([[float(v) for v in ln.split(",")] for ln in rows])
    return {k: vals[:, n].reshape(p.ny, p.nx) for n, k in enumerate(MAIN_VARS)}
