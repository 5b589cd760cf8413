"""The CRS text files of FEMSolver_%saveMatrix (FEMSolverClass.f90:1225-1306).

``name_data.txt`` holds the values, ``name_indices.txt`` the 1-based column
indices and ``name_indptr.txt`` the 1-based row pointers, one entry per line
(IO_%write of a vector, IOClass.f90:1409-1437: an integer is followed by one
space; a real is written list-directed, here with the 17 significant digits
that round-trip an FP64 value).  ``read_crs_files`` reads them back, so a
matrix saved by plantFEM can be handed to ``FEMSolver.setCRS(CRS=...)``.
"""
from __future__ import annotations

import numpy as np


def write_crs_files(name: str, row_ptr, col_idx, val) -> None:
    with open(name + "_data.txt", "w") as f:
        f.writelines(f"  {x:.17g}\n" for x in np.asarray(val, dtype=np.float64))
    with open(name + "_indices.txt", "w") as f:
        f.writelines(f"{int(c)} \n" for c in np.asarray(col_idx))
    with open(name + "_indptr.txt", "w") as f:
        f.writelines(f"{int(r)} \n" for r in np.asarray(row_ptr))


def read_crs_files(name: str):
    """(row_ptr int64, col_idx int32, val float64), 1-based as written."""
    val = np.loadtxt(name + "_data.txt", dtype=np.float64, ndmin=1)
    col = np.loadtxt(name + "_indices.txt", dtype=np.int64, ndmin=1).astype(np.int32)
    rp = np.loadtxt(name + "_indptr.txt", dtype=np.int64, ndmin=1)
    if rp.shape[0] < 1 or rp[-1] - rp[0] != val.shape[0] or col.shape[0] != val.shape[0]:
        raise ValueError(f"{name}_*.txt: row pointers, indices and values do not agree")
    return rp, col, val


def write_dense_csv(path: str, row_ptr, col_idx, val, zero_or_nonzero: bool = False, max_n: int = 20000) -> None:
    """CRS_as_dense: the matrix as an n x n CSV.

    With ``zero_or_nonzero`` each entry is one character, ``0`` or ``*``, with
    no separator between them, as FEMSolverClass.f90:1265-1285 writes it (its
    ``cycle`` skips the comma).
    """
    n = len(row_ptr) - 1
    if n > max_n:
        raise ValueError(f"dense CSV of a {n} x {n} matrix refused (limit {max_n})")
    with open(path, "w") as f:
        for i in range(n):
            row = np.zeros(n)
            lo, hi = row_ptr[i] - 1, row_ptr[i + 1] - 1
            row[np.asarray(col_idx[lo:hi]) - 1] = val[lo:hi]
            if zero_or_nonzero:
                f.write("".join("0" if x == 0.0 else "*" for x in row) + "\n")
            else:
                f.write(",".join(repr(float(x)) for x in row) + "\n")
