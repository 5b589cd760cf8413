"""CRS text files of saveMatrix: write then read back bit-exactly (CPU)."""
import numpy as np

from plantfem_gb300.crs_io import read_crs_files, write_crs_files, write_dense_csv


def test_crs_files_round_trip(tmp_path):
    rng = np.random.default_rng(0)
    rp = np.array([1, 3, 4, 6], dtype=np.int64)
    ci = np.array([1, 3, 2, 1, 3], dtype=np.int32)
    v = rng.standard_normal(5) * 10.0 ** rng.integers(-12, 12, 5)
    name = str(tmp_path / "K")
    write_crs_files(name, rp, ci, v)
    r2, c2, v2 = read_crs_files(name)
    assert np.array_equal(r2, rp) and np.array_equal(c2, ci) and np.array_equal(v2, v)
    assert open(name + "_indices.txt").readline() == "1 \n"
    write_dense_csv(str(tmp_path / "K_dense.csv"), rp, ci, v, zero_or_nonzero=True)
    assert open(str(tmp_path / "K_dense.csv")).read().splitlines() == ["*,0,*", "0,*,0", "*,0,*"]
