"""Host-side logic (no GPU): mesh generation, selection, problem builders."""
import numpy as np
import pytest

import oracle as O
from plantfem_gb300 import FEMDomain, problems


@pytest.mark.parametrize("shape", [(1, 1, 1), (2, 3, 4), (7, 5, 3), (20, 20, 20)])
def test_cube3d_bit_exact_vs_oracle(shape):
    d = FEMDomain().create("Cube3D", *shape, x_len=1.3, y_len=0.7, z_len=2.1)
    xyz, en = O.cube3d(*shape, 1.3, 0.7, 2.1)
    np.testing.assert_array_equal(d.nodcoord, xyz)
    np.testing.assert_array_equal(d.elemnod, en)


def test_resize_select_and_counts():
    d = FEMDomain().create("Cube3D", 10, 10, 100)
    d.resize(z=10.0)
    assert d.nn() == 11 * 11 * 101 and d.ne() == 10 * 10 * 100 and d.nne() == 8
    assert abs(d.z_max() - 10.0) < 1e-12
    bottom = d.select(z_max=d.z_min())
    assert bottom.shape[0] == 121 and bottom.min() == 1


def test_top_traction_sums_to_force():
    p = problems.cube(6)
    f = p["rhs"]
    assert abs(f[2::3].sum() - (-1.0)) < 1e-12
    assert np.abs(f[0::3]).max() == 0.0 and np.abs(f[1::3]).max() == 0.0
    h2 = (1.0 / 6) ** 2
    nz = f[2::3][f[2::3] != 0]
    assert set(np.round(nz / -h2, 12)) == {0.25, 0.5, 1.0}


def test_lognormal_field_is_seeded():
    a = problems.lognormal_E(1000)
    b = problems.lognormal_E(1000)
    np.testing.assert_array_equal(a, b)
    assert abs(np.log(a).mean() - np.log(1e4)) < 0.05 and abs(np.log(a).std() - 0.5) < 0.05


def test_slab_problem_shapes():
    nx, ny, nz, _ = problems.slab_sizes(512, seed=5)
    assert nx.min() >= 8 and nx.max() <= 64 and nz.min() >= 1 and nz.max() <= 3
    p = problems.slab(int(nx[0]), int(ny[0]), int(nz[0]), 1e4)
    d = p["domain"]
    assert abs(max(d.x_max(), d.y_max()) - 1.0) < 1e-12
    # clamped face x = 0 (y = 0 when nx > ny): it spans the longer in-plane
    # edge and the thickness
    assert p["fix_ids"].shape[0] == 3 * (nz[0] + 1) * (max(nx[0], ny[0]) + 1)
