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
    assert open(str(tmp_path / "K_dense.csv")).read().splitlines() == ["*0*", "0*0", "*0*"]


def test_vtk_hex8_mesh_with_fields(tmp_path):
    from plantfem_gb300 import FEMDomain
    dom = FEMDomain().create("Cube3D", 2, 1, 1)
    disp = np.zeros(3 * dom.nn())
    disp[2::3] = 0.5
    path = dom.vtk(str(tmp_path / "m"), scalar=np.arange(dom.ne(), dtype=float),
                   vector=np.ones((dom.nn(), 3)), displacement=disp)
    txt = open(path).read().splitlines()
    assert txt[0] == "# vtk DataFile Version 2.0" and txt[4] == f"POINTS {dom.nn()} float"
    pts = np.array([[float(v) for v in ln.split()] for ln in txt[5:5 + dom.nn()]])
    assert np.allclose(pts, dom.nodcoord + disp.reshape(-1, 3))  # deformed on output only
    k = 5 + dom.nn()
    assert txt[k] == f"CELLS {dom.ne()} {dom.ne() * 9}"
    assert txt[k + 1].split() == ["8"] + [str(int(c) - 1) for c in dom.elemnod[0]]
    assert f"CELL_DATA {dom.ne()}" in txt and f"POINT_DATA {dom.nn()}" in txt and "CELL_TYPES 2" in txt
    assert np.allclose(dom.nodcoord.max(axis=0), [1.0, 1.0, 1.0])  # domain unchanged


def test_vtk_import_round_trip_and_mixed_cells(tmp_path):
    """importVTKFile (ImportVTKFileFEMDomain, FEMDomainClass.f90:13254): a file
    written by FEMDomain.vtk reads back to the same mesh and fields; with mixed
    cell types only the cells of the largest type are kept."""
    from plantfem_gb300 import FEMDomain
    dom = FEMDomain().create("Cube3D", 3, 2, 2)
    dom.nodcoord = dom.nodcoord + np.random.default_rng(0).uniform(-0.01, 0.01, dom.nodcoord.shape)
    sc = np.linspace(0.0, 1.0, dom.ne())
    ve = np.random.default_rng(1).standard_normal((dom.nn(), 3))
    te = np.random.default_rng(2).standard_normal((dom.ne(), 3, 3))
    dom.vtk(str(tmp_path / "rt"), scalar=sc, vector=ve)
    back = FEMDomain().importVTKFile(str(tmp_path / "rt"))
    assert np.array_equal(back.nodcoord, dom.nodcoord) and np.array_equal(back.elemnod, dom.elemnod)
    assert np.array_equal(back.PhysicalField[0]["scalar"], sc)
    assert np.array_equal(back.PhysicalField[1]["vector"], ve)
    dom.vtk(str(tmp_path / "t"), tensor=te)
    assert np.array_equal(FEMDomain().importVTKFile(str(tmp_path / "t.vtk")).PhysicalField[0]["tensor"], te)
    # mixed cells, two points per line
    txt = ["# vtk DataFile Version 2.0", "mixed", "ASCII", "DATASET UNSTRUCTURED_GRID", "POINTS 9 float",
           "0 0 0 1 0 0", "1 1 0 0 1 0", "0 0 1 1 0 1", "1 1 1 0 1 1", "2 0 0",
           "CELLS 2 14", "4 1 2 8 0", "8 0 1 2 3 4 5 6 7", "CELL_TYPES 2", "10", "12"]
    (tmp_path / "mx.vtk").write_text("\n".join(txt) + "\n")
    m = FEMDomain().importVTKFile(str(tmp_path / "mx.vtk"))
    assert m.nn() == 9 and m.elemnod.tolist() == [[1, 2, 3, 4, 5, 6, 7, 8]]
    assert np.array_equal(m.nodcoord[8], [2.0, 0.0, 0.0])


def test_divide_known_answer_and_properties():
    """FEMDomain_%divide (divide_nFEMDomain, FEMDomainClass.f90:1077-1296): a 2x1x1
    cube split at its two elements shares the middle face; on a larger mesh the
    pieces partition the elements, each element lies nearest its own kernel,
    local and global numbering agree and the shared-node rows pair up."""
    from plantfem_gb300 import FEMDomain
    d = FEMDomain().create("Cube3D", 2, 1, 1)
    a, b = d.divide(2, centers=[1, 2])
    assert a.mpi_global_node_idx.tolist() == [1, 2, 4, 5, 7, 8, 10, 11]
    assert b.mpi_global_node_idx.tolist() == [2, 3, 5, 6, 8, 9, 11, 12]
    assert a.mpi_shared_node_info.tolist() == [[2, 1, 1], [4, 1, 3], [6, 1, 5], [8, 1, 7]]
    assert b.mpi_shared_node_info.tolist() == [[1, 0, 2], [3, 0, 4], [5, 0, 6], [7, 0, 8]]

    big = FEMDomain().create("Cube3D", 6, 5, 4)
    ps = big.divide(4, seed=3)
    assert sum(p.ne() for p in ps) == big.ne()
    # nearest kernel: the element centres of piece i are closest to kernel i
    kern = np.random.default_rng(3).choice(big.ne(), size=4, replace=False) + 1
    kc = big.centerPosition()[kern - 1]
    for i, p in enumerate(ps):
        pc = p.centerPosition()
        dist = ((pc[:, None, :] - kc[None, :, :]) ** 2).sum(axis=2)
        assert np.all(dist[:, i] <= dist.min(axis=1))
    rows = np.concatenate([p.mpi_global_node_idx[p.elemnod - 1] for p in ps])
    assert sorted(map(tuple, rows)) == sorted(map(tuple, big.elemnod))
    for i, p in enumerate(ps):
        g = p.mpi_global_node_idx
        assert np.all(np.diff(g) > 0)
        assert np.array_equal(p.nodcoord, big.nodcoord[g - 1])
        for loc, j, other in p.mpi_shared_node_info:
            assert g[loc - 1] == ps[j].mpi_global_node_idx[other - 1]
            assert [other, i, loc] in ps[j].mpi_shared_node_info.tolist()
    # every node used by two pieces is listed as shared
    owners = {}
    for i, p in enumerate(ps):
        for gnode in p.mpi_global_node_idx:
            owners.setdefault(int(gnode), set()).add(i)
    for i, p in enumerate(ps):
        listed = {int(p.mpi_global_node_idx[loc - 1]) for loc, _, _ in p.mpi_shared_node_info}
        assert listed == {gn for gn in map(int, p.mpi_global_node_idx) if len(owners[gn]) > 1}


def test_vtk_mpi_round_trip(tmp_path):
    """vtk_MPI_FEMDOmain (FEMDomainClass.f90:8309-8360) writes each piece's VTK file
    and node-map CSV; read_vtk (:16505-16513) reads a piece back."""
    from plantfem_gb300 import FEMDomain
    d = FEMDomain().create("Cube3D", 4, 3, 3)
    name = str(tmp_path / "Cube3D")
    paths = d.vtk_MPI(name, 3, seed=1)
    assert len(paths) == 6
    txt = open(name + "_000001.csv").read().splitlines()
    assert txt[0].startswith("# number of global node, number of local node, number of shared node,")
    assert txt[1].split(",")[0].strip() == str(d.nn()) and txt[1].split(",")[3].strip() == "3"
    ref = d.divide(3, seed=1)
    for rank in range(3):
        back = FEMDomain().read_vtk(name, rank)
        assert np.array_equal(back.elemnod, ref[rank].elemnod)
        assert np.array_equal(back.nodcoord, ref[rank].nodcoord)
        assert np.array_equal(back.mpi_global_node_idx, ref[rank].mpi_global_node_idx)
        assert np.array_equal(back.mpi_shared_node_info, ref[rank].mpi_shared_node_info)
