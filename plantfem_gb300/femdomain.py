"""FEMDomain: the structured hex8 mesh side of plantFEM's FEMDomain_.

Host-side mesh generation and selection (O(nodes) work, numpy).  Mirrors
``FEMDomain_%create("Cube3D", ...)`` (FEMDomainClass.f90:7215-7310 ->
MeshClass.f90:6348-6361, rectangular2D :6745-6805, Convert2Dto3D
:6992-7087), ``resize`` (FEMDomainClass.f90:2123-2130 -> MeshClass.f90:892-937)
and ``select`` (FEMDomainClass.f90:12854-12910).  Arrays keep the reference's
layout: ``nodcoord`` (nn, 3) float64 and ``elemnod`` (ne, 8) int32 with 1-based
node ids.
"""
from __future__ import annotations

import numpy as np


class FEMDomain:
    def __init__(self):
        self.nodcoord = np.zeros((0, 3))
        self.elemnod = np.zeros((0, 8), dtype=np.int32)

    # ------------------------------------------------------------------ create
    def create(self, meshtype: str = "Cube3D", x_num: int = 10, y_num: int = 10, z_num: int = 10,
               x_len: float = 1.0, y_len: float = 1.0, z_len: float = 1.0) -> "FEMDomain":
        if meshtype not in ("Cube", "Cube3D", "cube3D"):
            raise NotImplementedError(f"meshtype {meshtype!r}: only Cube3D is on this path")
        nx, ny, nz = int(x_num), int(y_num), int(z_num)
        if min(nx, ny, nz) < 1:
            raise ValueError("x_num, y_num, z_num must be >= 1")
        i = np.arange(nx + 1, dtype=np.float64)
        j = np.arange(ny + 1, dtype=np.float64)
        k = np.arange(nz + 1, dtype=np.float64)
        # coordinate = len / num * (index - 1)  (MeshClass.f90:6765-6766, :7041)
        xs = x_len / float(nx) * i
        ys = y_len / float(ny) * j
        zs = z_len / float(nz) * k
        Z, Y, X = np.meshgrid(zs, ys, xs, indexing="ij")
        self.nodcoord = np.stack([X.ravel(), Y.ravel(), Z.ravel()], axis=1)
        # quads (MeshClass.f90:6794-6803), then layers (:7062-7068)
        ii, jj = np.meshgrid(np.arange(1, nx + 1), np.arange(ny), indexing="xy")
        ii, jj = ii.ravel(), jj.ravel()
        q = np.stack([ii + jj * (nx + 1), ii + 1 + jj * (nx + 1), nx + 2 + ii + jj * (nx + 1),
                      nx + 1 + ii + jj * (nx + 1)], axis=1)
        nn2 = (nx + 1) * (ny + 1)
        layers = np.arange(nz)[:, None, None] * nn2
        bottom = (q[None, :, :] + layers).reshape(-1, 4)
        top = (q[None, :, :] + layers + nn2).reshape(-1, 4)
        self.elemnod = np.ascontiguousarray(np.concatenate([bottom, top], axis=1), dtype=np.int32)
        self.shape = (nx, ny, nz)
        return self

    def resize(self, x=None, y=None, z=None) -> "FEMDomain":
        """Scale each axis to the given length (MeshClass.f90:917-936)."""
        for d, L in enumerate((x, y, z)):
            if L is None:
                continue
            span = self.nodcoord[:, d].max() - self.nodcoord[:, d].min()
            self.nodcoord[:, d] = (L / span) * self.nodcoord[:, d]
        return self

    def vtk(self, name: str, scalar=None, vector=None, tensor=None, field: str | None = None, displacement=None):
        """FEMDomain_%vtk (FEMDomainClass.f90:8362 onwards): legacy ASCII VTK of the
        hex8 mesh (cell type 12, 0-based connectivity) with an optional point or
        cell scalar / vector / tensor field (its length picks points or cells);
        ``displacement`` writes the deformed mesh (the domain itself is not changed)."""
        if displacement is not None:
            d = np.asarray(displacement, dtype=np.float64).reshape(self.nn(), 3)
            saved = self.nodcoord
            self.nodcoord = saved + d
            try:
                return self.vtk(name, scalar, vector, tensor, field)
            finally:
                self.nodcoord = saved
        path = name if name.lower().endswith(".vtk") else name + ".vtk"
        nn, ne, nne = self.nn(), self.ne(), self.elemnod.shape[1]
        lines = ["# vtk DataFile Version 2.0", name, "ASCII", "DATASET UNSTRUCTURED_GRID", f"POINTS {nn} float"]
        lines += [" ".join(repr(float(c)) for c in row) for row in self.nodcoord]
        lines.append(f"CELLS {ne} {ne * (nne + 1)}")
        lines += [f"{nne} " + " ".join(str(int(k) - 1) for k in row) for row in self.elemnod]
        lines.append(f"CELL_TYPES {ne}")
        lines += ["12"] * ne

        def block(arr, kind):
            arr = np.asarray(arr, dtype=np.float64)
            n0 = arr.shape[0]
            if n0 == nn:
                where, label = f"POINT_DATA {nn}", f"point_{kind}"
            elif n0 == ne:
                where, label = f"CELL_DATA {ne}", f"cell_{kind}"
            else:
                raise ValueError(f"{kind}: {n0} rows, expected nn = {nn} or ne = {ne}")
            label = field or label
            out = [where]
            if kind == "scalars":
                out += [f"SCALARS {label} float", "LOOKUP_TABLE default"]
                out += [repr(float(v)) for v in arr]
            elif kind == "vectors":
                out.append(f"VECTORS {label} float")
                out += [" ".join(repr(float(v)) for v in row) for row in arr.reshape(n0, -1)]
            else:
                out.append(f"TENSORS {label} float")
                for t in arr.reshape(n0, 3, 3):
                    out += [" ".join(repr(float(v)) for v in r) for r in t]
            return out

        for arr, kind in ((scalar, "scalars"), (vector, "vectors"), (tensor, "tensors")):
            if arr is not None:
                lines += block(arr, kind)
        with open(path, "w") as f:
            f.write("\n".join(lines) + "\n")
        return path

    # nodes per cell of the VTK cell types ImportVTKFileFEMDomain knows
    # (FEMDomainClass.f90:13388-13421)
    _VTK_NODES = {1: 1, 2: 1, 3: 2, 5: 3, 8: 4, 9: 4, 10: 4, 11: 8, 12: 8, 13: 6, 21: 3, 22: 6, 23: 8, 24: 10,
                  25: 16}

    def importVTKFile(self, name: str) -> "FEMDomain":
        """FEMDomain_%importVTKFile (ImportVTKFileFEMDomain, FEMDomainClass.f90:13254 onwards):
        read a legacy ASCII VTK unstructured grid: POINTS into nodcoord, CELLS
        (0-based in the file) into 1-based elemnod, keeping only the cells of
        the largest CELL_TYPES value when types are mixed (as the reference),
        and POINT_DATA / CELL_DATA SCALARS, VECTORS and TENSORS into
        ``PhysicalField`` (a list of {"name", "scalar" | "vector" | "tensor"}).
        Values are read as whitespace-separated tokens, so files with several
        points per line load too, and VECTORS / TENSORS are read without a
        LOOKUP_TABLE line (the legacy format has none for them; the reference
        skips one line there)."""
        path = name if name.lower().endswith(".vtk") else name + ".vtk"
        with open(path) as f:
            raw = [ln.strip() for ln in f]
        header = [ln for ln in raw[:4]]
        if not any("ASCII" in ln for ln in header):
            raise ValueError("importVTKFile: the VTK file must be ASCII")
        if not any(ln.startswith("DATASET") and "UNSTRUCTURED_GRID" in ln for ln in raw[:6]):
            raise ValueError("importVTKFile: DATASET must be UNSTRUCTURED_GRID")
        lines = [ln for ln in raw[4:] if ln and not ln.startswith("#")]
        pos = 0

        def tokens(count):
            nonlocal pos
            out = []
            while len(out) < count:
                out += lines[pos].split()
                pos += 1
            return out

        cells = types = None
        data_count = 0
        self.PhysicalField = []
        nodcoord = None
        while pos < len(lines):
            head = lines[pos].split()
            pos += 1
            key = head[0].upper()
            if key == "POINTS":
                n = int(head[1])
                nodcoord = np.array(tokens(3 * n), dtype=np.float64).reshape(n, 3)
            elif key == "CELLS":
                n, m = int(head[1]), int(head[2])
                flat = np.array(tokens(m), dtype=np.int64)
                cells, k = [], 0
                for _ in range(n):
                    c = int(flat[k])
                    cells.append(flat[k + 1:k + 1 + c] + 1)
                    k += c + 1
            elif key == "CELL_TYPES":
                if cells is None:
                    raise ValueError("importVTKFile: no CELLS before CELL_TYPES")
                types = np.array(tokens(int(head[1])), dtype=np.int64)
            elif key in ("POINT_DATA", "CELL_DATA"):
                data_count = int(head[1])
            elif key == "SCALARS":
                ncomp = int(head[3]) if len(head) > 3 else 1
                if lines[pos].upper().startswith("LOOKUP_TABLE"):
                    pos += 1
                v = np.array(tokens(data_count * ncomp), dtype=np.float64)
                self.PhysicalField.append({"name": head[1], "scalar": v if ncomp == 1 else v.reshape(-1, ncomp)})
            elif key == "VECTORS":
                v = np.array(tokens(3 * data_count), dtype=np.float64).reshape(data_count, 3)
                self.PhysicalField.append({"name": head[1], "vector": v})
            elif key == "TENSORS":
                v = np.array(tokens(9 * data_count), dtype=np.float64).reshape(data_count, 3, 3)
                self.PhysicalField.append({"name": head[1], "tensor": v})
        if nodcoord is None or cells is None or types is None:
            raise ValueError("importVTKFile: POINTS, CELLS and CELL_TYPES are required")
        keep = int(types.max())
        nne = self._VTK_NODES.get(keep)
        if nne is None:
            raise ValueError(f"importVTKFile: unknown cell type {keep}")
        sel = [c for c, t in zip(cells, types) if t == keep and c.shape[0] == nne]
        self.nodcoord = nodcoord
        self.elemnod = np.array(sel, dtype=np.int32).reshape(len(sel), nne)
        return self

    # ------------------------------------------------ domain decomposition
    def centerPosition(self, ElementID: int | None = None) -> np.ndarray:
        """centerPositionFEMDomain (FEMDomainClass.f90:9879 onwards): the mean of the
        element's node coordinates (ElementID 1-based); all elements' when None."""
        en = self.elemnod - 1
        c = np.zeros((self.ne(), 3))
        for a in range(en.shape[1]):  # sum, then scale, as the reference
            c = c + self.nodcoord[en[:, a]]
        c = (1.0 / en.shape[1]) * c
        return c if ElementID is None else c[int(ElementID) - 1]

    def divide(self, n: int, seed: int | None = None, centers=None) -> list["FEMDomain"]:
        """FEMDomain_%divide(n) (divide_nFEMDomain, FEMDomainClass.f90:1077-1296):
        n element "kernels" are drawn, every element goes to the kernel whose centre
        is nearest (squared distance, the first on ties), and each piece gets
        ``mpi_global_node_idx`` (its nodes' 1-based global ids, ascending; local
        node j is global node mpi_global_node_idx[j-1]), local coordinates and
        connectivity, and ``mpi_shared_node_info`` rows (local node, other piece
        (0-based), that piece's local node) for the nodes shared with each other
        piece in piece order.  The reference draws the kernels with an unseeded
        generator; here ``seed`` seeds the draw, or ``centers`` gives the n
        kernel element ids (1-based)."""
        if n == 1:
            return [self]
        ne = self.ne()
        if centers is None:
            centers = np.random.default_rng(seed).choice(ne, size=n, replace=False) + 1
        centers = np.asarray(centers, dtype=np.int64)
        cen = self.centerPosition()
        cc = cen[centers - 1]
        d = cen[:, None, :] - cc[None, :, :]
        norms = d[:, :, 0] * d[:, :, 0] + d[:, :, 1] * d[:, :, 1] + d[:, :, 2] * d[:, :, 2]
        sub = np.argmin(norms, axis=1)
        pieces, g2ls = [], []
        for i in range(n):
            en = self.elemnod[sub == i]
            gidx = np.unique(en).astype(np.int32)
            g2l = np.zeros(self.nn() + 1, dtype=np.int32)
            g2l[gidx] = np.arange(1, gidx.shape[0] + 1, dtype=np.int32)
            part = FEMDomain()
            part.nodcoord = self.nodcoord[gidx - 1].copy()
            part.elemnod = g2l[en].astype(np.int32)
            part.mpi_global_node_idx = gidx
            pieces.append(part)
            g2ls.append(g2l)
        for i in range(n):
            rows = []
            for j in range(n):
                if i == j:
                    continue
                shared = np.intersect1d(pieces[i].mpi_global_node_idx, pieces[j].mpi_global_node_idx)
                if shared.shape[0] == 0:
                    continue
                rows.append(np.stack([g2ls[i][shared], np.full(shared.shape[0], j, np.int32), g2ls[j][shared]],
                                     axis=1))
            pieces[i].mpi_shared_node_info = (np.concatenate(rows).astype(np.int32) if rows
                                              else np.zeros((0, 3), np.int32))
        return pieces

    _MPI_CSV_HEADER = ("# number of global node, number of local node, number of shared node,"
                       "                        number of division ")

    def vtk_MPI(self, name: str, num_division: int, seed: int | None = None, centers=None) -> list[str]:
        """FEMDomain_%vtk(name, num_division) (vtk_MPI_FEMDOmain, FEMDomainClass.f90:8309-8360):
        divide the domain and write, for piece i, ``name_<i:06d>.vtk`` and
        ``name_<i:06d>.csv`` (global and local node counts, its shared-node count
        and the number of pieces; the local-to-global node map; the shared-node
        rows).  Returns the written paths."""
        nn = self.nn()
        paths = []
        for i, part in enumerate(self.divide(num_division, seed=seed, centers=centers)):
            stem = f"{name}_{i:06d}"
            paths.append(part.vtk(stem))
            info = part.mpi_shared_node_info
            lines = [self._MPI_CSV_HEADER,
                     f"{nn} ,{part.nn()} ,{info.shape[0]} ,{num_division}",
                     "# local node Idx, global node Idx "]
            lines += [f"{j + 1} ,{g}" for j, g in enumerate(part.mpi_global_node_idx)]
            lines.append("# local node Idx, domain Idx, shared local node Idx ")
            lines += [f"{a} ,{b} ,{c}" for a, b, c in info]
            with open(stem + ".csv", "w") as f:
                f.write("\n".join(lines) + "\n")
            paths.append(stem + ".csv")
        return paths

    def read_mpi_property(self, name: str) -> int:
        """read_mpi_propertyFEMDomain (FEMDomainClass.f90:16472-16502): the node map
        and shared-node rows of a piece -> the number of pieces."""
        with open(name) as f:
            lines = [ln.strip() for ln in f if ln.strip()]
        counts = [int(t) for t in lines[1].replace(",", " ").split()]
        _, n_loc, n_shared, n_div = counts[:4]
        self.mpi_global_node_idx = np.zeros(n_loc, dtype=np.int32)
        for ln in lines[3:3 + n_loc]:
            idx, val = (int(t) for t in ln.replace(",", " ").split()[:2])
            self.mpi_global_node_idx[idx - 1] = val
        rows = [[int(t) for t in ln.replace(",", " ").split()[:3]] for ln in lines[4 + n_loc:4 + n_loc + n_shared]]
        self.mpi_shared_node_info = np.array(rows, dtype=np.int32).reshape(n_shared, 3)
        return n_div

    def read_vtk(self, name: str, myrank: int) -> "FEMDomain":
        """read_vtk (read_vtk_domain_decomposed_FEMDOmain, FEMDomainClass.f90:16505-16513):
        piece ``myrank`` written by vtk_MPI.  The reference reads
        ``Cube3D_<rank>`` whatever name it is given; here the name is used."""
        self.importVTKFile(f"{name}_{int(myrank):06d}.vtk")
        self.read_mpi_property(f"{name}_{int(myrank):06d}.csv")
        return self

    def deform(self, disp) -> "FEMDomain":
        """nodcoord += reshape(disp, nn, nd) with plantFEM's row-major reshape
        (FEMDomainClass.f90:14482, ArrayClass.f90:5328-5344)."""
        self.nodcoord = self.nodcoord + np.asarray(disp, dtype=np.float64).reshape(self.nn(), 3)
        return self

    # ---------------------------------------------------------------- queries
    def nn(self) -> int:
        return int(self.nodcoord.shape[0])

    def ne(self) -> int:
        return int(self.elemnod.shape[0])

    def nne(self) -> int:
        return int(self.elemnod.shape[1])

    def nd(self) -> int:
        return 3

    def x_min(self):
        return float(self.nodcoord[:, 0].min())

    def x_max(self):
        return float(self.nodcoord[:, 0].max())

    def y_min(self):
        return float(self.nodcoord[:, 1].min())

    def y_max(self):
        return float(self.nodcoord[:, 1].max())

    def z_min(self):
        return float(self.nodcoord[:, 2].min())

    def z_max(self):
        return float(self.nodcoord[:, 2].max())

    def select(self, x_min=None, x_max=None, y_min=None, y_max=None, z_min=None, z_max=None) -> np.ndarray:
        """1-based ids of the nodes inside the box (FEMDomainClass.f90:12854-12910)."""
        m = np.ones(self.nn(), dtype=bool)
        for d, lo, hi in ((0, x_min, x_max), (1, y_min, y_max), (2, z_min, z_max)):
            if lo is not None:
                m &= self.nodcoord[:, d] >= lo
            if hi is not None:
                m &= self.nodcoord[:, d] <= hi
        return (np.nonzero(m)[0] + 1).astype(np.int32)

    def element_coords(self, element_id: int) -> np.ndarray:
        return self.nodcoord[self.elemnod[element_id - 1] - 1]
