"""The linear-elastic benchmark problems, as seeded synthetic inputs.

Each builder returns a dict with the mesh (``FEMDomain``), per-element
properties, the fixed DOF ids (1-based) and the nodal load vector.  The
reference has no surface-traction integrator, so a uniform traction ``t`` on
the top face is applied as consistent nodal loads: each top face of area A
gives ``t * A / 4`` to each of its four nodes, which for a uniform grid is
``t h^2`` at interior nodes, ``t h^2 / 2`` on edges and ``t h^2 / 4`` at corners.

Problems (seeds are recorded in each dict):

* ``cube``      -- unit cube n^3, E = 1e4, nu = 0.3, z = 0 fixed, traction -1 z on top
                   (n = 20: 27,783 DOF, BiCGSTAB to 1e-10);
* ``lognormal`` -- the same with E_e = exp(N(ln 1e4, 0.5^2)) per element
                   (n = 100: 3,090,903 DOF, CG FP64 vs FP32 inner + FP64 refinement);
* ``cantilever``-- unit cube n^3 with consistent mass rho = 1e3, x = 0 fixed
                   (n = 60: lowest modes by LOBPCG);
* ``slabs``     -- 512 thin slabs nx, ny ~ U{8..64}, nz ~ U{1..3}, one short edge fixed.
"""
from __future__ import annotations

import numpy as np

from .femdomain import FEMDomain

SEED_LOGNORMAL = 20261203


def top_traction(dom: FEMDomain, t: float = -1.0) -> np.ndarray:
    """Consistent nodal loads of a uniform z-traction on the z = z_max face."""
    rhs = np.zeros(dom.nn() * 3)
    zt = dom.z_max()
    en = dom.elemnod - 1
    xyz = dom.nodcoord
    top = en[:, 4:8]  # the +z face of each element (local nodes 5..8)
    on_top = np.all(xyz[top, 2] >= zt, axis=1)
    faces = top[on_top]
    # face area from its two edge vectors (rectangular faces)
    p0, p1, p3 = xyz[faces[:, 0]], xyz[faces[:, 1]], xyz[faces[:, 3]]
    area = np.linalg.norm(np.cross(p1 - p0, p3 - p0), axis=1)
    np.add.at(rhs, 3 * faces.ravel() + 2, np.repeat(t * area / 4.0, 4))
    return rhs


def fixed_face_dofs(dom: FEMDomain, axis: int = 2, value: float | None = None, dofs=(0, 1, 2)) -> np.ndarray:
    """1-based DOF ids of all nodes on the face coordinate[axis] == min."""
    v = dom.nodcoord[:, axis].min() if value is None else value
    nodes = np.nonzero(dom.nodcoord[:, axis] <= v)[0]
    ids = np.concatenate([3 * nodes + d for d in dofs]) + 1
    return np.sort(ids).astype(np.int32)


def lognormal_E(ne: int, seed: int = SEED_LOGNORMAL, mu: float = np.log(1.0e4), sigma: float = 0.5) -> np.ndarray:
    rng = np.random.default_rng(seed)
    return np.exp(rng.normal(mu, sigma, size=ne))


def cube(n: int = 20, E: float = 1.0e4, nu: float = 0.3, traction: float = -1.0) -> dict:
    dom = FEMDomain().create("Cube3D", x_num=n, y_num=n, z_num=n)
    return {"name": f"cube{n}", "domain": dom, "E": np.full(dom.ne(), E), "nu": np.full(dom.ne(), nu),
            "fix_ids": fixed_face_dofs(dom, axis=2), "rhs": top_traction(dom, traction), "seed": None}


def lognormal(n: int = 100, nu: float = 0.3, traction: float = -1.0, seed: int = SEED_LOGNORMAL) -> dict:
    dom = FEMDomain().create("Cube3D", x_num=n, y_num=n, z_num=n)
    return {"name": f"lognormal{n}", "domain": dom, "E": lognormal_E(dom.ne(), seed), "nu": np.full(dom.ne(), nu),
            "fix_ids": fixed_face_dofs(dom, axis=2), "rhs": top_traction(dom, traction), "seed": seed}


def cantilever(n: int = 60, E: float = 1.0e4, nu: float = 0.3, rho: float = 1.0e3) -> dict:
    dom = FEMDomain().create("Cube3D", x_num=n, y_num=n, z_num=n)
    return {"name": f"cantilever{n}", "domain": dom, "E": np.full(dom.ne(), E), "nu": np.full(dom.ne(), nu),
            "rho": np.full(dom.ne(), rho), "fix_ids": fixed_face_dofs(dom, axis=0), "seed": None}


def slab_sizes(count: int = 512, seed: int = 5):
    rng = np.random.default_rng(seed)
    nx = rng.integers(8, 65, size=count)
    ny = rng.integers(8, 65, size=count)
    nz = rng.integers(1, 4, size=count)
    return nx, ny, nz, rng


def slab(nx: int, ny: int, nz: int, E, nu: float = 0.3, traction: float = -1.0) -> dict:
    h = 1.0 / max(nx, ny)
    dom = FEMDomain().create("Cube3D", x_num=nx, y_num=ny, z_num=nz, x_len=nx * h, y_len=ny * h, z_len=nz * h)
    # clamped face: x = 0, or y = 0 when nx > ny (the slab's "short edge" in
    # the batched-organ benchmark's definition)
    axis = 0 if nx <= ny else 1
    Ev = np.broadcast_to(np.asarray(E, dtype=np.float64), (dom.ne(),)).copy()
    return {"name": f"slab{nx}x{ny}x{nz}", "domain": dom, "E": Ev, "nu": np.full(dom.ne(), nu),
            "fix_ids": fixed_face_dofs(dom, axis=axis), "rhs": top_traction(dom, traction)}
