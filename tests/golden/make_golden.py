"""Generate the golden fixtures of tests/golden from the CPU oracle.

Run from the repository root:  python tests/golden/make_golden.py
Writes <name>.npz files and MANIFEST.json (SHA-256 of each file).  The
fixtures pin the oracle's outputs on small cases so that regressions of
either the oracle or the GPU path show up as a fixture mismatch.
"""
import hashlib
import json
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))

import oracle as O  # noqa: E402


def save(name, **arrays):
    path = os.path.join(HERE, name + ".npz")
    np.savez_compressed(path, **arrays)
    return path


def main():
    files = []
    # hex8 element matrices: unit cube, a brick, and a general (skewed) hexahedron
    # whose Jacobian is not diagonal (pins the J^-T form of the reference's B).
    cube = np.array([[0, 0, 0], [1, 0, 0], [1, 1, 0], [0, 1, 0], [0, 0, 1], [1, 0, 1], [1, 1, 1], [0, 1, 1]], float)
    brick = cube * np.array([0.5, 0.25, 2.0])
    skew = cube + np.array([[0.0, 0.0, 0.0], [0.1, 0.05, 0.0], [0.2, 0.1, 0.05], [0.05, 0.0, 0.1],
                            [0.0, 0.1, 0.0], [0.1, 0.0, 0.2], [0.0, 0.15, 0.1], [0.1, 0.1, 0.0]])
    Ke = np.stack([O.hex8_stiffness(x, 1.0e4, 0.3) for x in (cube, brick, skew)])
    Me = np.stack([O.hex8_mass(x, 1.0e3) for x in (cube, brick, skew)])
    Fe = np.stack([O.hex8_mass_vector(x, 2.4, [0, 0, -9.8]) for x in (cube, brick, skew)])
    files.append(save("hex8_elements", xe=np.stack([cube, brick, skew]), Ke=Ke, Me=Me, Fe=Fe, E=1.0e4, nu=0.3,
                      rho=1.0e3))
    # sparsity patterns (first-appearance column order) of small meshes
    pats = {}
    for (nx, ny, nz) in ((1, 1, 1), (2, 2, 2), (3, 2, 1)):
        xyz, en = O.cube3d(nx, ny, nz)
        rp, ci = O.zero_matrix(xyz.shape[0], en, 3)
        pats[f"rp_{nx}{ny}{nz}"] = rp
        pats[f"ci_{nx}{ny}{nz}"] = ci
        pats[f"xyz_{nx}{ny}{nz}"] = xyz
        pats[f"en_{nx}{ny}{nz}"] = en
    files.append(save("patterns", **pats))
    # assembled, eliminated and solved 4^3 cube with lognormal E (oracle FP64, tol 1e-13)
    n = 4
    xyz, en = O.cube3d(n, n, n)
    nn = xyz.shape[0]
    rng = np.random.default_rng(7)
    E = np.exp(rng.normal(np.log(1e4), 0.5, size=en.shape[0]))
    rp, ci = O.zero_matrix(nn, en, 3)
    val = O.assemble(xyz, en, rp, ci, "stiffness", E=E, nu=0.3)
    rhs = np.zeros(3 * nn)
    top = np.nonzero(xyz[:, 2] >= 1.0)[0]
    rhs[3 * top + 2] = -1.0 / (n * n)
    fixed = np.zeros(3 * nn, np.uint8)
    bot = np.nonzero(xyz[:, 2] <= 0.0)[0]
    for d in range(3):
        fixed[3 * bot + d] = 1
    val_assembled = val.copy()
    rhs_in = rhs.copy()
    O.apply_fix(rp, ci, val, rhs, fixed, np.zeros(3 * nn))
    x, rc, it, rr = O.pcg(rp, ci, val, rhs, tol=1e-13)
    assert rc == 0
    files.append(save("cube4_lognormal", xyz=xyz, en=en, E=E, rp=rp, ci=ci, val_assembled=val_assembled,
                      rhs_in=rhs_in, fixed=fixed, val_eliminated=val, rhs_eliminated=rhs, x=x))
    manifest = {}
    for f in files:
        manifest[os.path.basename(f)] = hashlib.sha256(open(f, "rb").read()).hexdigest()
    with open(os.path.join(HERE, "MANIFEST.json"), "w") as fh:
        json.dump({"generator": "tests/golden/make_golden.py (CPU oracle)", "files": manifest}, fh, indent=1)
    print(json.dumps(manifest, indent=1))


if __name__ == "__main__":
    main()
