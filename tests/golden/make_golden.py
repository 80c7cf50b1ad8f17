"""Generates the golden fixtures of the reference's own mesh assets
(assets/fem_meshes/icosphere.obj and tube.obj of the reference project):

    python tests/golden/make_golden.py <reference>/assets/fem_meshes
    FEA_REFERENCE_ASSETS=<reference>/assets/fem_meshes python tests/golden/make_golden.py

- reference_meshes.npz: the two meshes as the OBJ reader returns them
  (float32 positions, triangles as uint16), so that the tests, on this machine
  and on the GPU machine, run the reference's fixtures without the reference
  checkout;
- reference_meshes.json: the sha256 of each source OBJ file, counts, pattern
  checksums and a few oracle results per mesh.

Quads of tube.obj are split as fans (0, k, k+1): tinyobjloader's split rule
is not vendored with the reference.
"""
import hashlib
import json
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, os.path.join(ROOT, "fea-visualizer_gb300"))
sys.path.insert(0, os.path.join(ROOT, "oracle"))

# mesh name -> boundary condition it is summarised with (tube: Dirichlet, 192 boundary points)
MESHES = {"icosphere": 1, "tube": 0}


def _sig(x):
    return float(f"{float(x):.10g}")


def summarise(oracle, xyz, tri, bc):
    S = oracle.System(xyz, tri, bc=bc)
    out = {
        "bc": bc, "V": int(S.V), "T": int(S.T), "num_boundary": int(S.num_boundary), "N": int(S.N),
        "nnz": int(S.nnz), "max_row": int(S.max_row_nonzeros),
        "row_ptr_sha256": hashlib.sha256(S.row_ptr.tobytes()).hexdigest(),
        "col_sha256": hashlib.sha256(S.col.tobytes()).hexdigest(),
        "mass_sum": _sig(S.M.sum()), "stiffness_fro": _sig(np.linalg.norm(S.K)),
        "advection_fro": _sig(np.linalg.norm(S.Adv)),
    }
    # three reference-default heat steps (EquationParameters.hpp:8-15) from z^2
    u0 = S.gather((xyz[:, 2].astype(np.float64)) ** 2)
    p = oracle.params(oracle.HEAT, 0.01, kappa=0.05, tol=1e-14)
    u, *_ = S.step(p, u0, np.zeros(S.N), nsteps=3)
    out["heat3_norm"] = _sig(np.linalg.norm(u))
    out["heat3_mass"] = _sig(np.sum(S.scipy("M") @ u))
    return out


def load_fixture():
    """name -> (xyz float32 [V, 3], tri uint32 [T, 3]) from reference_meshes.npz."""
    z = np.load(os.path.join(HERE, "reference_meshes.npz"))
    return {n: (z[n + "_xyz"], z[n + "_tri"].astype(np.uint32)) for n in MESHES}


def main(asset_dir):
    import oracle
    from fea_gb300 import meshgen as mg
    oracle.build()
    arrays, gold = {}, {"source": "reference assets/fem_meshes", "meshes": {}}
    for name, bc in MESHES.items():
        path = os.path.join(asset_dir, name + ".obj")
        with open(path, "rb") as fh:
            digest = hashlib.sha256(fh.read()).hexdigest()
        xyz, tri = mg.read_obj(path)
        assert xyz.shape[0] < 65536
        arrays[name + "_xyz"] = xyz.astype(np.float32)
        arrays[name + "_tri"] = tri.astype(np.uint16)
        gold["meshes"][name] = dict(summarise(oracle, xyz, tri, bc), obj_sha256=digest)
    np.savez_compressed(os.path.join(HERE, "reference_meshes.npz"), **arrays)
    with open(os.path.join(HERE, "reference_meshes.json"), "w") as fh:
        json.dump(gold, fh, indent=1, sort_keys=True)
    print(json.dumps(gold, indent=1))


if __name__ == "__main__":
    src = sys.argv[1] if len(sys.argv) > 1 else os.environ.get("FEA_REFERENCE_ASSETS")
    if not src:
        sys.exit("usage: make_golden.py <reference>/assets/fem_meshes (or set FEA_REFERENCE_ASSETS)")
    main(src)
