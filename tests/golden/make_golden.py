"""Generates tests/golden/reference_meshes.json from the reference's own mesh
assets (assets/fem_meshes/icosphere.obj and tube.obj of the reference project).

    python tests/golden/make_golden.py /root/reference/assets/fem_meshes

The fixture holds counts, pattern checksums and a few oracle results per mesh;
it pins the oracle when the reference checkout is present and documents the
reference meshes' known sizes when it is not.  Quads of tube.obj are split as
fans (0, k, k+1): tinyobjloader's split rule is not vendored with the reference.
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


def _sig(x):
    return float(f"{float(x):.10g}")


def summarise(oracle, path, bc):
    from fea_gb300 import meshgen as mg
    xyz, tri = mg.read_obj(path)
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


def main(asset_dir):
    import oracle
    oracle.build()
    gold = {"source": "reference assets/fem_meshes", "meshes": {
        "icosphere": summarise(oracle, os.path.join(asset_dir, "icosphere.obj"), oracle.NEUMANN),
        "tube": summarise(oracle, os.path.join(asset_dir, "tube.obj"), oracle.DIRICHLET),
    }}
    with open(os.path.join(HERE, "reference_meshes.json"), "w") as fh:
        json.dump(gold, fh, indent=1, sort_keys=True)
    print(json.dumps(gold, indent=1))


if __name__ == "__main__":
    main(sys.argv[1] if len(sys.argv) > 1 else "/root/reference/assets/fem_meshes")
