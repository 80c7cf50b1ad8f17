"""CPU cross-check of the oracle's assembly against a second, independent
implementation of the documented contract.

The reference assembles with Eigen (FEMContext.cpp:97-112, 134-149,
186-201): triplets, `setFromTriplets` (duplicates summed), `makeCompressed`
(sorted inner indices, explicit zeros kept).  Eigen is absent here, so the
oracle's C restatement has no reference output to match.  This test builds the
same matrices a second way -- element blocks in numpy (FP64) from the
reference's formulas, triplets filtered as the reference filters them, and
scipy's COO -> CSR conversion, which sums duplicates and keeps explicit zeros
-- and checks that the oracle agrees: the pattern bit for bit, the values to
FP64 rounding.  Meshes: the reference's own icosphere.obj (Neumann) and
tube.obj (Dirichlet and Neumann), and a jittered grid.
"""
import numpy as np
import pytest
import scipy.sparse as sp

from conftest import reference_meshes
from fea_gb300 import meshgen as mg

VELOCITY = np.array([1.0, 0.0, 0.0])


def element_blocks(xyz, tri, velocity=VELOCITY):
    """Local K, M and Adv [T, 3, 3] in FP64 (FEMContext.cpp:72-95, 121-133, 158-183)."""
    x = xyz.astype(np.float64)
    a, b, c = x[tri[:, 0]], x[tri[:, 1]], x[tri[:, 2]]
    e1, e2 = b - a, c - a
    cr = np.cross(e1, e2)
    jac = np.linalg.norm(cr, axis=1)
    n = cr / jac[:, None]
    A = np.stack([e1, e2, n], axis=2)  # columns b - a, c - a, normal
    G = np.transpose(np.linalg.inv(A), (0, 2, 1))  # A^-T
    ref = np.array([[-1.0, -1.0, 0.0], [1.0, 0.0, 0.0], [0.0, 1.0, 0.0]])
    grads = np.einsum("tij,kj->tki", G, ref)  # [T, 3 basis, 3 xyz]
    K = 0.5 * jac[:, None, None] * np.einsum("tix,tjx->tij", grads, grads)
    M = (jac / 24.0)[:, None, None] * (np.ones((3, 3)) + np.eye(3))[None]
    vt = velocity[None, :] - (n @ velocity)[:, None] * n  # tangential velocity, then normalised
    nv = np.linalg.norm(vt, axis=1)
    vt = np.where(nv[:, None] > 0, vt / np.where(nv > 0, nv, 1.0)[:, None], 0.0)
    adv_j = np.einsum("tx,tjx->tj", vt, grads)
    Adv = (jac / 6.0)[:, None, None] * np.broadcast_to(adv_j[:, None, :], (tri.shape[0], 3, 3))
    return K, M, Adv


def scipy_assembly(xyz, tri, bc, on_boundary):
    """CSR of K, M (filter: Neumann, or neither vertex on the boundary) and
    Adv (filter ignores the BC, FEMContext.cpp:188) through COO -> CSR."""
    V = xyz.shape[0]
    idx = np.full(V, -1, dtype=np.int64)
    keep = np.ones(V, bool) if bc == 1 else on_boundary == 0
    idx[keep] = np.arange(int(keep.sum()))
    N = int(keep.sum())
    K, M, Adv = element_blocks(xyz, tri)
    ti = np.repeat(tri[:, :, None], 3, axis=2)  # [T, i, j] -> vertex i
    tj = np.repeat(tri[:, None, :], 3, axis=1)  # [T, i, j] -> vertex j
    ob_i, ob_j = on_boundary[ti] != 0, on_boundary[tj] != 0
    interior = ~ob_i & ~ob_j
    km = np.ones_like(interior) if bc == 1 else interior
    out = {}
    for name, loc, m in (("K", K, km), ("M", M, km), ("Adv", Adv, interior)):
        r, c, v = idx[ti[m]], idx[tj[m]], loc[m]
        A = sp.coo_matrix((v, (r, c)), shape=(N, N)).tocsr()  # sums duplicates, keeps explicit zeros
        A.sort_indices()
        out[name] = A
    return out, N


@pytest.mark.parametrize("case", ["icosphere-neumann", "tube-dirichlet", "tube-neumann", "grid-dirichlet"])
def test_oracle_matches_independent_assembly(oracle_mod, case):
    name, bcs = case.split("-")
    bc = oracle_mod.DIRICHLET if bcs == "dirichlet" else oracle_mod.NEUMANN
    if name == "grid":
        xyz, tri = mg.jittered_grid(40, seed=5)
    else:
        xyz, tri = reference_meshes()[name]
    S = oracle_mod.System(xyz, tri, bc=bc)
    ref, N = scipy_assembly(xyz, tri, bc, S.on_boundary)
    assert S.N == N
    # pattern: Eigen's compressed storage of the K/M triplets, bit for bit
    assert np.array_equal(S.row_ptr, ref["K"].indptr.astype(np.int32))
    assert np.array_equal(S.col, ref["K"].indices.astype(np.int32))
    assert np.array_equal(ref["M"].indptr, ref["K"].indptr) and np.array_equal(ref["M"].indices, ref["K"].indices)
    # values: same sums in another order (FP64)
    for key, val in (("K", S.K), ("M", S.M)):
        scale = np.abs(ref[key].data).max()
        assert np.max(np.abs(val - ref[key].data)) <= 1e-12 * scale, key
    # advection: its own (BC-blind) filter, a subset of the K/M pattern
    adv_dense_rows = ref["Adv"].tocoo()
    got = sp.csr_matrix((S.Adv, S.col, S.row_ptr), shape=(N, N))
    present = sp.csr_matrix((S.adv_present.astype(np.float64), S.col, S.row_ptr), shape=(N, N))
    # every reference advection entry sits in the pattern and is marked present
    assert np.all(np.asarray(present[adv_dense_rows.row, adv_dense_rows.col]).ravel() == 1)
    assert int(S.adv_present.sum()) == ref["Adv"].nnz
    diff = np.asarray(got[adv_dense_rows.row, adv_dense_rows.col]).ravel() - adv_dense_rows.data
    assert np.max(np.abs(diff)) <= 1e-12 * max(np.abs(adv_dense_rows.data).max(), 1e-30)


def test_explicit_zeros_survive_compression(oracle_mod):
    """Two triangles whose contributions to an entry cancel leave an explicit
    zero in the compressed pattern (makeCompressed keeps stored zeros); scipy's
    conversion keeps it too."""
    # a square split along its diagonal: K's entry between the two off-diagonal
    # corners is 0 exactly (right angles at both), yet it is stored
    xyz = np.array([[0, 0, 0], [1, 0, 0], [1, 1, 0], [0, 1, 0]], dtype=np.float32)
    tri = np.array([[0, 1, 2], [0, 2, 3]], dtype=np.uint32)
    S = oracle_mod.System(xyz, tri, bc=oracle_mod.NEUMANN)
    ref, _ = scipy_assembly(xyz, tri, 1, S.on_boundary)
    assert S.nnz == ref["K"].nnz == 4 + 2 * 5
    zeros = np.flatnonzero(S.K == 0.0)
    assert zeros.size > 0 and np.array_equal(S.col, ref["K"].indices)
