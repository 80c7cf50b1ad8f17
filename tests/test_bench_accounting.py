"""The bench's roofline arithmetic on CPU: the algorithmic bytes of one CG
iteration at the 1M-vertex workload's sizes, the textbook figures they are
compared with, and the kernel named for each CG variant."""
import os
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)

import bench  # noqa: E402

N, NNZ = 1_048_576, 7_331_842  # 1024 x 1024 grid: V = n^2, nnz = V + 2E, E = (n-1)(3n-1)


def test_workload_sizes():
    n = bench.GRID_N
    assert n * n == N
    assert n * n + 2 * (n - 1) * (3 * n - 1) == NNZ


def test_iteration_bytes():
    # 12 B per stored entry (two FP32 values, int32 column), row pointers, 88 B per row
    assert bench.iter_bytes(N, NNZ) == 12 * NNZ + 4 * (N + 1) + 88 * N == 184_451_100
    # one field: 8 B per entry, 44 B per row
    assert bench.iter_bytes(N, NNZ, nfields=1) == 8 * NNZ + 4 * (N + 1) + 44 * N


def test_textbook_comparison():
    # a standalone FP32 SpMV and a textbook Jacobi-PCG iteration per field
    b_spmv = 8 * NNZ + 4 * (N + 1) + 8 * N
    b_it = b_spmv + 44 * N
    assert b_spmv == 71_237_652 and b_it == 117_374_996
    assert bench.iter_bytes(N, NNZ) < 2 * b_it  # u and v share columns and row pointers


def test_kernel_names():
    names = {v: bench.cg_kernel_name(v) for v in (0, 1, 2, 3, 6, 7, 10, 11, 13, 14, 15, 4, 8, 16)}
    assert names[0] == names[1] == "k_cgcg_iter_ell"
    assert all(names[v] == "k_cgcg_iter_stream" for v in (2, 3, 6, 7))
    assert names[10] == names[11] == "k_cgcg_iter_stream (deferred finish)"
    assert names[13] == "k_cgcg_iter_direct"
    assert names[14] == names[15] == "k_cgcg_iter_ring"
    assert all(names[v] == "k_cgcg_iter" for v in (4, 8, 16))


# the variants that a new handle starts on, or that the autotuner has picked,
# on this workload
PICKED_ON_WORKLOAD = (14, 15)


def test_traffic_figures_cover_default_variants():
    # the in-loop ncu traffic is recorded for every variant a new handle or the
    # autotuner picks on this workload (the bench would report traffic null
    # for another), and is below the algorithmic bytes
    for v in PICKED_ON_WORKLOAD:
        assert v in bench.IN_LOOP_TRAFFIC, f"no in-loop DRAM traffic recorded for CG variant {v}"
        assert 0 < bench.IN_LOOP_TRAFFIC[v] < bench.iter_bytes(N, NNZ)
