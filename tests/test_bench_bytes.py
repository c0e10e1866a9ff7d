"""The algorithmic byte counts bench.py's roofline figures divide by, pinned
to the values the documentation quotes for the 128^3 benchmark system
(n = 2,097,152, nnz = 14,581,760; L and U of ParILU(0) hold 8,339,456
entries each, diagonals included), and the batched workload's default."""
from types import SimpleNamespace

import bench

A = SimpleNamespace(n=2097152, nnz=14581760)
NNZ_T = (14581760 + 2097152) // 2


def test_arnoldi_step_bytes():
    assert bench.step_bytes(A, 15) == 820901888


def test_spmv_and_sptrsv_bytes():
    b = bench.algorithmic_bytes(A, NNZ_T, NNZ_T, "fp32")
    assert b["spmv"] == 216924160
    assert b["sptrsv_pair"] == 158597120


def test_parilu_sweep_bytes():
    assert bench.parilu_sweep_bytes(A.nnz, A.n, NNZ_T, NNZ_T, 4) == 400293888


def test_batched_workload_default():
    w = bench.workload5()
    assert w.startswith("batch_aniso: 256 independent") and "side U{32..256}" in w
