"""lace_gpu_parcsrtrsv_noalloc against LACE's iteration and data_parcsrtrsv.

lace_gpu_parcsrtrsv_noalloc is data_parcsrtrsv for callers that cannot
allocate device memory (a caller whose device memory belongs to its own pool,
or a latency-critical loop in which cudaMalloc/cudaFree would synchronise the
device): it takes device arrays and keeps its scratch in one fixed device
array.  It runs the same sweeps in LACE's order, so its iterate equals the
oracle's restatement of LACE's one-thread sweeps bit for bit, with the same
sweep count, and equals data_parcsrtrsv's.  Two calls in a row check that the
shared scratch (whose counters every call clears) carries nothing from one
call into the next.  A system of 216,000 rows, near the scratch's limit, runs
the full step reduction grid and the upper part of the scratch.  This file is
collected last on purpose.
"""
import ctypes as C

import numpy as np
import pytest

from lace_gb300 import problems as P
from oracle import oracle as orc

pytestmark = pytest.mark.gpu

MAX_ROWS = 262144       # LACE_GPU_NOALLOC_MAX_ROWS
DEV_ERR_NOT_SUPPORTED = -103


def relmax(a, b):
    a = np.asarray(a)
    b = np.asarray(b)
    return float(np.max(np.abs(a - b)) / max(np.max(np.abs(b)), 1e-300))


def _call(torch, lib, uplo, storage, diag, T, b, y0, tol):
    d_row = torch.tensor(np.asarray(T.ptr, dtype=np.int32), device="cuda")
    d_col = torch.tensor(np.asarray(T.idx, dtype=np.int32), device="cuda")
    d_val = torch.tensor(np.asarray(T.val, dtype=np.float64), device="cuda")
    d_rhs = torch.tensor(b, dtype=torch.float64, device="cuda")
    y = torch.tensor(y0, dtype=torch.float64, device="cuda")
    it = C.c_int(-1)
    rc = lib.lace_gpu_parcsrtrsv_noalloc(uplo, storage, diag, len(T.ptr) - 1, d_val.data_ptr(), d_row.data_ptr(),
                                         d_col.data_ptr(), d_rhs.data_ptr(), y.data_ptr(), tol, C.byref(it), None)
    return y.cpu().numpy(), it.value, rc


def test_noalloc_parcsrtrsv_matches_lace_order(torch_cuda):
    import lace_gb300 as lg
    from lace_gb300 import dropin
    lib = lg.lib()
    A = P.convdiff3d(12)
    F = orc.parilu(A.row, A.col, A.val, 3, mode="sync")
    Ur = F.U_csr()
    rng = np.random.default_rng(5)
    b = rng.standard_normal(A.n) * 10.0
    y0 = rng.standard_normal(A.n)
    cases = [(dropin.MagmaLower, dropin.Magma_CSRL, dropin.Magma_UNITY, F.L, 0),
             (dropin.MagmaUpper, dropin.Magma_CSRU, dropin.Magma_VALUE, Ur, 1)]
    for uplo, storage, diag, T, u in cases:
        for tol in (1.0, 1e-6):
            ref, itref = orc.parcsrtrsv(u, T.ptr, T.idx, T.val, b, y0=y0, tol=tol)
            yd, itd, rc = dropin.parcsrtrsv(uplo, storage, diag, T.ptr, T.idx, T.val, b, y0=y0, tol=tol)
            assert rc == 0 and itd == itref and np.array_equal(yd, ref)
            for _ in range(2):  # two calls in a row through the shared scratch
                y, it, rc = _call(torch_cuda, lib, uplo, storage, diag, T, b, y0, tol)
                assert rc == 0
                assert it == itref
                assert np.array_equal(y, ref)


def test_noalloc_parcsrtrsv_near_the_row_limit(torch_cuda):
    import lace_gb300 as lg
    from lace_gb300 import dropin
    lib = lg.lib()
    A = P.convdiff3d(60)  # 216,000 rows
    assert 200000 < A.n <= MAX_ROWS
    F = orc.parilu(A.row, A.col, A.val, 3, mode="sync")
    Ur = F.U_csr()
    b = np.random.default_rng(6).standard_normal(A.n)
    cases = [(dropin.MagmaLower, dropin.Magma_CSRL, dropin.Magma_UNITY, F.L, 0, True, True),
             (dropin.MagmaUpper, dropin.Magma_CSRU, dropin.Magma_VALUE, Ur, 1, False, False)]
    for uplo, storage, diag, T, u, lower, unit in cases:
        ref, itref = orc.parcsrtrsv(u, T.ptr, T.idx, T.val, b, tol=1e-24)
        for _ in range(2):
            y, it, rc = _call(torch_cuda, lib, uplo, storage, diag, T, b, np.zeros(A.n), 1e-24)
            assert rc == 0 and it == itref
            assert np.array_equal(y, ref)
        assert relmax(y, orc.trsv(T.ptr, T.idx, T.val, b, lower, unit)) <= 1e-12


def test_noalloc_parcsrtrsv_limits(torch_cuda):
    torch = torch_cuda
    import lace_gb300 as lg
    from lace_gb300 import dropin
    lib = lg.lib()
    small = torch.zeros(4, dtype=torch.float64, device="cuda")
    idx = torch.zeros(4, dtype=torch.int32, device="cuda")
    it = C.c_int(-1)
    # more rows than the fixed scratch holds: refused before anything runs
    rc = lib.lace_gpu_parcsrtrsv_noalloc(dropin.MagmaLower, dropin.Magma_CSRL, dropin.Magma_UNITY, MAX_ROWS + 1,
                                         small.data_ptr(), idx.data_ptr(), idx.data_ptr(), small.data_ptr(),
                                         small.data_ptr(), 1e-12, C.byref(it), None)
    assert rc == DEV_ERR_NOT_SUPPORTED
    assert lg.lib().lace_gpu_last_error() == DEV_ERR_NOT_SUPPORTED
    # uplo / storage mismatch: -1 as data_parcsrtrsv (src/trisolve.cpp:298-304)
    rc = lib.lace_gpu_parcsrtrsv_noalloc(dropin.MagmaLower, dropin.Magma_CSRU, dropin.Magma_UNITY, 4,
                                         small.data_ptr(), idx.data_ptr(), idx.data_ptr(), small.data_ptr(),
                                         small.data_ptr(), 1e-12, C.byref(it), None)
    assert rc == -1
