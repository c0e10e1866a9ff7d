"""Failure handling on the GPU, with no GPU fault.

LACE exits on allocation failure (LACE_CALLOC, include/dense_types.h:430-449)
and returns DEV_ERR_* codes elsewhere (dense_types.h:134-160).  This library
returns a code for every failure and keeps the device usable:
  * a bounded device wait that runs out (a row group withheld from the
    ParCSRTRSV sweep, so later rows wait for values nothing writes) ends with
    a status bit the host reads, and the same kernel then runs normally;
  * a device allocation that fails (injected) surfaces as
    DEV_ERR_DEVICE_ALLOC from whichever call needed it;
  * malformed CSR input, a zero or non-finite pivot, and a non-finite
    right-hand side surface as codes too.
"""
import ctypes as C

import numpy as np
import pytest

from lace_gb300 import problems as P
from oracle import oracle as orc

pytestmark = pytest.mark.gpu

DEV_ERR_NOT_SUPPORTED = -103
DEV_ERR_ILLEGAL_VALUE = -104
DEV_ERR_DEVICE_ALLOC = -113
DEV_ERR_BADPRECOND = -204


@pytest.fixture(scope="module")
def lg(torch_cuda):
    import lace_gb300
    lace_gb300.lib()
    return lace_gb300


@pytest.mark.parametrize("polls", [2000, 50000])
def test_bounded_wait_runs_out_and_the_device_stays_usable(lg, polls):
    st = C.c_int(-1)
    rc = lg.lib().lace_gpu_selftest_wait_limit(polls, C.byref(st))
    assert rc == 0, lg.lib().lace_gpu_error_string(rc)
    assert st.value & 1  # a wait gave up


def _pipeline(lg, torch, A, b):
    """create, upload, factorise, solve; returns the solution"""
    with lg.Context(0) as ctx:
        ctx.upload(A)
        ctx.parilu0(3)
        xd = torch.zeros(A.n, dtype=torch.float64, device="cuda")
        bd = torch.tensor(b, dtype=torch.float64, device="cuda")
        res = ctx.fgmres(bd, xd, search_max=30, restart_max=5, rtol=1e-10)
        assert res.converged
        return xd.cpu().numpy()


def test_injected_allocation_failures(lg, torch_cuda):
    """Every device allocation of a fresh create / upload / ParILU / FGMRES
    sequence fails in turn: the call that needed it raises
    DEV_ERR_DEVICE_ALLOC and the context is destroyed; with the injection
    off, the same sequence gives the oracle's solution."""
    A = P.convdiff3d(10)
    b = np.random.default_rng(4).standard_normal(A.n)
    L = lg.lib()
    failures = 0
    try:
        for k in range(200):
            L.lace_gpu_inject_alloc_failure(k)
            try:
                _pipeline(lg, torch_cuda, A, b)
            except lg.LaceError as e:
                assert e.code == DEV_ERR_DEVICE_ALLOC, (k, e.code)
                failures += 1
                continue
            break  # k allocations were enough for the whole sequence
        else:
            pytest.fail("the sequence never completed under the injection")
    finally:
        L.lace_gpu_inject_alloc_failure(-1)
    assert failures >= 5
    x = _pipeline(lg, torch_cuda, A, b)
    F = orc.parilu(A.row, A.col, A.val, 3, mode="sync")
    r = orc.fgmres({"kind": "csr", "row": A.row, "col": A.col, "val": A.val}, orc.ilu_precond(F), b,
                   search_max=30, restart_max=5, rtol=1e-10)
    assert np.linalg.norm(x - r.x) <= 1e-8 * np.linalg.norm(r.x)


def test_malformed_csr_is_rejected(lg):
    """Upload-time checks: row pointers, column range, sorted rows, a
    diagonal entry in every row."""
    A = P.laplace2d(6)
    cases = []
    row = A.row.copy()
    row[0] = 1
    cases.append((row, A.col, DEV_ERR_ILLEGAL_VALUE))         # row[0] != 0
    row = A.row.copy()
    row[4] = row[3] - 1
    cases.append((row, A.col, DEV_ERR_ILLEGAL_VALUE))         # decreasing row pointers
    col = A.col.copy()
    col[7] = A.n
    cases.append((A.row, col, DEV_ERR_ILLEGAL_VALUE))         # column outside the matrix
    col = A.col.copy()
    col[A.row[5]], col[A.row[5] + 1] = col[A.row[5] + 1], col[A.row[5]]
    cases.append((A.row, col, DEV_ERR_NOT_SUPPORTED))         # unsorted row
    keep = np.ones(len(A.col), bool)
    keep[np.flatnonzero(A.col == 0)[0]] = False               # row 0's diagonal removed
    row = np.concatenate([[0], np.cumsum(np.add.reduceat(keep.astype(int), A.row[:-1]))]).astype(np.int32)
    cases.append((row, A.col[keep], DEV_ERR_NOT_SUPPORTED))   # missing diagonal
    with lg.Context(0) as ctx:
        for r, c, code in cases:
            with pytest.raises(lg.LaceError) as e:
                ctx.upload(P.CSR(A.n, r, c, np.ones(len(c))))
            assert e.value.code == code
        ctx.upload(A)  # and the context still takes a good matrix
        ctx.parilu0(2)


@pytest.mark.parametrize("bad", ["zero_pivot", "nan_in_A"])
def test_bad_pivots_are_reported(lg, bad):
    A = P.laplace2d(8)
    val = A.val.copy()
    d0 = int(np.flatnonzero((A.col == 0))[0])
    val[d0] = 0.0 if bad == "zero_pivot" else np.nan
    with lg.Context(0) as ctx:
        ctx.upload(P.CSR(A.n, A.row, A.col, val))
        with pytest.raises(lg.LaceError) as e:
            ctx.parilu0(3)
        assert e.value.code == DEV_ERR_BADPRECOND
        ctx.upload(A)  # the same context factorises a good matrix afterwards
        ctx.parilu0(3)


def test_non_finite_rhs_does_not_converge(lg, torch_cuda):
    A = P.laplace2d(8)
    b = np.ones(A.n)
    b[3] = np.inf
    with lg.Context(0) as ctx:
        ctx.upload(A)
        ctx.parilu0(3)
        xd = torch_cuda.zeros(A.n, dtype=torch_cuda.float64, device="cuda")
        res = ctx.fgmres(torch_cuda.tensor(b, dtype=torch_cuda.float64, device="cuda"), xd, search_max=10,
                         restart_max=2, rtol=1e-10)
        assert not res.converged
