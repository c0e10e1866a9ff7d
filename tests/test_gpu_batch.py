"""GPU parity for batched solves: many independent uneven systems with
several right-hand sides each, all advanced together (lace_gpu_batch_*).
Every (system, rhs) pair must reach its own 1e-10 relative residual with an
iteration count within +-2 of the oracle's FGMRES-Householder on that system
alone (same ParILU sweeps, FP64 factors)."""
import ctypes as C

import numpy as np
import pytest

from lace_gb300 import problems as P
from oracle import oracle as orc

pytestmark = pytest.mark.gpu


def make_batch(systems):
    n = [s.A.n for s in systems]
    row_off = np.concatenate([[0], np.cumsum(n)[:-1]]).astype(np.int32)
    nnz_off = np.concatenate([[0], np.cumsum([s.A.nnz for s in systems])[:-1]]).astype(np.int32)
    row = np.concatenate([s.A.row for s in systems]).astype(np.int32)
    col = np.concatenate([s.A.col for s in systems]).astype(np.int32)
    val = np.concatenate([s.A.val for s in systems])
    return np.array(n, dtype=np.int32), row_off, nnz_off, row, col, val


@pytest.mark.parametrize("prec", ["fp64", "fp32"])
@pytest.mark.parametrize("graph", [True, False])
def test_batched_uneven_systems(torch_cuda, prec, graph):
    import lace_gb300 as lg
    torch = torch_cuda
    systems = P.batch_aniso(count=7, side_lo=9, side_hi=40, nrhs=3, seed=5)
    n, row_off, nnz_off, row, col, val = make_batch(systems)
    N = int(n.sum())
    nrhs = 3
    L = lg.lib()
    with lg.Context(0) as ctx:
        ctx.set_options(precision=prec, use_graph=graph)
        bh = C.c_void_p()
        rc = L.lace_gpu_batch_create(C.byref(bh), ctx.h, len(systems), n.ctypes.data, row_off.ctypes.data,
                                     nnz_off.ctypes.data, row.ctypes.data, col.ctypes.data, val.ctypes.data, nrhs)
        assert rc == 0
        B = np.zeros((nrhs, N))
        for s, sy in enumerate(systems):
            B[:, row_off[s]:row_off[s] + n[s]] = sy.B
        bd = torch.tensor(B.ravel(), dtype=torch.float64, device="cuda")
        xd = torch.zeros(nrhs * N, dtype=torch.float64, device="cuda")
        iters = np.zeros(len(systems) * nrhs, dtype=np.int32)
        rc = L.lace_gpu_batch_solve(bh, 3, 30, 20, 1e-10, bd.data_ptr(), xd.data_ptr(), iters.ctypes.data)
        L.lace_gpu_batch_destroy(bh)
        assert rc == 0
        X = xd.cpu().numpy().reshape(nrhs, N)
    for s, sy in enumerate(systems):
        F = orc.parilu(sy.A.row, sy.A.col, sy.A.val, 3, mode="sync")
        for r in range(nrhs):
            x = X[r, row_off[s]:row_off[s] + n[s]]
            b = sy.B[r]
            assert np.linalg.norm(b - sy.A.matvec(x)) <= 2e-10 * np.linalg.norm(b)
            ref = orc.fgmres({"kind": "csr", "row": sy.A.row, "col": sy.A.col, "val": sy.A.val},
                             orc.ilu_precond(F, "trsv_f32" if prec == "fp32" else "trsv"), b,
                             search_max=30, restart_max=20, rtol=1e-10)
            assert abs(int(iters[s * nrhs + r]) - ref.total_iterations) <= 2, (s, r, iters[s * nrhs + r],
                                                                              ref.total_iterations)


def test_batched_32_systems_against_the_oracle(torch_cuda):
    """32 uneven systems (side 32..96: 1,024-9,216 rows; eps log-uniform in
    [0.05, 1]), two right-hand sides each, FP32 factors: the persistent launch
    gives every (system, rhs) pair its own 1e-10 relative residual in +-2 of
    the directions the oracle's FGMRES-Householder needs on that pair alone."""
    import lace_gb300 as lg
    torch = torch_cuda
    systems = P.batch_aniso(count=32, side_lo=32, side_hi=96, eps_lo=0.05, nrhs=2, seed=11)
    n, row_off, nnz_off, row, col, val = make_batch(systems)
    N = int(n.sum())
    nrhs = 2
    L = lg.lib()
    with lg.Context(0) as ctx:
        ctx.set_options(precision="fp32")
        bh = C.c_void_p()
        assert L.lace_gpu_batch_create(C.byref(bh), ctx.h, len(systems), n.ctypes.data, row_off.ctypes.data,
                                       nnz_off.ctypes.data, row.ctypes.data, col.ctypes.data, val.ctypes.data,
                                       nrhs) == 0
        B = np.zeros((nrhs, N))
        for s, sy in enumerate(systems):
            B[:, row_off[s]:row_off[s] + n[s]] = sy.B
        bd = torch.tensor(B.ravel(), dtype=torch.float64, device="cuda")
        xd = torch.zeros(nrhs * N, dtype=torch.float64, device="cuda")
        iters = np.zeros(len(systems) * nrhs, dtype=np.int32)
        rc = L.lace_gpu_batch_solve(bh, 3, 30, 40, 1e-10, bd.data_ptr(), xd.data_ptr(), iters.ctypes.data)
        L.lace_gpu_batch_destroy(bh)
        assert rc == 0
        X = xd.cpu().numpy().reshape(nrhs, N)
    for s, sy in enumerate(systems):
        F = orc.parilu(sy.A.row, sy.A.col, sy.A.val, 3, mode="sync")
        op = {"kind": "csr", "row": sy.A.row, "col": sy.A.col, "val": sy.A.val}
        for r in range(nrhs):
            x = X[r, row_off[s]:row_off[s] + n[s]]
            b = sy.B[r]
            assert np.linalg.norm(b - sy.A.matvec(x)) <= 2e-10 * np.linalg.norm(b), (s, r)
            ref = orc.fgmres(op, orc.ilu_precond(F, "trsv_f32"), b, search_max=30, restart_max=40, rtol=1e-10)
            assert abs(int(iters[s * nrhs + r]) - ref.total_iterations) <= 2, (s, r, iters[s * nrhs + r],
                                                                              ref.total_iterations)
