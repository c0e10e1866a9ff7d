"""Parity at the benchmark configurations' full sizes (the other GPU tests use
small systems): the 128^3 convection-diffusion system (n = 2,097,152) and
the 5x5-block system on 64^3 cells (n = 1,310,720), mixed precision and
FP64, against the oracle's FGMRES-Householder with the same synchronous
ParILU(0) sweeps, on the host's cores: directions within +-2, the true
relative residual at the tolerance, the solutions close.  The 128^3 case is
also held against LACE's own in-place ParILU (its OpenMP form), as the
benchmark's CPU baseline runs it."""
import os

import numpy as np
import pytest

from lace_gb300 import problems as P
from oracle import oracle as orc

pytestmark = pytest.mark.gpu

RTOL = 1e-10


@pytest.fixture(scope="module")
def lg(torch_cuda):
    import lace_gb300
    lace_gb300.lib()
    orc.set_threads(os.cpu_count() or 1)
    return lace_gb300


def gpu_solve(lg, torch, A, b, prec):
    with lg.Context(0) as ctx:
        ctx.set_options(precision=prec)
        ctx.upload(A)
        ctx.parilu0(3, residual=False)
        xd = torch.zeros(A.n, dtype=torch.float64, device="cuda")
        res = ctx.fgmres(torch.tensor(b, dtype=torch.float64, device="cuda"), xd, search_max=50, restart_max=20,
                         rtol=RTOL)
        return res, xd.cpu().numpy()


@pytest.mark.parametrize("prec", ["fp32", "fp64"])
def test_convdiff_128_full_size(lg, torch_cuda, prec):
    A = P.convdiff3d(128)
    b = P.rhs_normal(A.n, 0)
    res, x = gpu_solve(lg, torch_cuda, A, b, prec)
    assert res.converged
    rel = np.linalg.norm(b - A.matvec(x)) / np.linalg.norm(b)
    assert rel <= 1.05 * RTOL
    op = {"kind": "csr", "row": A.row, "col": A.col, "val": A.val}
    F = orc.parilu(A.row, A.col, A.val, 3, mode="sync")
    ref = orc.fgmres(op, orc.ilu_precond(F, "trsv_f32" if prec == "fp32" else "trsv"), b, search_max=50,
                     restart_max=20, rtol=RTOL)
    assert ref.converged
    assert abs(res.total_iterations - ref.total_iterations) <= 2, (res.total_iterations, ref.total_iterations)
    assert np.linalg.norm(x - ref.x) <= 1e-6 * np.linalg.norm(ref.x)
    if prec == "fp32":
        # LACE's own factorisation (in place, OpenMP) with exact FP64 solves
        E = orc.parilu(A.row, A.col, A.val, 3, mode="async_omp")
        lace = orc.fgmres(op, orc.ilu_precond(E), b, search_max=50, restart_max=20, rtol=RTOL)
        assert abs(res.total_iterations - lace.total_iterations) <= 2


@pytest.mark.parametrize("prec", ["fp32", "fp64"])
def test_bcsr_64_cells_full_size(lg, torch_cuda, prec):
    B = P.bcsr3d(64)
    b = P.rhs_normal(B.n, 0)
    res, x = gpu_solve(lg, torch_cuda, B, b, prec)
    assert res.converged
    Acsr = B.to_csr()
    rel = np.linalg.norm(b - Acsr.matvec(x)) / np.linalg.norm(b)
    assert rel <= 1.05 * RTOL
    F = orc.bcsr_parilu(B, 3, mode="sync")
    op = {"kind": "bcsr", "bs": B.bs, "row": B.row, "col": B.col, "val": B.val}
    ref = orc.fgmres(op, orc.bcsr_precond(F, f32=prec == "fp32"), b, search_max=50, restart_max=20, rtol=RTOL)
    assert ref.converged
    assert abs(res.total_iterations - ref.total_iterations) <= 2, (res.total_iterations, ref.total_iterations)
    assert np.linalg.norm(x - ref.x) <= 1e-6 * np.linalg.norm(ref.x)
