"""GPU parity for the block (BCSR 5x5) path and the adjoint (backward) entry.

BCSR: SpMV, block ParILU sweeps, block SpTRSV and FGMRES against the oracle's
block restatement (FP64 within 1e-12; FP32 factors reach the same 1e-10
relative residual).
Adjoint: dL/db and dL/dA from lace_gpu_solve_backward against central finite
differences (step 1e-6, random unit directions, agreement 1e-6 relative) and
against the oracle's FP64 adjoint solve.
"""
import numpy as np
import pytest

from lace_gb300 import problems as P
from oracle import oracle as orc

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def lg(torch_cuda):
    import lace_gb300
    lace_gb300.lib()
    return lace_gb300


def dev(torch, a):
    return torch.tensor(np.ascontiguousarray(a), dtype=torch.float64, device="cuda")


def relmax(a, b):
    return float(np.max(np.abs(a - b)) / max(np.max(np.abs(b)), 1e-300))


def test_bcsr_spmv(lg, torch_cuda):
    B = P.bcsr3d(6, 5, 4, seed=2)
    x = np.random.default_rng(0).standard_normal(B.n)
    with lg.Context(0) as ctx:
        ctx.upload(B)
        y = torch_cuda.zeros(B.n, dtype=torch_cuda.float64, device="cuda")
        ctx.spmv(dev(torch_cuda, x), y)
    ref = orc.bcsr_spmv(B.row, B.col, B.val, B.bs, x)
    assert relmax(y.cpu().numpy(), ref) <= 1e-14


def test_bcsr_dropin_parilu_matches_oracle(lg):
    """data_PariLU_v0_3 with A->storage_type == Magma_BCSR dispatches to the
    block sweep (LACE: src/parilu_v0_3_bcsr.cpp); values equal the oracle's
    synchronous block sweeps after the same count."""
    from lace_gb300 import dropin
    B = P.bcsr3d(5, seed=1)
    (lp, li, lv), (up, ui, uv), info = dropin.parilu(dropin.bcsr(B), reduction=1e-24)
    F = orc.bcsr_parilu(B, info["sweeps"], mode="sync")
    assert np.array_equal(lp, F.L.ptr) and np.array_equal(li, F.L.idx)
    assert np.array_equal(up, F.U.ptr) and np.array_equal(ui, F.U.idx)
    assert relmax(lv, F.L.val.ravel()) <= 1e-12
    assert relmax(uv, F.U.val.ravel()) <= 1e-12
    # converged (step below the reduction) to the one-thread block ILU(0)
    E = orc.bcsr_parilu(B, 1, mode="async")
    assert relmax(lv, E.L.val.ravel()) <= 1e-10 and relmax(uv, E.U.val.ravel()) <= 1e-10


@pytest.mark.parametrize("prec", ["fp64", "fp32"])
def test_bcsr_fgmres_mgs(lg, torch_cuda, prec):
    """The Gram-Schmidt FGMRES on a BCSR operator (the separate-kernel step:
    the one-kernel step takes CSR operators) against the oracle's mirror of
    data_fgmres_restart with block factors."""
    B = P.bcsr3d(8, seed=4)
    b = P.rhs_normal(B.n, 0)
    F = orc.bcsr_parilu(B, 3, mode="sync")
    op = {"kind": "bcsr", "bs": B.bs, "row": B.row, "col": B.col, "val": B.val}
    r = orc.fgmres_mgs(op, orc.bcsr_precond(F), b, search_max=50, restart_max=20, rtol=1e-10)
    with lg.Context(0) as ctx:
        ctx.set_options(precision=prec)
        ctx.upload(B)
        ctx.parilu0(3)
        xd = torch_cuda.zeros(B.n, dtype=torch_cuda.float64, device="cuda")
        res = ctx.fgmres(dev(torch_cuda, b), xd, search_max=50, restart_max=20, rtol=1e-10,
                         orthogonalization="mgs")
        x = xd.cpu().numpy()
    assert res.converged and r.converged
    if prec == "fp64":
        assert abs(res.total_iterations - r.total_iterations) <= 2
    assert np.linalg.norm(b - B.to_csr().matvec(x)) <= 2e-10 * np.linalg.norm(b)


@pytest.mark.parametrize("prec", ["fp64", "fp32"])
def test_bcsr_fgmres(lg, torch_cuda, prec):
    B = P.bcsr3d(8, seed=4)
    b = P.rhs_normal(B.n, 0)
    F = orc.bcsr_parilu(B, 3, mode="sync")
    op = {"kind": "bcsr", "bs": B.bs, "row": B.row, "col": B.col, "val": B.val}
    r = orc.fgmres(op, orc.bcsr_precond(F), b, search_max=50, restart_max=20, rtol=1e-10)
    with lg.Context(0) as ctx:
        ctx.set_options(precision=prec)
        ctx.upload(B)
        ctx.parilu0(3)
        xd = torch_cuda.zeros(B.n, dtype=torch_cuda.float64, device="cuda")
        res = ctx.fgmres(dev(torch_cuda, b), xd, search_max=50, restart_max=20, rtol=1e-10)
        x = xd.cpu().numpy()
        # block triangular solves against the oracle's
        z = torch_cuda.zeros(B.n, dtype=torch_cuda.float64, device="cuda")
        q = np.random.default_rng(2).standard_normal(B.n)
        ctx.apply_precond(dev(torch_cuda, q), z)
    Ur = F.U_rows()
    t = np.zeros(B.n)
    lib = orc.lib()
    lib.orc_bcsr_trsv_lower_unit(B.nb, B.bs, F.L.ptr, F.L.idx, np.ascontiguousarray(F.L.val.ravel()), q, t)
    zr = np.zeros(B.n)
    lib.orc_bcsr_trsv_upper(B.nb, B.bs, Ur.ptr, Ur.idx, np.ascontiguousarray(Ur.val.ravel()),
                            np.ascontiguousarray(F.dinv().ravel()), t, zr)
    assert relmax(z.cpu().numpy(), zr) <= (1e-12 if prec == "fp64" else 1e-4)
    assert res.converged and r.converged
    Bc = B.to_csr()
    assert np.linalg.norm(b - Bc.matvec(x)) <= 2e-10 * np.linalg.norm(b)
    assert abs(res.total_iterations - r.total_iterations) <= 2


@pytest.mark.parametrize("method", ["householder", "mgs"])
@pytest.mark.parametrize("prec", ["fp64", "fp32"])
def test_dropin_bcsr_fgmres(lg, torch_cuda, prec, method):
    """The block system through the LACE-named calls (a BCSR operator in
    data_fgmres_householder_restart / data_fgmres_restart is this library's
    extension: LACE's data_z_spmv takes CSR only):
    data_PariLU_v0_3_prescribedSweeps on the Magma_BCSR operator returns BCSR
    / BCSC factors, which the FGMRES call takes with the operator; the second
    round reuses the analysis.  The solution equals the Context path's, the
    directions are within +-2 of the oracle's block solve, the true residual
    is at the tolerance."""
    from lace_gb300 import dropin
    B = P.bcsr3d(8, seed=4)
    b = P.rhs_normal(B.n, 0)
    F = orc.bcsr_parilu(B, 3, mode="sync")
    op = {"kind": "bcsr", "bs": B.bs, "row": B.row, "col": B.col, "val": B.val}
    solver = orc.fgmres if method == "householder" else orc.fgmres_mgs
    r = solver(op, orc.bcsr_precond(F, f32=prec == "fp32"), b, search_max=50, restart_max=20, rtol=1e-10)
    with lg.Context(0) as ctx:
        ctx.set_options(precision=prec)
        ctx.upload(B)
        ctx.parilu0(3, residual=False)
        xd = torch_cuda.zeros(B.n, dtype=torch_cuda.float64, device="cuda")
        res = ctx.fgmres(dev(torch_cuda, b), xd, search_max=50, restart_max=20, rtol=1e-10,
                         orthogonalization=method)
        xc = xd.cpu().numpy()
    Am = dropin.bcsr(B)
    Bc = B.to_csr()
    call = dropin.fgmres_householder_restart if method == "householder" else dropin.fgmres_restart
    dropin.set_options(precision=prec)
    try:
        for _ in range(2):
            L, U, info = dropin.parilu_mats(Am, max_sweeps=3)
            assert L.m.storage_type == dropin.Magma_BCSR and U.m.storage_type == dropin.Magma_BCSCU
            assert L.m.blocksize == B.bs and U.m.blocksize == B.bs
            x, rc, glog = call(Am, b, np.zeros(B.n), L, U, search_max=50, restart_max=20, rtol=1e-10, tol_type=1)
            assert rc == 0
            assert glog["restarts"] == 0 and glog["search_directions"] == res.total_iterations
            assert abs(glog["search_directions"] - r.total_iterations) <= 2
            assert np.linalg.norm(b - Bc.matvec(x)) <= 1.05e-10 * np.linalg.norm(b)
            assert relmax(x, xc) <= 1e-12
            del L, U
    finally:
        dropin.set_options()


# ------------------------------------------------------------------ adjoint

def _solve(lg, torch, ctx, A, b, sweeps=40):
    ctx.upload(A)
    ctx.parilu0(sweeps)
    x = torch.zeros(A.n, dtype=torch.float64, device="cuda")
    r = ctx.fgmres(dev(torch, b), x, search_max=50, restart_max=40, rtol=1e-14)
    assert r.converged
    return x


def test_adjoint_against_finite_differences(lg, torch_cuda):
    """L(x) = 0.5||x - x_t||^2 with A x = b (convection-diffusion, 8^3):
    gradients w.r.t. b and A's values vs central FD (h = 1e-6) along random
    unit directions; backward solve through FP32 transposed factors."""
    A = P.convdiff3d(8)
    rng = np.random.default_rng(1)
    xt = rng.standard_normal(A.n)
    b = P.rhs_normal(A.n, 0)
    torch = torch_cuda

    def loss(Aval, bvec):
        with lg.Context(0) as c:
            c.set_options(precision="fp64")
            x = _solve(lg, torch, c, P.CSR(A.n, A.row, A.col, Aval), bvec)
            xv = x.cpu().numpy()
        return 0.5 * float(np.sum((xv - xt) ** 2)), xv

    L0, x0 = loss(A.val, b)
    with lg.Context(0) as ctx:
        ctx.set_options(precision="fp32")
        ctx.upload(A)
        ctx.parilu0(3)
        xd = dev(torch, x0)
        dLdx = dev(torch, x0 - xt)
        gb = torch.zeros(A.n, dtype=torch.float64, device="cuda")
        gA = torch.zeros(A.nnz, dtype=torch.float64, device="cuda")
        ctx.backward(xd, dLdx, gb, gA, search_max=50, restart_max=40, rtol=1e-13)
        gb, gA = gb.cpu().numpy(), gA.cpu().numpy()
    # FP64 CPU adjoint: A^T lambda = x - x_t with the oracle's FGMRES on A^T
    atp, ati, atv, _ = orc.transpose(A.row, A.col, A.val, A.n)
    F = orc.parilu(A.row, A.col, A.val, 3, mode="sync")
    ra = orc.fgmres({"kind": "csr", "row": atp, "col": ati, "val": atv}, orc.ilu_precond_adjoint(F), x0 - xt,
                    search_max=50, restart_max=40, rtol=1e-13)
    assert ra.converged
    assert relmax(gb, ra.x) <= 1e-8
    # relative gradient error |fd - g.d| / ||g|| <= 1e-6 (the loss is O(n) while
    # a directional derivative along a random unit direction is O(||g||/sqrt(n)),
    # so a per-direction relative bound would measure the FD's own rounding)
    h = 1e-6
    for k in range(8):
        d = rng.standard_normal(A.n)
        d /= np.linalg.norm(d)
        fd = (loss(A.val, b + h * d)[0] - loss(A.val, b - h * d)[0]) / (2 * h)
        assert abs(fd - gb @ d) <= 1e-6 * np.linalg.norm(gb)
    for k in range(6):
        d = rng.standard_normal(A.nnz)
        d /= np.linalg.norm(d)
        fd = (loss(A.val + h * d, b)[0] - loss(A.val - h * d, b)[0]) / (2 * h)
        assert abs(fd - gA @ d) <= 1e-6 * np.linalg.norm(gA)


def test_bcsr_block_system_at_20_cubed(lg, torch_cuda):
    """The block configuration's generator (5x5 blocks on a 7-point cell
    stencil, dominant diagonal blocks) at 20^3 cells (40,000 rows): the GPU's
    block ParILU (3 synchronous sweeps, FP64) equals the oracle's to 1e-12
    (through the context and through data_PariLU_v0_3 with Magma_BCSR), the
    FP64 FGMRES-Householder matches the oracle's directions within +-2, and
    the FP32 and BF16-stored factors reach the same 1e-10 relative residual."""
    from lace_gb300 import dropin
    B = P.bcsr3d(20)
    b = P.rhs_normal(B.n, 0)
    F = orc.bcsr_parilu(B, 3, mode="sync")
    op = {"kind": "bcsr", "bs": B.bs, "row": B.row, "col": B.col, "val": B.val}
    r = orc.fgmres(op, orc.bcsr_precond(F), b, search_max=50, restart_max=20, rtol=1e-10)
    assert r.converged
    Bc = B.to_csr()
    for prec in ("fp64", "fp32", "bf16"):
        with lg.Context(0) as ctx:
            ctx.set_options(precision=prec)
            ctx.upload(B)
            ctx.parilu0(3)
            xd = torch_cuda.zeros(B.n, dtype=torch_cuda.float64, device="cuda")
            res = ctx.fgmres(dev(torch_cuda, b), xd, search_max=50, restart_max=20, rtol=1e-10)
            x = xd.cpu().numpy()
        assert res.converged
        assert np.linalg.norm(b - Bc.matvec(x)) <= 2e-10 * np.linalg.norm(b)
        if prec == "fp64":
            assert abs(res.total_iterations - r.total_iterations) <= 2
            assert relmax(x, r.x) <= 1e-8
    (lp, li, lv), (up, ui, uv), info = dropin.parilu(dropin.bcsr(B), reduction=1e-12)
    Fd = orc.bcsr_parilu(B, info["sweeps"], mode="sync")
    assert relmax(lv, Fd.L.val.ravel()) <= 1e-12 and relmax(uv, Fd.U.val.ravel()) <= 1e-12


def test_adjoint_at_64_cubed(lg, torch_cuda):
    """The adjoint configuration at its size: the convection-diffusion
    operator on 64^3 (n = 262,144), L = 0.5||x - x_t||^2 with x_t ~ N(0,1)
    (seed 1); the backward solve through the transposed FP32 factors and the
    FP64 FGMRES gives dL/db and dL/dA, checked against central finite
    differences (step 1e-6) along 32 random unit directions in b and 32 in
    A's values (|fd - g.d| <= 1e-6 ||g||), and dL/db against the oracle's
    FP64 adjoint solve.  The loss is O(n) here while a directional difference
    is O(h ||g||), so the central difference is formed from the two
    solutions, L(+) - L(-) = 0.5 sum (x+ - x-)(x+ + x- - 2 x_t), which is the
    same difference without the cancellation of two O(n) numbers."""
    A = P.convdiff3d(64)
    rng = np.random.default_rng(1)
    xt = rng.standard_normal(A.n)
    b = P.rhs_normal(A.n, 0)
    torch = torch_cuda
    with lg.Context(0) as c:
        c.set_options(precision="fp64")

        def solution(Aval, bvec):
            return _solve(lg, torch, c, P.CSR(A.n, A.row, A.col, Aval), bvec).cpu().numpy()

        def central(xp, xm):
            return 0.5 * float(np.sum((xp - xm) * (xp + xm - 2.0 * xt))) / (2 * h)

        h = 1e-6
        x0 = solution(A.val, b)
        with lg.Context(0) as ctx:
            ctx.set_options(precision="fp32")
            ctx.upload(A)
            ctx.parilu0(3)
            xd = dev(torch, x0)
            dLdx = dev(torch, x0 - xt)
            gb = torch.zeros(A.n, dtype=torch.float64, device="cuda")
            gA = torch.zeros(A.nnz, dtype=torch.float64, device="cuda")
            ctx.backward(xd, dLdx, gb, gA, search_max=50, restart_max=40, rtol=1e-13)
            gb, gA = gb.cpu().numpy(), gA.cpu().numpy()
        for k in range(32):
            d = rng.standard_normal(A.n)
            d /= np.linalg.norm(d)
            fd = central(solution(A.val, b + h * d), solution(A.val, b - h * d))
            assert abs(fd - gb @ d) <= 1e-6 * np.linalg.norm(gb), k
        for k in range(32):
            d = rng.standard_normal(A.nnz)
            d /= np.linalg.norm(d)
            fd = central(solution(A.val + h * d, b), solution(A.val - h * d, b))
            assert abs(fd - gA @ d) <= 1e-6 * np.linalg.norm(gA), k
    atp, ati, atv, _ = orc.transpose(A.row, A.col, A.val, A.n)
    F = orc.parilu(A.row, A.col, A.val, 3, mode="sync")
    ra = orc.fgmres({"kind": "csr", "row": atp, "col": ati, "val": atv}, orc.ilu_precond_adjoint(F), x0 - xt,
                    search_max=50, restart_max=40, rtol=1e-13)
    assert ra.converged
    assert relmax(gb, ra.x) <= 1e-8


@pytest.mark.parametrize("case", ["lace_layout", "bcsr_u", "random"])
def test_dropin_zilures_bcsr(lg, case):
    """data_zilures_bcsr on the GPU against the oracle's restatement (pinned
    to LACE's build in test_oracle.py): res over the product's pattern and
    nonlinres over A's entries it holds, 1e-12 relative."""
    from lace_gb300 import dropin
    from test_oracle import _zilures_bcsr_cases
    A, L, U, bs = _zilures_bcsr_cases()[case]
    r_or, nl_or = orc.zilures_bcsr(A.row, A.col, A.val, L, U, bs)
    nb = len(L[0]) - 1
    Lb = dropin.bcsr(P.BCSR(nb, bs, L[0], L[1], np.asarray(L[2]).reshape(-1, bs, bs)))
    Ub = dropin.bcsr(P.BCSR(nb, bs, U[0], U[1], np.asarray(U[2]).reshape(-1, bs, bs)))
    r, nl, rc = dropin.zilures_bcsr(dropin.csr(A.row, A.col, A.val, A.n), Lb, Ub)
    assert rc == 0
    assert r == pytest.approx(r_or, rel=1e-12)
    assert nl == pytest.approx(nl_or, rel=1e-10, abs=1e-13 * r_or)
    # an A whose size is not blocks x blocksize answers with a code
    S = P.laplace2d(4)
    _, _, rc = dropin.zilures_bcsr(dropin.csr(S.row, S.col, S.val, S.n), Lb, Ub)
    assert rc == -104
