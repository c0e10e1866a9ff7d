"""data_parcsrtrsv and FGMRES's ParCSRTRSV mode against LACE's own iteration.

LACE's data_parcsrtrsv (src/trisolve.cpp:256-351) sweeps in place: L rows
upwards from row 0, U rows down from the last, each row summing its
off-diagonal products in storage order and dividing by the stored diagonal,
until sum (y_old - y_new)^2 <= tol.  The GPU sweeps in the same order
(sync-free, one warp per row) with separately rounded products and sums and
an IEEE division, so its iterates equal LACE's one-thread iterates BIT FOR
BIT (the oracle's orc_parcsrtrsv is pinned bit-exactly to LACE's build, and
the golden vectors are LACE's own outputs).  The sweep count is compared
exactly too: it only differs where a step lands within rounding of tol,
which none of these cases does.
"""
import numpy as np
import pytest

from lace_gb300 import problems as P
from oracle import oracle as orc

pytestmark = pytest.mark.gpu

G = np.load(__import__("os").path.join(__import__("os").path.dirname(__file__), "golden", "lace_golden.npz"))
DEV_ERR_ILLEGAL_VALUE = -104


@pytest.fixture(scope="module")
def lg(torch_cuda):
    import lace_gb300
    lace_gb300.lib()
    return lace_gb300


def relmax(a, b):
    return float(np.max(np.abs(a - b)) / max(np.max(np.abs(b)), 1e-300))


def _triangles(S, sweeps=3):
    F = orc.parilu(S.row, S.col, S.val, sweeps, mode="sync")
    return F.L, F.U_csr()


CASES = {
    "cd12": lambda: P.convdiff3d(12),
    "lap40": lambda: P.laplace2d(40),
    "tref19": lambda: P.trefethen(19),
    "cd_33x5x3": lambda: P.convdiff3d(33, 5, 3),
}


@pytest.mark.parametrize("name", ["lap32", "cd8", "cd12"])
def test_parcsrtrsv_equals_lace_golden(lg, name):
    """LACE's own outputs (its build, one thread): L at tol 1.0 and U at tol
    1e-20 from y = 0, on LACE's factors of the synthetic systems."""
    from lace_gb300 import dropin
    S = {"lap32": P.laplace2d(32), "cd8": P.convdiff3d(8), "cd12": P.convdiff3d(12)}[name]
    F = orc.initial_factors(S.row, S.col, S.val)
    F.L.val = G[f"{name}_L_val"]
    F.U.val = G[f"{name}_U_val"]
    Ur = F.U_csr()
    rhs = G[f"{name}_partrsv_rhs"]
    yl, itl, rc = dropin.parcsrtrsv(dropin.MagmaLower, dropin.Magma_CSRL, dropin.Magma_UNITY,
                                    F.L.ptr, F.L.idx, F.L.val, rhs, tol=1.0)
    assert rc == 0
    yu, itu, rc = dropin.parcsrtrsv(dropin.MagmaUpper, dropin.Magma_CSRU, dropin.Magma_VALUE,
                                    Ur.ptr, Ur.idx, Ur.val, rhs, tol=1e-20)
    assert rc == 0
    assert np.array_equal(yl, G[f"{name}_partrsv_L"])
    assert np.array_equal(yu, G[f"{name}_partrsv_U"])
    assert [itl, itu] == list(G[f"{name}_partrsv_iters"])


@pytest.mark.parametrize("name", list(CASES))
@pytest.mark.parametrize("tol", [1.0, 1e-6, 1e-24, 0.0])
@pytest.mark.parametrize("start", ["zero", "random", "exact"])
def test_parcsrtrsv_matches_lace_order(lg, name, tol, start):
    """Both triangles, LACE's tolerance inside FGMRES (1.0) and tighter ones,
    from a zero, a random and an already solved start vector (the last makes
    the first sweep's step small, so LACE stops after one sweep)."""
    from lace_gb300 import dropin
    S = CASES[name]()
    L, Ur = _triangles(S)
    rng = np.random.default_rng(7)
    b = rng.standard_normal(S.n) * 10.0
    for uplo, storage, diag, T in ((dropin.MagmaLower, dropin.Magma_CSRL, dropin.Magma_UNITY, L),
                                   (dropin.MagmaUpper, dropin.Magma_CSRU, dropin.Magma_VALUE, Ur)):
        u = 0 if uplo == dropin.MagmaLower else 1
        if start == "zero":
            y0 = np.zeros(S.n)
        elif start == "random":
            y0 = rng.standard_normal(S.n)
        else:
            y0, _ = orc.parcsrtrsv(u, T.ptr, T.idx, T.val, b, tol=1e-30)
        ref, itref = orc.parcsrtrsv(u, T.ptr, T.idx, T.val, b, y0=y0, tol=tol)
        y, it, rc = dropin.parcsrtrsv(uplo, storage, diag, T.ptr, T.idx, T.val, b, y0=y0, tol=tol)
        assert rc == 0
        assert it == itref, (uplo, it, itref)
        assert np.array_equal(y, ref)
        if start == "exact" and tol == 1.0:
            assert it == 1


def _gauss_seidel_triangle(n, lower, seed):
    """A CSRL / CSRU container whose rows also hold entries on the wrong side
    of the diagonal (diagonally dominant): LACE's sweep is then a true
    Gauss-Seidel iteration, new values for columns already passed in the
    sweep, old ones for the rest."""
    rng = np.random.default_rng(seed)
    ptr = [0]
    idx = []
    val = []
    for i in range(n):
        cols = sorted(set(rng.integers(0, n, size=4).tolist()) - {i})
        vals = (rng.standard_normal(len(cols)) * 0.2).tolist()
        if lower:
            idx += cols + [i]
            val += vals + [4.0 + rng.random()]
        else:
            idx += [i] + cols
            val += [4.0 + rng.random()] + vals
        ptr.append(len(idx))
    return np.array(ptr, np.int32), np.array(idx, np.int32), np.array(val)


@pytest.mark.parametrize("lower", [True, False])
def test_parcsrtrsv_gauss_seidel_order(lg, lower):
    from lace_gb300 import dropin
    n = 3000
    ptr, idx, val = _gauss_seidel_triangle(n, lower, 11 if lower else 12)
    b = np.random.default_rng(3).standard_normal(n)
    u = 0 if lower else 1
    ref, itref = orc.parcsrtrsv(u, ptr, idx, val, b, tol=1e-20)
    assert itref > 3
    uplo = dropin.MagmaLower if lower else dropin.MagmaUpper
    st = dropin.Magma_CSRL if lower else dropin.Magma_CSRU
    y, it, rc = dropin.parcsrtrsv(uplo, st, dropin.Magma_VALUE, ptr, idx, val, b, tol=1e-20)
    assert rc == 0 and it == itref
    assert np.array_equal(y, ref)


def test_parcsrtrsv_rejects_indices_outside_the_arrays(lg):
    """Where LACE would read outside its arrays (a column outside the matrix,
    an empty first L row whose diagonal would be val[-1]) the call returns
    DEV_ERR_ILLEGAL_VALUE; the kernel checks every such index before it
    follows it."""
    from lace_gb300 import dropin
    S = P.laplace2d(12)
    L, _ = _triangles(S, 1)
    b = np.ones(S.n)
    bad = L.idx.copy()
    bad[5] = S.n + 7
    _, _, rc = dropin.parcsrtrsv(dropin.MagmaLower, dropin.Magma_CSRL, dropin.Magma_UNITY, L.ptr, bad, L.val, b)
    assert rc == DEV_ERR_ILLEGAL_VALUE
    ptr = np.concatenate([[0], L.ptr.copy()])  # one more row, empty, in front
    _, _, rc = dropin.parcsrtrsv(dropin.MagmaLower, dropin.Magma_CSRL, dropin.Magma_UNITY, ptr,
                                 L.idx + 1, L.val, np.ones(S.n + 1))
    assert rc == DEV_ERR_ILLEGAL_VALUE
    # and the next call is unaffected
    y, it, rc = dropin.parcsrtrsv(dropin.MagmaLower, dropin.Magma_CSRL, dropin.Magma_UNITY, L.ptr, L.idx, L.val, b)
    ref, itref = orc.parcsrtrsv(0, L.ptr, L.idx, L.val, b)
    assert rc == 0 and it == itref and np.array_equal(y, ref)


def test_fgmres_parcsrtrsv_mode_equals_lace_trefethen(lg):
    """LACE's FGMRESHouseholderPreconditionedRestart with ParCSRTRSV
    (user_csrtrsv_choice 1; testing/test_linearSolver.cpp:621-726) on LACE's
    own factors of Trefethen_20: the same search directions, restarts and
    solution as LACE's own run (golden)."""
    from lace_gb300 import dropin
    T = P.trefethen(19)
    Am = dropin.csr(T.row, T.col, T.val, T.n)
    L = dropin.csr(G["tref_L_row"], G["tref_L_col"], G["tref_L_val"], T.n, dropin.Magma_CSRL)
    U = dropin.csr(G["tref_U_ptr"], G["tref_U_idx"], G["tref_U_val"], T.n, dropin.Magma_CSCU)
    lg_ = G["tref_fgmres1_log"]
    x, rc, log = dropin.fgmres_householder_restart(Am, np.ones(T.n), np.zeros(T.n), L, U, search_max=20,
                                                   restart_max=20, rtol=1e-3, tol_type=0, choice=1,
                                                   monitor_orthog=1)
    assert rc == 0
    assert log["restarts"] == int(lg_[1])
    assert abs(log["search_directions"] - int(lg_[2])) <= 2
    assert relmax(x, G["tref_fgmres1_x"]) <= 1e-10
    assert np.linalg.norm(np.ones(T.n) - T.matvec(x)) <= 1e-3


@pytest.mark.parametrize("method", ["householder", "mgs"])
def test_fgmres_parcsrtrsv_mode_matches_oracle(lg, method):
    """Choice 1 on the 16^3 convection-diffusion system to 1e-10: search
    directions within +-2 of the oracle's run with LACE's ParCSRTRSV (tol
    1.0), solution to 1e-8 relative."""
    from lace_gb300 import dropin
    S = P.convdiff3d(16)
    F = orc.parilu(S.row, S.col, S.val, 3, mode="sync")
    b = np.random.default_rng(0).standard_normal(S.n)
    op = {"kind": "csr", "row": S.row, "col": S.col, "val": S.val}
    prec = orc.ilu_precond(F, "partrsv", tol=1.0)
    run = orc.fgmres if method == "householder" else orc.fgmres_mgs
    ref = run(op, prec, b, search_max=50, restart_max=10, rtol=1e-10, tol_type=1)
    Am = dropin.csr(S.row, S.col, S.val, S.n)
    L = dropin.csr(F.L.ptr, F.L.idx, F.L.val, S.n, dropin.Magma_CSRL)
    U = dropin.csr(F.U.ptr, F.U.idx, F.U.val, S.n, dropin.Magma_CSCU)
    call = dropin.fgmres_householder_restart if method == "householder" else dropin.fgmres_restart
    x, rc, log = call(Am, b, np.zeros(S.n), L, U, search_max=50, restart_max=10, rtol=1e-10, tol_type=1, choice=1)
    assert rc == 0
    assert log["restarts"] == ref.restarts
    assert abs(log["search_directions"] - ref.search_directions) <= 2
    assert relmax(x, ref.x) <= 1e-8
