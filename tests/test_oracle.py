"""CPU tests: the oracle is pinned against LACE's own outputs.

Two anchors:
  * tests/golden/lace_golden.npz - outputs of LACE's unmodified sources
    (generated by tests/golden/make_golden.py), always available;
  * the live LACE build in oracle/_ref (only where the LACE source tree is
    present; skipped elsewhere).
The oracle's one-thread restatements reproduce LACE operation by operation,
so most checks are bit-exact.
"""
import os

import numpy as np
import pytest

from lace_gb300 import problems as P
from oracle import oracle as orc
from oracle import reference as ref

G = np.load(os.path.join(os.path.dirname(__file__), "golden", "lace_golden.npz"))


@pytest.fixture(autouse=True, scope="module")
def one_thread():
    orc.set_threads(1)
    yield


# ----------------------------------------------------------- conversions

def test_io_test_known_answers():
    """LACE's CSR->CSRL / CSR->CSRU known-answer tests
    (testing/test_matrix_io.cpp:605-735) on io_test.mtx."""
    row, col, val = G["io_row"], G["io_col"], G["io_val"]
    Lv = orc.split_lower(row, col, val, diag="value")
    assert np.array_equal(Lv.ptr, G["kat_csrl_rowcheck"].astype(int))
    assert np.array_equal(Lv.val, G["kat_csrl_valcheck"])
    Ur = orc.split_upper(row, col, val)
    assert np.array_equal(Ur.ptr, G["kat_csru_rowcheck"].astype(int))
    assert np.array_equal(Ur.val, G["kat_csru_valcheck"])
    # and the full LACE outputs, column indices included
    for tag, T in (("csrl_value", Lv), ("csrl_unity", orc.split_lower(row, col, val, "unity")), ("csru", Ur)):
        assert np.array_equal(T.ptr, G[f"io_{tag}_row"])
        assert np.array_equal(T.idx, G[f"io_{tag}_col"])
        assert np.array_equal(T.val, G[f"io_{tag}_val"])
    cp, ci, cv, _ = orc.transpose(Ur.ptr, Ur.idx, Ur.val, 4)
    assert np.array_equal(cp, G["io_cscu_row"]) and np.array_equal(ci, G["io_cscu_col"])
    assert np.array_equal(cv, G["io_cscu_val"])


def test_trefethen_generator_matches_lace_fixture():
    T = P.trefethen(19)
    assert T.n == 19 and T.nnz == 147
    # the factor patterns LACE built from its own copy of the file (golden)
    # are the generated matrix's: CSRL (unit diagonal last) and CSCU
    Lg = orc.split_lower(T.row, T.col, T.val, "unity")
    assert np.array_equal(Lg.ptr, G["tref_L_row"]) and np.array_equal(Lg.idx, G["tref_L_col"])
    F0 = orc.initial_factors(T.row, T.col, T.val)
    assert np.array_equal(F0.U.ptr, G["tref_U_ptr"]) and np.array_equal(F0.U.idx, G["tref_U_idx"])
    # the generated matrix is LACE's Trefethen_20 (checked against the file
    # itself when the LACE tree is present)
    if ref.available():
        n, _, r, c, v = ref.read_mtx(os.path.join(ref.REF_SRC, "testing/matrices/Trefethen_20.mtx"))
        assert np.array_equal(r, T.row) and np.array_equal(c, T.col) and np.array_equal(v, T.val)


# ------------------------------------------------------------------ ParILU

def test_parilu_async_equals_lace_trefethen():
    """data_PariLU_v0_3 (reduction 1e-15) on Trefethen_20: identical factors."""
    T = P.trefethen(19)
    F = orc.initial_factors(T.row, T.col, T.val)
    assert np.array_equal(F.L.ptr, G["tref_L_row"]) and np.array_equal(F.L.idx, G["tref_L_col"])
    assert np.array_equal(F.U.ptr, G["tref_U_ptr"]) and np.array_equal(F.U.idx, G["tref_U_idx"])
    sweeps = int(G["tref_parilu_log"][0])
    F = orc.parilu(T.row, T.col, T.val, sweeps, mode="async")
    assert np.array_equal(F.L.val, G["tref_L_val"])
    assert np.array_equal(F.U.val, G["tref_U_val"])
    res, nl = orc.zilures(T.row, T.col, T.val, orc.initial_factors(T.row, T.col, T.val))
    assert res == pytest.approx(G["tref_parilu_log"][3], rel=1e-14)
    assert nl == pytest.approx(G["tref_parilu_log"][4], rel=1e-14)
    res, nl = orc.zilures(T.row, T.col, T.val, F)
    assert res == pytest.approx(G["tref_zilures"][0], rel=1e-12)
    assert nl == pytest.approx(G["tref_zilures"][1], rel=1e-6, abs=1e-15)


@pytest.mark.parametrize("name", ["lap32", "cd8", "cd12"])
def test_parilu_prescribed_equals_lace(name):
    S = {"lap32": P.laplace2d(32), "cd8": P.convdiff3d(8), "cd12": P.convdiff3d(12)}[name]
    log = G[f"{name}_parilu_log"]
    F = orc.parilu(S.row, S.col, S.val, int(log[0]), mode="async")
    assert np.array_equal(F.L.val, G[f"{name}_L_val"])
    assert np.array_equal(F.U.val, G[f"{name}_U_val"])


def test_parilu_openmp_form_on_one_thread_equals_lace():
    """The OpenMP form of LACE's in-place sweep (the loop split statically
    over the threads, as LACE runs it; the CPU baseline) is LACE's one-thread
    sweep when it runs on one thread, and on several threads its residual
    stays at the same (rounding) level on these orderings."""
    S = P.convdiff3d(12)
    log = G["cd12_parilu_log"]
    try:
        orc.set_threads(1)
        F = orc.parilu(S.row, S.col, S.val, int(log[0]), mode="async_omp")
        assert np.array_equal(F.L.val, G["cd12_L_val"]) and np.array_equal(F.U.val, G["cd12_U_val"])
        orc.set_threads(4)
        F = orc.parilu(S.row, S.col, S.val, 3, mode="async_omp")
        assert orc.ilu_nonlinres(S.row, S.col, S.val, F) <= 1e-12 * np.linalg.norm(S.val)
    finally:
        orc.set_threads(os.cpu_count() or 1)


def test_sync_sweeps_converge_to_exact_ilu0():
    """The synchronous iteration's fixed point is LACE's (one-thread) ILU(0):
    residual on S(A) reaches rounding after enough sweeps."""
    A = P.laplace2d(16)
    E = orc.parilu(A.row, A.col, A.val, 1, mode="async")
    F = orc.parilu(A.row, A.col, A.val, 40, mode="sync")
    assert np.max(np.abs(F.L.val - E.L.val)) <= 1e-12 * np.max(np.abs(E.L.val))
    assert np.max(np.abs(F.U.val - E.U.val)) <= 1e-12 * np.max(np.abs(E.U.val))
    assert orc.ilu_nonlinres(A.row, A.col, A.val, F) <= 1e-12 * np.linalg.norm(A.val)


# ------------------------------------------------------------------ FGMRES

def test_fgmres_equals_lace_trefethen():
    """testing/test_linearSolver.cpp:621-726 with LACE's own factors: the
    restatement reproduces LACE's x, log, residual and orthogonality history."""
    T = P.trefethen(19)
    F = orc.Factors(orc.Tri(G["tref_L_row"], G["tref_L_col"], G["tref_L_val"]),
                    orc.Tri(G["tref_U_ptr"], G["tref_U_idx"], G["tref_U_val"]), [])
    for choice, kind in ((0, "trsv"), (1, "partrsv")):
        r = orc.fgmres({"kind": "csr", "row": T.row, "col": T.col, "val": T.val},
                       orc.ilu_precond(F, kind, tol=1.0), np.ones(T.n), search_max=20, restart_max=20,
                       rtol=1e-3, tol_type=0, monitor_orthog=True)
        lg = G[f"tref_fgmres{choice}_log"]
        assert r.info == int(lg[0])
        assert r.restarts == int(lg[1]) and r.search_directions == int(lg[2])
        assert r.initial_residual == lg[3] and r.final_residual == lg[4]
        assert np.array_equal(r.x, G[f"tref_fgmres{choice}_x"])
        assert np.array_equal(r.resid_hist, G[f"tref_fgmres{choice}_hist"])
        assert np.allclose(r.orth_hist, G[f"tref_fgmres{choice}_orth"], rtol=1e-15, atol=0)
        assert np.linalg.norm(np.ones(T.n) - T.matvec(r.x)) <= 1e-3


@pytest.mark.parametrize("name", ["lap32", "cd8", "cd12"])
def test_fgmres_equals_lace_synthetic(name):
    S = {"lap32": P.laplace2d(32), "cd8": P.convdiff3d(8), "cd12": P.convdiff3d(12)}[name]
    F = orc.initial_factors(S.row, S.col, S.val)
    F.L.val = G[f"{name}_L_val"]
    F.U.val = G[f"{name}_U_val"]
    lg = G[f"{name}_fgmres_log"]
    r = orc.fgmres({"kind": "csr", "row": S.row, "col": S.col, "val": S.val}, orc.ilu_precond(F),
                   G[f"{name}_b"], search_max=int(lg[5]), restart_max=50, rtol=1e-10, tol_type=1)
    assert r.restarts == int(lg[1]) and r.search_directions == int(lg[2])
    assert np.array_equal(r.x, G[f"{name}_fgmres_x"])
    assert np.array_equal(r.resid_hist, G[f"{name}_fgmres_hist"])


@pytest.mark.parametrize("restarted", [1, 0])
def test_fgmres_mgs_equals_lace_trefethen(restarted):
    """data_fgmres_restart (src/fgmres_restart.cpp) and data_fgmres
    (src/fgmres.cpp) on Trefethen_20 with LACE's factors: x, log, residual
    and orthogonality history reproduced exactly."""
    T = P.trefethen(19)
    F = orc.Factors(orc.Tri(G["tref_L_row"], G["tref_L_col"], G["tref_L_val"]),
                    orc.Tri(G["tref_U_ptr"], G["tref_U_idx"], G["tref_U_val"]), [])
    for choice, kind in ((0, "trsv"), (1, "partrsv")):
        r = orc.fgmres_mgs({"kind": "csr", "row": T.row, "col": T.col, "val": T.val},
                           orc.ilu_precond(F, kind, tol=1.0), np.ones(T.n), search_max=20, restart_max=20,
                           rtol=1e-3, tol_type=0, monitor_orthog=True, restarted=bool(restarted))
        k = f"tref_mgs{restarted}{choice}"
        lg = G[f"{k}_log"]
        assert r.info == int(lg[0])
        assert r.restarts == int(lg[1]) and r.search_directions == int(lg[2])
        assert r.initial_residual == lg[3] and r.final_residual == lg[4]
        assert np.array_equal(r.x, G[f"{k}_x"])
        assert np.array_equal(r.resid_hist, G[f"{k}_hist"])
        assert np.allclose(r.orth_hist, G[f"{k}_orth"], rtol=1e-15, atol=0)


@pytest.mark.parametrize("name", ["lap32", "cd8", "cd12"])
def test_fgmres_mgs_equals_lace_synthetic(name):
    """LACE's Gram-Schmidt FGMRES with restarts (lap32 restarts once; cd8
    reorthogonalises every direction, reorth = 2)."""
    S = {"lap32": P.laplace2d(32), "cd8": P.convdiff3d(8), "cd12": P.convdiff3d(12)}[name]
    F = orc.initial_factors(S.row, S.col, S.val)
    F.L.val = G[f"{name}_L_val"]
    F.U.val = G[f"{name}_U_val"]
    lg = G[f"{name}_mgs_log"]
    r = orc.fgmres_mgs({"kind": "csr", "row": S.row, "col": S.col, "val": S.val}, orc.ilu_precond(F),
                       G[f"{name}_b"], search_max=int(lg[5]), restart_max=50, rtol=1e-10, tol_type=1,
                       reorth=int(lg[6]))
    assert r.info == int(lg[0])
    assert r.restarts == int(lg[1]) and r.search_directions == int(lg[2])
    assert r.initial_residual == lg[3] and r.final_residual == lg[4]
    assert np.array_equal(r.x, G[f"{name}_mgs_x"])
    assert np.array_equal(r.resid_hist, G[f"{name}_mgs_hist"])


def blk2_system():
    """20 decoupled [[2,1],[1,2]] blocks (two eigenvalues): the second Krylov
    direction is already in the space, so LACE's Brown/Hindmarsh test
    reorthogonalises and (one cycle, DBL_EPSILON threshold) breaks down."""
    return P.CSR(40, G["blk2_row"], G["blk2_col"], G["blk2_val"])


@pytest.mark.parametrize("restarted", [1, 0])
@pytest.mark.parametrize("choice", [0, 2])
def test_fgmres_mgs_reorthogonalisation_equals_lace(restarted, choice):
    S = blk2_system()
    F = orc.parilu(S.row, S.col, S.val, 1, mode="async")
    k = f"blk2_mgs{restarted}{choice}"
    lg = G[f"{k}_log"]
    assert lg[5] == 1  # LACE reorthogonalised once
    r = orc.fgmres_mgs({"kind": "csr", "row": S.row, "col": S.col, "val": S.val},
                       orc.ilu_precond(F, "trsv" if choice == 0 else "none"), G["blk2_b"], search_max=10,
                       restart_max=3, rtol=1e-12, tol_type=1, restarted=bool(restarted))
    assert r.info == int(lg[0]) and r.search_directions == int(lg[2])
    assert r.initial_residual == lg[3] and r.final_residual == lg[4]
    assert np.array_equal(r.x, G[f"{k}_x"])
    assert np.array_equal(r.resid_hist, G[f"{k}_hist"])


@pytest.mark.parametrize("name", ["lap32", "cd8", "cd12"])
def test_parcsrtrsv_and_spmv_equal_lace(name):
    S = {"lap32": P.laplace2d(32), "cd8": P.convdiff3d(8), "cd12": P.convdiff3d(12)}[name]
    F = orc.initial_factors(S.row, S.col, S.val)
    F.L.val = G[f"{name}_L_val"]
    F.U.val = G[f"{name}_U_val"]
    Ur = F.U_csr()
    rhs = G[f"{name}_partrsv_rhs"]
    yl, itl = orc.parcsrtrsv(0, F.L.ptr, F.L.idx, F.L.val, rhs, tol=1.0)
    yu, itu = orc.parcsrtrsv(1, Ur.ptr, Ur.idx, Ur.val, rhs, tol=1e-20)
    assert np.array_equal(yl, G[f"{name}_partrsv_L"]) and np.array_equal(yu, G[f"{name}_partrsv_U"])
    assert [itl, itu] == list(G[f"{name}_partrsv_iters"])
    # one-thread ParCSRTRSV is an exact (Gauss-Seidel ordered) solve, summed
    # in a different order than the direct substitution
    ex = orc.trsv(F.L.ptr, F.L.idx, F.L.val, rhs, True, True)
    assert np.max(np.abs(yl - ex)) <= 1e-13 * np.max(np.abs(ex))
    xs, ys = G[f"{name}_spmv_in"]
    y = orc.spmv(S.row, S.col, S.val, xs, 1.25, -0.75, ys)
    assert np.array_equal(y, G[f"{name}_spmv_out"])


def test_givens_and_orthogonality_equal_lace():
    eps = float(np.nextafter(0.0, 1.0))
    for (a, b), (c, s) in zip(G["givens_in"], G["givens_out"]):
        assert orc.givens(a, b, eps) == (c, s)
    Q = G["orth_Q"]
    got = [orc.orthogonality_error(Q, s) for s in range(1, 13)]
    assert np.array_equal(np.array(got), G["orth_err"])


def test_bcsr_parilu_async_matches_lace():
    """BCSR ParILU (src/parilu_v0_3_bcsr.cpp): the restatement's block sweep
    (exact block inverse where LACE inverts iteratively) agrees to 1e-12."""
    B = P.bcsr3d(3, seed=11)
    Lr, Lc, Lv = G["bcsr3_L_0"], G["bcsr3_L_1"], G["bcsr3_L_2"]
    Up, Ui, Uv = G["bcsr3_U_0"], G["bcsr3_U_1"], G["bcsr3_U_2"]
    F = orc.initial_factors(B.row, B.col, np.arange(B.nblk, dtype=float))
    assert np.array_equal(F.L.ptr, Lr) and np.array_equal(F.L.idx, Lc)
    assert np.array_equal(F.U.ptr, Up) and np.array_equal(F.U.idx, Ui)
    rid = B.rowidx()
    bs, ld = B.bs, B.bs * B.bs
    A = B.val.reshape(B.nblk, ld)
    L = np.zeros((len(F.L.idx), ld))
    lrid = np.repeat(np.arange(B.nb), np.diff(F.L.ptr))
    for p in range(len(F.L.idx)):
        if F.L.idx[p] == lrid[p]:
            L[p] = np.eye(bs).ravel()
    lpos = {(lrid[p], F.L.idx[p]): p for p in range(len(F.L.idx))}
    ucid = np.repeat(np.arange(B.nb), np.diff(F.U.ptr))
    upos = {(F.U.idx[q], ucid[q]): q for q in range(len(F.U.idx))}
    U = np.zeros((len(F.U.idx), ld))
    for k in range(B.nblk):
        i, j = rid[k], B.col[k]
        if i > j:
            L[lpos[(i, j)]] = A[k]
        else:
            U[upos[(i, j)]] = A[k]
    Ld, Ud = L.ravel().copy(), U.ravel().copy()
    lib = orc.lib()
    for _ in range(int(G["bcsr3_sweeps"][0])):
        lib.orc_bcsr_parilu_sweep(0, bs, B.nblk, rid.astype(np.int32), B.col, A.ravel().copy(), F.L.ptr,
                                  F.L.idx, Ld, Ld, F.U.ptr, F.U.idx, Ud, Ud)
    assert np.max(np.abs(Ld - Lv)) <= 1e-12 * np.max(np.abs(Lv))
    assert np.max(np.abs(Ud - Uv)) <= 1e-12 * np.max(np.abs(Uv))


# ---------------------------------------------------------- live reference

needs_ref = pytest.mark.skipif(not ref.available(), reason="LACE source tree not present")


@needs_ref
@pytest.mark.parametrize("seed", [0, 1])
def test_live_reference_random_convdiff(seed):
    """Fresh inputs through LACE's own build and the restatement: bit-exact."""
    rng = np.random.default_rng(seed)
    S = P.convdiff3d(int(rng.integers(5, 9)), int(rng.integers(5, 9)), int(rng.integers(3, 6)),
                     pe=float(rng.uniform(0.5, 20)))
    Sm = ref.Mat.from_arrays(ref.Magma_CSR, S.n, S.n, S.row, S.col, S.val)
    import contextlib
    import io
    Lm, Um, log = ref.parilu(Sm, 1e-15, max_sweeps=3)
    F = orc.parilu(S.row, S.col, S.val, int(log["sweeps"]), mode="async")
    assert np.array_equal(Lm.arrays()[2], F.L.val) and np.array_equal(Um.arrays()[2], F.U.val)
    b = rng.standard_normal(S.n)
    Ucsr = ref.convert(Um, ref.Magma_CSC, ref.Magma_CSR)
    x, info, glog = ref.fgmres_householder_restart(Sm, b, np.zeros(S.n), Lm, Ucsr, search_max=7,
                                                   restart_max=30, rtol=1e-10, tol_type=1)
    r = orc.fgmres({"kind": "csr", "row": S.row, "col": S.col, "val": S.val}, orc.ilu_precond(F), b,
                   search_max=7, restart_max=30, rtol=1e-10, tol_type=1)
    assert np.array_equal(x, r.x)
    assert r.search_directions == glog["search_directions"] and r.restarts == glog["restarts"]
    del contextlib, io


@needs_ref
@pytest.mark.parametrize("restarted", [True, False])
def test_live_reference_fgmres_mgs(restarted):
    """Fresh inputs through LACE's Gram-Schmidt FGMRES and the restatement."""
    rng = np.random.default_rng(7)
    S = P.convdiff3d(7, 6, 5, pe=float(rng.uniform(0.5, 20)))
    Sm = ref.Mat.from_arrays(ref.Magma_CSR, S.n, S.n, S.row, S.col, S.val)
    Lm, Um, log = ref.parilu(Sm, 1e-15, max_sweeps=3)
    F = orc.parilu(S.row, S.col, S.val, int(log["sweeps"]), mode="async")
    b = rng.standard_normal(S.n)
    Ucsr = ref.convert(Um, ref.Magma_CSC, ref.Magma_CSR)
    x, info, glog = ref.fgmres_mgs(Sm, b, np.zeros(S.n), Lm, Ucsr, search_max=6, restart_max=30, rtol=1e-10,
                                   tol_type=1, restarted=restarted)
    r = orc.fgmres_mgs({"kind": "csr", "row": S.row, "col": S.col, "val": S.val}, orc.ilu_precond(F), b,
                       search_max=6, restart_max=30, rtol=1e-10, tol_type=1, restarted=restarted)
    assert np.array_equal(x, r.x) and info == r.info
    assert r.search_directions == glog["search_directions"] and r.restarts == glog["restarts"]


@needs_ref
def test_live_reference_block_inverse():
    a = np.eye(5) * 5 + 0.1 * np.random.default_rng(0).standard_normal((5, 5))
    assert np.allclose(ref.dense_inverse(a), orc.block_inverse(a), rtol=1e-12, atol=1e-14)


def _zilures_bcsr_cases():
    """(A scalar CSR, L triple, U triple, bs) for data_zilures_bcsr: LACE's
    own factor layout (BCSRL, and BCSCU read as BCSR as LACE does), U as
    genuine block rows, and random block patterns."""
    B = P.bcsr3d(3, seed=2)
    A = B.to_csr()
    F = orc.bcsr_parilu(B, 1, mode="async")
    L = (F.L.ptr, F.L.idx, F.L.val)
    U_bcsc = (F.U.ptr, F.U.idx, F.U.val)
    # the same U with its blocks gathered by block row
    nb = B.nb
    cols = np.repeat(np.arange(nb), np.diff(F.U.ptr))
    order = np.lexsort((cols, F.U.idx))
    rp = np.zeros(nb + 1, dtype=np.int32)
    np.cumsum(np.bincount(F.U.idx, minlength=nb), out=rp[1:])
    U_bcsr = (rp, cols[order].astype(np.int32), np.asarray(F.U.val).reshape(-1, B.bs, B.bs)[order])
    rng = np.random.default_rng(5)
    def rand_bcsr(nb, bs, per_row):
        ptr = [0]
        idx = []
        for _ in range(nb):
            c = sorted(set(rng.integers(0, nb, size=per_row).tolist()))
            idx += c
            ptr.append(len(idx))
        return (np.array(ptr, np.int32), np.array(idx, np.int32), rng.standard_normal((len(idx), bs, bs)))
    R = P.bcsr3d(2, bs=3, seed=7)
    return {"lace_layout": (A, L, U_bcsc, B.bs), "bcsr_u": (A, L, U_bcsr, B.bs),
            "random": (R.to_csr(), rand_bcsr(R.nb, 3, 3), rand_bcsr(R.nb, 3, 4), 3)}


@needs_ref
@pytest.mark.parametrize("case", ["lace_layout", "bcsr_u", "random"])
def test_live_reference_zilures_bcsr(case):
    """The oracle's data_zilures_bcsr against LACE's own (control/norms.cpp:
    409-468) built here."""
    A, L, U, bs = _zilures_bcsr_cases()[case]
    Am = ref.Mat.from_arrays(ref.Magma_CSR, A.n, A.n, A.row, A.col, A.val)
    nb = len(L[0]) - 1
    Lm = ref.Mat.from_arrays(ref.Magma_BCSR, nb, nb, L[0], L[1], np.asarray(L[2]).ravel(), blocksize=bs)
    Um = ref.Mat.from_arrays(ref.Magma_BCSR, nb, nb, U[0], U[1], np.asarray(U[2]).ravel(), blocksize=bs)
    r_ref, nl_ref = ref.zilures_bcsr(Am, Lm, Um)
    r, nl = orc.zilures_bcsr(A.row, A.col, A.val, L, U, bs)
    assert r == pytest.approx(r_ref, rel=1e-12)
    assert nl == pytest.approx(nl_ref, rel=1e-10, abs=1e-13 * r_ref)
    if case == "bcsr_u":  # the genuine product: block ILU(0) after one in-place sweep
        assert nl < 1e-10 * r
