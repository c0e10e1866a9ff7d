"""Generate tests/golden/lace_golden.npz from LACE's own implementation.

Runs LACE's unmodified sources, compiled by `make -C oracle ref` from the
LACE source tree (the tree oracle/Makefile reads; LACE_REF_SRC overrides),
on small inputs and stores
inputs and outputs as fixtures.  The inputs are this project's seeded
synthetic systems plus two of LACE's own tiny test fixtures
(testing/matrices/io_test.mtx, 4x4; the Trefethen_20 matrix, which is also
generated here from its definition and checked against LACE's copy).  The
expected arrays of LACE's CSR->CSRL/CSRU known-answer tests
(testing/test_matrix_io.cpp:605-735) are read from that test source as text.

Run:  python tests/golden/make_golden.py
"""
from __future__ import annotations

import os
import re
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from lace_gb300 import problems as P  # noqa: E402
from oracle import reference as ref  # noqa: E402

OUT = os.path.join(HERE, "lace_golden.npz")


class CaptureStdout:
    """fd-level capture of what LACE's C code prints."""

    def __enter__(self):
        sys.stdout.flush()
        self.tmp = tempfile.TemporaryFile(mode="w+b")
        self.saved = os.dup(1)
        os.dup2(self.tmp.fileno(), 1)
        return self

    def __exit__(self, *a):
        sys.stdout.flush()
        try:
            import ctypes
            ctypes.CDLL(None).fflush(None)
        except Exception:
            pass
        os.dup2(self.saved, 1)
        os.close(self.saved)
        self.tmp.seek(0)
        self.text = self.tmp.read().decode(errors="replace")
        self.tmp.close()


def hist_from(text: str, tag: str = "mkltrsv", solver: str = "FGMRES_Householders_") -> np.ndarray:
    """|g_{j+1}| per search direction as LACE prints it (solver: the printed
    prefix, "FGMRES_" for the Gram-Schmidt FGMRES)."""
    vals = re.findall(rf"{solver}{tag}_search\((\d+)\) = ([-+0-9.eE]+);", text)
    return np.array([float(v) for _, v in vals])


def orth_from(text: str, tag: str = "mkltrsv", solver: str = "FGMRES_Householders_") -> np.ndarray:
    vals = re.findall(rf"{solver}{tag}_ortherr\((\d+)\) = ([-+0-9.eE]+);", text)
    return np.array([float(v) for _, v in vals])


def kat_arrays(src: str, name: str):
    m = re.search(rf"{name}\[\d+\] = \{{([^}}]*)\}}", src)
    return np.array([float(t) for t in m.group(1).replace("\n", " ").split(",")])


def csr_of(A):
    return ref.Mat.from_arrays(ref.Magma_CSR, A.n, A.n, A.row, A.col, A.val)


def main():
    if not ref.available():
        raise SystemExit("LACE sources / oracle/_ref not available")
    g = {}
    # ---------------------------------------------------------- io_test KAT
    n, _, row, col, val = ref.read_mtx(os.path.join(ref.REF_SRC, "testing/matrices/io_test.mtx"))
    g["io_row"], g["io_col"], g["io_val"] = row, col, val
    A = ref.Mat.from_arrays(ref.Magma_CSR, n, n, row, col, val)
    for tag, fmt, diag in (("csrl_value", ref.Magma_CSRL, ref.Magma_VALUE),
                           ("csrl_unity", ref.Magma_CSRL, ref.Magma_UNITY),
                           ("csru", ref.Magma_CSRU, 0), ("cscu", ref.Magma_CSCU, ref.Magma_VALUE)):
        B = ref.convert(A, ref.Magma_CSR, fmt, diag)
        r, c, v = B.arrays()
        g[f"io_{tag}_row"], g[f"io_{tag}_col"], g[f"io_{tag}_val"] = r, c, v
    src = open(os.path.join(ref.REF_SRC, "testing/test_matrix_io.cpp")).read()
    for k in ("csrl_rowcheck", "csrl_valcheck", "csru_rowcheck", "csru_valcheck"):
        g[f"kat_{k}"] = kat_arrays(src, k)

    # -------------------------------------------------------- Trefethen_20
    T = P.trefethen(19)
    nt, _, tr, tc, tv = ref.read_mtx(os.path.join(ref.REF_SRC, "testing/matrices/Trefethen_20.mtx"))
    assert nt == T.n and np.array_equal(tr, T.row) and np.array_equal(tc, T.col) and np.array_equal(tv, T.val)
    Tm = csr_of(T)
    with CaptureStdout():
        Lm, Um, log = ref.parilu(Tm, 1e-15)
    g["tref_L_row"], g["tref_L_col"], g["tref_L_val"] = Lm.arrays()
    g["tref_U_ptr"], g["tref_U_idx"], g["tref_U_val"] = Um.arrays()
    g["tref_parilu_log"] = np.array([log["sweeps"], log["tol"], log["A_Frobenius"], log["initial_residual"],
                                     log["initial_nonlinear_residual"]])
    g["tref_zilures"] = np.array(ref.zilures(Tm, Lm, Um))
    M = csr_of(T)
    ref.csrilu0(M)
    Lk = ref.convert(M, ref.Magma_CSR, ref.Magma_CSRL, ref.Magma_UNITY)
    Uk = ref.convert(M, ref.Magma_CSR, ref.Magma_CSCU, ref.Magma_VALUE)
    g["tref_mkl_zilures"] = np.array(ref.zilures(Tm, Lk, Uk))
    Ucsr = ref.convert(Um, ref.Magma_CSC, ref.Magma_CSR)
    ref.set_storage(Ucsr, ref.Magma_CSRU)  # as testing/test_linearSolver.cpp:671 does
    Lt, Ut = Lm, Ucsr  # Trefethen_20's factors, for the Gram-Schmidt FGMRES below
    for choice in (0, 1):
        with CaptureStdout() as cap:
            x, info, glog = ref.fgmres_householder_restart(Tm, np.ones(T.n), np.zeros(T.n), Lm, Ucsr,
                                                           search_max=20, restart_max=20, rtol=1e-3,
                                                           tol_type=0, choice=choice, monitor_orthog=1)
        tag = "mkltrsv" if choice == 0 else "partrsv"
        g[f"tref_fgmres{choice}_x"] = x
        g[f"tref_fgmres{choice}_log"] = np.array([info, glog["restarts"], glog["search_directions"],
                                                  glog["initial_residual"], glog["final_residual"]])
        g[f"tref_fgmres{choice}_hist"] = hist_from(cap.text, tag)
        g[f"tref_fgmres{choice}_orth"] = orth_from(cap.text, tag)

    # ------------------------------------- synthetic systems, LACE's own path
    systems = {"lap32": (P.laplace2d(32), None, 30, 5), "cd8": (P.convdiff3d(8), 0, 20, 3),
               "cd12": (P.convdiff3d(12), 0, 30, 3)}
    for name, (S, seed, m, sweeps) in systems.items():
        b = S.matvec(np.ones(S.n)) if seed is None else P.rhs_normal(S.n, seed)
        Sm = csr_of(S)
        g[f"{name}_b"] = b
        with CaptureStdout():
            Lm, Um, log = ref.parilu(Sm, 1e-15, max_sweeps=sweeps)
        g[f"{name}_L_val"] = Lm.arrays()[2]
        g[f"{name}_U_val"] = Um.arrays()[2]
        g[f"{name}_parilu_log"] = np.array([log["sweeps"], log["finalStep"], log["A_Frobenius"],
                                            log["initial_residual"], log["initial_nonlinear_residual"]])
        Ucsr = ref.convert(Um, ref.Magma_CSC, ref.Magma_CSR)
        with CaptureStdout() as cap:
            x, info, glog = ref.fgmres_householder_restart(Sm, b, np.zeros(S.n), Lm, Ucsr, search_max=m,
                                                           restart_max=50, rtol=1e-10, tol_type=1, choice=0)
        g[f"{name}_fgmres_x"] = x
        g[f"{name}_fgmres_log"] = np.array([info, glog["restarts"], glog["search_directions"],
                                            glog["initial_residual"], glog["final_residual"], m])
        g[f"{name}_fgmres_hist"] = hist_from(cap.text)
        # the same system through LACE's FGMRES with modified Gram-Schmidt
        # (src/fgmres_restart.cpp); cd8 with reorthogonalisation always on
        reorth = 2 if name == "cd8" else 0
        with CaptureStdout() as cap:
            x, info, glog = ref.fgmres_mgs(Sm, b, np.zeros(S.n), Lm, Ucsr, search_max=m, restart_max=50,
                                           rtol=1e-10, tol_type=1, choice=0, reorth=reorth)
        g[f"{name}_mgs_x"] = x
        g[f"{name}_mgs_log"] = np.array([info, glog["restarts"], glog["search_directions"],
                                         glog["initial_residual"], glog["final_residual"], m, reorth])
        g[f"{name}_mgs_hist"] = hist_from(cap.text, solver="FGMRES_")
        # LACE's ParCSRTRSV on these factors (tol 1.0 as FGMRES uses it)
        rng = np.random.default_rng(5)
        rhs = rng.standard_normal(S.n)
        lr, lc, lv = Lm.arrays()
        ur, uc, uv = Ucsr.arrays()
        with CaptureStdout():
            yl, itl, _ = ref.parcsrtrsv(ref.MagmaLower, ref.Magma_CSRL, ref.Magma_UNITY, lr, lc, lv, rhs, tol=1.0)
            yu, itu, _ = ref.parcsrtrsv(ref.MagmaUpper, ref.Magma_CSRU, ref.Magma_VALUE, ur, uc, uv, rhs,
                                        tol=1e-20)
        g[f"{name}_partrsv_rhs"] = rhs
        g[f"{name}_partrsv_L"] = yl
        g[f"{name}_partrsv_U"] = yu
        g[f"{name}_partrsv_iters"] = np.array([itl, itu])
        # data_z_spmv
        xs = rng.standard_normal(S.n)
        ys = rng.standard_normal(S.n)
        y, _ = ref.spmv(Sm, xs, alpha=1.25, beta=-0.75, y=ys)
        g[f"{name}_spmv_in"] = np.stack([xs, ys])
        g[f"{name}_spmv_out"] = y

    # ------------------------- FGMRES with modified Gram-Schmidt (LACE)
    # Trefethen_20 as in the Householder case above: data_fgmres_restart
    # (restarted 1) and data_fgmres (restarted 0), exact solves and ParCSRTRSV
    for restarted in (1, 0):
        for choice in (0, 1):
            with CaptureStdout() as cap:
                x, info, glog = ref.fgmres_mgs(Tm, np.ones(T.n), np.zeros(T.n), Lt, Ut, search_max=20,
                                               restart_max=20, rtol=1e-3, tol_type=0, choice=choice,
                                               monitor_orthog=1, restarted=bool(restarted))
            tag = "mkltrsv" if choice == 0 else "partrsv"
            k = f"tref_mgs{restarted}{choice}"
            g[f"{k}_x"] = x
            g[f"{k}_log"] = np.array([info, glog["restarts"], glog["search_directions"],
                                      glog["initial_residual"], glog["final_residual"]])
            g[f"{k}_hist"] = hist_from(cap.text, tag, "FGMRES_")
            g[f"{k}_orth"] = orth_from(cap.text, tag, "FGMRES_")
    # Brown/Hindmarsh reorthogonalisation and happy breakdown: 20 decoupled
    # [[2,1],[1,2]] blocks have two eigenvalues, so the second direction is
    # already in the Krylov space (LACE prints "Reorthogonalize")
    nb2 = 40
    r2 = np.repeat(np.arange(nb2, dtype=np.int32), 2)
    c2 = np.array([[i - i % 2, i - i % 2 + 1] for i in range(nb2)], dtype=np.int32).ravel()
    v2 = np.array([[2.0, 1.0] if i % 2 == 0 else [1.0, 2.0] for i in range(nb2)]).ravel()
    B2 = P.CSR(nb2, np.concatenate([[0], np.cumsum(np.bincount(r2, minlength=nb2))]).astype(np.int32), c2, v2)
    g["blk2_row"], g["blk2_col"], g["blk2_val"] = B2.row, B2.col, B2.val
    g["blk2_b"] = b2 = np.random.default_rng(3).standard_normal(nb2)
    B2m = csr_of(B2)
    with CaptureStdout():
        L2, U2, _ = ref.parilu(B2m, 1e-15)
    U2c = ref.convert(U2, ref.Magma_CSC, ref.Magma_CSR)
    for restarted in (1, 0):
        for choice in (0, 2):
            with CaptureStdout() as cap:
                x, info, glog = ref.fgmres_mgs(B2m, b2, np.zeros(nb2), L2, U2c, search_max=10, restart_max=3,
                                               rtol=1e-12, tol_type=1, choice=choice, restarted=bool(restarted))
            k = f"blk2_mgs{restarted}{choice}"
            g[f"{k}_x"] = x
            g[f"{k}_log"] = np.array([info, glog["restarts"], glog["search_directions"],
                                      glog["initial_residual"], glog["final_residual"],
                                      cap.text.count("Reorthogonalize"), cap.text.count("happy breakdown")])
            g[f"{k}_hist"] = hist_from(cap.text, "mkltrsv" if choice == 0 else "partrsv", "FGMRES_")

    # --------------------------------------------------- BCSR ParILU (LACE)
    B = P.bcsr3d(3, seed=11)
    Bm = ref.Mat.from_arrays(ref.Magma_BCSR, B.nb, B.nb, B.row, B.col, B.val, blocksize=B.bs,
                             L=ref.lib_bcsr())
    with CaptureStdout():
        Lb, Ub, blog = ref.bcsr_parilu(Bm, 1e-28)
    g["bcsr3_L"] = Lb.arrays(B.nb + 1)
    g["bcsr3_U"] = Ub.arrays(B.nb + 1)
    g["bcsr3_sweeps"] = np.array([blog["sweeps"]])

    # ------------------------------------------- Givens / orthogonality KATs
    rng = np.random.default_rng(9)
    pairs = [(3.0, 4.0), (4.0, -3.0), (0.0, 2.0), (1e-300, 1e-310), (2.0, 0.0), (-1.5, 2.5)]
    pairs += [tuple(v) for v in rng.standard_normal((10, 2))]
    eps = float(np.nextafter(0.0, 1.0))
    g["givens_in"] = np.array(pairs)
    g["givens_out"] = np.array([ref.givens(a, b, eps) for a, b in pairs])
    Q = np.linalg.qr(rng.standard_normal((300, 12)))[0].T.copy()
    Q[3] += 1e-7 * rng.standard_normal(300)
    g["orth_Q"] = Q
    g["orth_err"] = np.array([ref.orthogonality_error(Q, s) for s in range(1, 13)])

    # ---------------------------------------- Matrix Market files (LACE's IO)
    # LACE's own reader and writer on generated files: SHA-256 digests of the
    # arrays read and of the files written (row- and column-major)
    sys.path.insert(0, os.path.dirname(HERE))
    import mtx_cases as MC
    tmp = tempfile.mkdtemp()
    texts = dict(MC.cases())
    texts["large"] = MC.large_text()
    for name, text in texts.items():
        fn = os.path.join(tmp, name + ".mtx")
        with open(fn, "w", newline="") as f:
            f.write(text)
        with CaptureStdout():
            info, nr, nc, r, c, v = ref.read_csr_mtx(fn)
        g[f"mtx_{name}_info"] = np.array([info])
        if info != 0:
            continue
        g[f"mtx_{name}_read"] = np.array([MC.digest_arrays(nr, nc, r, c, v)])
        if "symmetric" not in text.split("\n", 1)[0].lower() and "hermitian" not in text.split("\n", 1)[0].lower():
            with CaptureStdout():
                ci, cnr, cnc, crr, ccc, cvv = ref.read_coo_mtx(fn)
            g[f"mtx_{name}_coo"] = np.array([MC.digest_arrays(cnr, cnc, crr, ccc, cvv)])
        Am = ref.Mat.from_arrays(ref.Magma_CSR, nr, nc, r, c, v)
        for major in ((101, 102) if nr == nc else (101,)):  # LACE's transpose asserts on non-square input
            out = fn + ".%d" % major
            with CaptureStdout():
                ref.write_csr_mtx(Am, out, major)
            g[f"mtx_{name}_write{major}"] = np.array([MC.digest_file(out)])
    # ------------------------ setup conversions (LACE's data_zmconvert etc.)
    # digests of every field and array of LACE's output for each job
    import convert_cases as CC
    from test_convert import run_lace
    for key, *_ in CC.jobs():
        with CaptureStdout():
            g[key] = np.array([CC.digest(run_lace(key))])
    n, r, c, v = MC.write_values_matrix()
    Am = ref.Mat.from_arrays(ref.Magma_CSR, n, n, r, c, v)
    for major in (101, 102):
        out = os.path.join(tmp, "values.%d" % major)
        with CaptureStdout():
            ref.write_csr_mtx(Am, out, major)
        g[f"mtx_values_write{major}"] = np.array([MC.digest_file(out)])

    np.savez_compressed(OUT, **{k: np.asarray(v) for k, v in g.items() if not isinstance(v, tuple)},
                        **{f"{k}_{i}": np.asarray(a) for k, v in g.items() if isinstance(v, tuple)
                           for i, a in enumerate(v)})
    print(f"wrote {OUT}: {os.path.getsize(OUT)} bytes, {len(g)} entries")


if __name__ == "__main__":
    main()
