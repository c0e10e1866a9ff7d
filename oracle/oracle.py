"""Python face of the CPU oracle (TEST INFRASTRUCTURE).

Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg may
import this module, as the checker or the timed CPU baseline; the lace_gb300
product never does.

Structural conversions are restated in numpy here (integer work); the
numeric iterations call the C restatement in lace_oracle.c.  Each function
names the LACE source lines it follows.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess
from dataclasses import dataclass

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_build", "liblace_oracle.so")

_lib = None


def build() -> str:
    subprocess.run(["make", "-s", "-C", HERE], check=True)
    return LIB_PATH


def lib() -> C.CDLL:
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            build()
        _lib = C.CDLL(LIB_PATH)
        _setup(_lib)
    return _lib


_ip = np.ctypeslib.ndpointer(dtype=np.int32, flags="C_CONTIGUOUS")
_dp = np.ctypeslib.ndpointer(dtype=np.float64, flags="C_CONTIGUOUS")
_fp = np.ctypeslib.ndpointer(dtype=np.float32, flags="C_CONTIGUOUS")


class OrcOperator(C.Structure):
    _fields_ = [("kind", C.c_int), ("n", C.c_int), ("bs", C.c_int),
                ("row", C.c_void_p), ("col", C.c_void_p), ("val", C.c_void_p)]


class OrcPrecond(C.Structure):
    _fields_ = [("kind", C.c_int),
                ("t1_row", C.c_void_p), ("t1_col", C.c_void_p), ("t1_val", C.c_void_p),
                ("t1_val32", C.c_void_p), ("t1_lower", C.c_int), ("t1_unit", C.c_int),
                ("t2_row", C.c_void_p), ("t2_col", C.c_void_p), ("t2_val", C.c_void_p),
                ("t2_val32", C.c_void_p), ("t2_lower", C.c_int), ("t2_unit", C.c_int),
                ("bdinv", C.c_void_p), ("bdinv32", C.c_void_p),
                ("tol", C.c_double), ("max_sweeps", C.c_int)]


class OrcGmresPar(C.Structure):
    _fields_ = [("search_max", C.c_int), ("restart_max", C.c_int), ("tol_type", C.c_int),
                ("rtol", C.c_double), ("monitor_orthog", C.c_int), ("reorth", C.c_int)]


class OrcGmresLog(C.Structure):
    _fields_ = [("restarts", C.c_int), ("search_directions", C.c_int),
                ("total_iterations", C.c_int), ("initial_residual", C.c_double),
                ("final_residual", C.c_double), ("converged", C.c_int),
                ("lost_update", C.c_int), ("info", C.c_int)]


def _setup(L: C.CDLL) -> None:
    L.orc_set_threads.argtypes = [C.c_int]
    L.orc_parilu_sweep.restype = C.c_double
    L.orc_parilu_sweep.argtypes = [C.c_int, C.c_int, _ip, _ip, _dp, _ip, _ip, _dp, _dp, _ip, _ip, _dp, _dp]
    L.orc_parilu_sweep_sync_f32.restype = C.c_double
    L.orc_parilu_sweep_sync_f32.argtypes = [C.c_int, _ip, _ip, _dp, _ip, _ip, _fp, _fp, _ip, _ip, _fp, _fp]
    L.orc_ilu_nonlinres.restype = C.c_double
    L.orc_ilu_nonlinres.argtypes = [C.c_int, _ip, _ip, _dp, _ip, _ip, _dp, _ip, _ip, _dp]
    L.orc_zilures.argtypes = [C.c_int, _ip, _ip, _dp, _ip, _ip, _dp, _ip, _ip, _dp,
                              C.POINTER(C.c_double), C.POINTER(C.c_double)]
    L.orc_spmv.argtypes = [C.c_int, _ip, _ip, _dp, C.c_double, _dp, C.c_double, _dp]
    L.orc_bcsr_spmv.argtypes = [C.c_int, C.c_int, _ip, _ip, _dp, _dp, _dp]
    L.orc_trsv.argtypes = [C.c_int, _ip, _ip, _dp, C.c_int, C.c_int, _dp, _dp]
    L.orc_trsv_f32.argtypes = [C.c_int, _ip, _ip, _fp, C.c_int, C.c_int, _fp, _fp]
    L.orc_levels.restype = C.c_int
    L.orc_levels.argtypes = [C.c_int, _ip, _ip, C.c_int, _ip]
    L.orc_parcsrtrsv.argtypes = [C.c_int, C.c_int, _dp, _ip, _ip, _dp, _dp, C.c_double, C.POINTER(C.c_int)]
    L.orc_jacobi_trsv.argtypes = [C.c_int, C.c_int, _dp, _ip, _ip, _dp, _dp, C.c_double, C.c_int,
                                  C.POINTER(C.c_int)]
    L.orc_bcsr_parilu_sweep.restype = C.c_double
    L.orc_bcsr_parilu_sweep.argtypes = [C.c_int, C.c_int, C.c_int, _ip, _ip, _dp, _ip, _ip, _dp, _dp,
                                        _ip, _ip, _dp, _dp]
    L.orc_block_inverse.restype = C.c_int
    L.orc_block_inverse.argtypes = [C.c_int, _dp, _dp]
    L.orc_bcsr_trsv_lower_unit.argtypes = [C.c_int, C.c_int, _ip, _ip, _dp, _dp, _dp]
    L.orc_bcsr_trsv_upper.argtypes = [C.c_int, C.c_int, _ip, _ip, _dp, _dp, _dp, _dp]
    L.orc_givens.argtypes = [C.c_double, C.c_double, C.c_double, C.POINTER(C.c_double), C.POINTER(C.c_double)]
    L.orc_orthogonality_error.restype = C.c_double
    L.orc_orthogonality_error.argtypes = [C.c_int, C.c_int, _dp, C.c_int]
    L.orc_fgmres_householder.restype = C.c_int
    L.orc_fgmres_householder.argtypes = [C.POINTER(OrcOperator), C.POINTER(OrcPrecond), _dp, _dp,
                                         C.POINTER(OrcGmresPar), C.POINTER(OrcGmresLog), C.c_void_p,
                                         C.c_void_p]
    L.orc_fgmres_mgs.restype = C.c_int
    L.orc_fgmres_mgs.argtypes = [C.POINTER(OrcOperator), C.POINTER(OrcPrecond), _dp, _dp,
                                 C.POINTER(OrcGmresPar), C.c_int, C.POINTER(OrcGmresLog), C.c_void_p,
                                 C.c_void_p]


def set_threads(n: int) -> None:
    lib().orc_set_threads(int(n))


def _i(a):
    return np.ascontiguousarray(a, dtype=np.int32)


def _d(a):
    return np.ascontiguousarray(a, dtype=np.float64)


# --------------------------------------------------------------- structure

@dataclass
class Tri:
    """A triangular factor in compressed form: ptr/idx/val (CSR or CSC)."""

    ptr: np.ndarray
    idx: np.ndarray
    val: np.ndarray


def split_lower(row, col, val, diag: str = "unity") -> Tri:
    """CSR -> CSRL (control/magma_zmconverter.cpp:304-379): strict lower part
    plus the diagonal, which stays last in its row; diag 'unity' writes 1.0,
    'value' keeps a_ii."""
    n = len(row) - 1
    rid = np.repeat(np.arange(n, dtype=np.int32), np.diff(row))
    keep = col <= rid
    ptr = np.zeros(n + 1, dtype=np.int32)
    np.cumsum(np.bincount(rid[keep], minlength=n), out=ptr[1:])
    v = _d(val[keep]).copy()
    if diag == "unity":
        v[col[keep] == rid[keep]] = 1.0
    return Tri(ptr, _i(col[keep]), v)


def split_upper(row, col, val) -> Tri:
    """CSR -> CSRU (control/magma_zmconverter.cpp:381-460): diagonal first."""
    n = len(row) - 1
    rid = np.repeat(np.arange(n, dtype=np.int32), np.diff(row))
    keep = col >= rid
    ptr = np.zeros(n + 1, dtype=np.int32)
    np.cumsum(np.bincount(rid[keep], minlength=n), out=ptr[1:])
    return Tri(ptr, _i(col[keep]), _d(val[keep]).copy())


def transpose(ptr, idx, val, ncols: int | None = None):
    """CSR <-> CSC by a stable counting sort (control/magma_zmtranspose.cpp:85):
    the entries of each output row keep increasing input-row order.
    Returns (ptr, idx, val, perm) with out.val = in.val[perm]."""
    n = len(ptr) - 1
    m = n if ncols is None else ncols
    rid = np.repeat(np.arange(n, dtype=np.int32), np.diff(ptr))
    perm = np.lexsort((rid, idx)).astype(np.int64)
    optr = np.zeros(m + 1, dtype=np.int32)
    np.cumsum(np.bincount(idx, minlength=m), out=optr[1:])
    return optr, _i(rid[perm]), val[perm] if val is not None else None, perm


def lumerge(L: Tri, Ur: Tri):
    """data_zmlumerge (control/magma_zmlumerge.cpp:43-109): per row the strict
    lower entries of L then all entries of U (CSR)."""
    n = len(L.ptr) - 1
    lr = np.repeat(np.arange(n, dtype=np.int32), np.diff(L.ptr))
    ur = np.repeat(np.arange(n, dtype=np.int32), np.diff(Ur.ptr))
    ks = L.idx < lr
    rows = np.concatenate([lr[ks], ur])
    cols = np.concatenate([L.idx[ks], Ur.idx])
    vals = np.concatenate([L.val[ks], Ur.val])
    order = np.lexsort((cols, rows))
    ptr = np.zeros(n + 1, dtype=np.int32)
    np.cumsum(np.bincount(rows, minlength=n), out=ptr[1:])
    return ptr, _i(cols[order]), _d(vals[order])


# --------------------------------------------------------------- ParILU

@dataclass
class Factors:
    L: Tri          # CSRL, unit diagonal last
    U: Tri          # CSCU: column pointers / row indices, diagonal last
    steps: list

    def U_csr(self) -> Tri:
        n = len(self.U.ptr) - 1
        ptr, idx, val, _ = transpose(self.U.ptr, self.U.idx, self.U.val, n)
        return Tri(ptr, idx, val)


def initial_factors(row, col, val) -> Factors:
    """A-initial guess of src/parilu_v0_3.cpp:22-27: L = strict-lower(A) + I
    (CSRL, UNITY), U = upper(A) (CSCU)."""
    L = split_lower(row, col, val, "unity")
    Ur = split_upper(row, col, val)
    n = len(row) - 1
    ptr, idx, v, _ = transpose(Ur.ptr, Ur.idx, Ur.val, n)
    return Factors(L, Tri(ptr, idx, v), [])


def parilu(row, col, val, sweeps: int, mode: str = "sync", f32: bool = False,
           stop_eps: bool = False) -> Factors:
    """`sweeps` ParILU(0) sweeps from the A-initial guess.  mode 'async' is
    LACE's in-place sweep (src/parilu_v0_3.cpp:62-108, one-thread order);
    'async_omp' the same loop split statically over the OpenMP threads, as
    LACE runs it (racy across the threads' ranges, so not reproducible);
    'sync' the Jacobi form.  stop_eps mirrors the prescribed-sweeps stop
    (step <= 4*eps, src/parilu_v0_3_prescribedSweeps.cpp:62). Steps recorded
    are normalised by ||A||_F (:104)."""
    F = initial_factors(row, col, val)
    rid = np.repeat(np.arange(len(row) - 1, dtype=np.int32), np.diff(row))
    anorm = float(np.sqrt(np.sum(np.asarray(val) ** 2)))
    lb = lib()
    col = _i(col)
    val = _d(val)
    if f32:
        Lc = F.L.val.astype(np.float32)
        Uc = F.U.val.astype(np.float32)
    else:
        Lc = F.L.val.copy()
        Uc = F.U.val.copy()
    Ln = Lc.copy()
    Un = Uc.copy()
    step = np.finfo(np.float64).max
    it = 0
    while it < sweeps and (not stop_eps or step > 4.0 * np.finfo(np.float64).eps):
        if f32:
            s = lb.orc_parilu_sweep_sync_f32(len(col), rid, col, val, F.L.ptr, F.L.idx, Lc, Ln,
                                             F.U.ptr, F.U.idx, Uc, Un)
            Lc, Ln = Ln, Lc
            Uc, Un = Un, Uc
            Ln[:] = Lc
            Un[:] = Uc
        elif mode in ("async", "async_omp"):
            s = lb.orc_parilu_sweep(0 if mode == "async" else 2, len(col), rid, col, val, F.L.ptr, F.L.idx, Lc,
                                    Lc, F.U.ptr, F.U.idx, Uc, Uc)
        else:
            s = lb.orc_parilu_sweep(1, len(col), rid, col, val, F.L.ptr, F.L.idx, Lc, Ln,
                                    F.U.ptr, F.U.idx, Uc, Un)
            Lc, Ln = Ln, Lc
            Uc, Un = Un, Uc
            Ln[:] = Lc
            Un[:] = Uc
        step = s / anorm
        F.steps.append(step)
        it += 1
    F.L.val = Lc
    F.U.val = Uc
    return F


def ilu_nonlinres(row, col, val, F: Factors) -> float:
    """||(A - LU)|_S(A)||_F (control/norms.cpp:375-387)."""
    rid = np.repeat(np.arange(len(row) - 1, dtype=np.int32), np.diff(row))
    return lib().orc_ilu_nonlinres(len(col), rid, _i(col), _d(val), F.L.ptr, F.L.idx,
                                   _d(F.L.val), F.U.ptr, F.U.idx, _d(F.U.val))


def zilures(row, col, val, F: Factors) -> tuple[float, float]:
    """data_zilures (control/norms.cpp:301-405) -> (res, nonlinres)."""
    Ur = F.U_csr()
    r = C.c_double()
    nl = C.c_double()
    lib().orc_zilures(len(row) - 1, _i(row), _i(col), _d(val), F.L.ptr, F.L.idx, _d(F.L.val),
                      Ur.ptr, Ur.idx, _d(Ur.val), C.byref(r), C.byref(nl))
    return r.value, nl.value


def bcsr_expand(row, col, val, bs):
    """LACE's BCSR -> CSR conversion (control/magma_zmconverter.cpp:802-836,
    through mkl_dcsrbsr): every entry of every block, blocks row-major ->
    (ptr, idx, val) scalar CSR, each row in block order."""
    row = np.asarray(row)
    col = np.asarray(col)
    blk = np.asarray(val, dtype=np.float64).reshape(-1, bs, bs)
    nb = len(row) - 1
    ptr = [0]
    idx = []
    out = []
    for I in range(nb):
        for r in range(bs):
            for p in range(row[I], row[I + 1]):
                idx.extend(range(col[p] * bs, col[p] * bs + bs))
                out.extend(blk[p, r, :].tolist())
            ptr.append(len(idx))
    return np.array(ptr, np.int32), np.array(idx, np.int32), np.array(out)


def zilures_bcsr(arow, acol, aval, L, U, bs) -> tuple[float, float]:
    """data_zilures_bcsr (control/norms.cpp:409-468) -> (res, nonlinres).
    A scalar CSR; L and U as (row, col, val) BCSR triples read with the BCSR
    reader (:427-432), every block entry kept; LU = L U with the structural
    pattern of the sparse product (:436); then LACE's two sums (:439-460):
    entries of A the product holds become LU - A, nonlinres over those, res
    over all of LU.  Loops: small cases only."""
    lp, li, lv = bcsr_expand(*L, bs)
    up, ui, uv = bcsr_expand(*U, bs)
    n = len(lp) - 1
    res = 0.0
    nl = 0.0
    for i in range(n):
        lu = {}
        for a in range(lp[i], lp[i + 1]):
            k = li[a]
            for b in range(up[k], up[k + 1]):
                lu[ui[b]] = lu.get(ui[b], 0.0) + lv[a] * uv[b]
        for p in range(arow[i], arow[i + 1]):
            j = int(acol[p])
            if j in lu:
                t = lu[j] - aval[p]
                lu[j] = t
                nl += t * t
        for v in lu.values():
            res += v * v
    return float(np.sqrt(res)), float(np.sqrt(nl))


# ------------------------------------------------------------ kernels

def spmv(row, col, val, x, alpha=1.0, beta=0.0, y=None) -> np.ndarray:
    n = len(row) - 1
    y = np.zeros(n) if y is None else _d(y).copy()
    lib().orc_spmv(n, _i(row), _i(col), _d(val), alpha, _d(x), beta, y)
    return y


def bcsr_spmv(row, col, val, bs, x) -> np.ndarray:
    nb = len(row) - 1
    y = np.zeros(nb * bs)
    lib().orc_bcsr_spmv(nb, bs, _i(row), _i(col), _d(val).reshape(-1), _d(x), y)
    return y


def trsv(ptr, idx, val, b, lower: bool, unit: bool, f32: bool = False) -> np.ndarray:
    n = len(ptr) - 1
    if f32:
        x = np.zeros(n, dtype=np.float32)
        lib().orc_trsv_f32(n, _i(ptr), _i(idx), np.ascontiguousarray(val, dtype=np.float32),
                           int(lower), int(unit), np.ascontiguousarray(b, dtype=np.float32), x)
        return x
    x = np.zeros(n)
    lib().orc_trsv(n, _i(ptr), _i(idx), _d(val), int(lower), int(unit), _d(b), x)
    return x


def levels(ptr, idx, lower: bool) -> tuple[int, np.ndarray]:
    n = len(ptr) - 1
    lev = np.zeros(n, dtype=np.int32)
    nl = lib().orc_levels(n, _i(ptr), _i(idx), int(lower), lev)
    return nl, lev


def parcsrtrsv(uplo: int, ptr, idx, val, rhs, y0=None, tol=1.0):
    n = len(ptr) - 1
    y = np.zeros(n) if y0 is None else _d(y0).copy()
    it = C.c_int()
    lib().orc_parcsrtrsv(uplo, n, _d(val), _i(ptr), _i(idx), _d(rhs), y, tol, C.byref(it))
    return y, it.value


def jacobi_trsv(uplo: int, ptr, idx, val, rhs, tol=0.0, maxiter=100, y0=None):
    n = len(ptr) - 1
    y = np.zeros(n) if y0 is None else _d(y0).copy()
    it = C.c_int()
    lib().orc_jacobi_trsv(uplo, n, _d(val), _i(ptr), _i(idx), _d(rhs), y, tol, maxiter, C.byref(it))
    return y, it.value


def givens(a: float, b: float, tol: float):
    c = C.c_double()
    s = C.c_double()
    lib().orc_givens(a, b, tol, C.byref(c), C.byref(s))
    return c.value, s.value


def orthogonality_error(Q: np.ndarray, search: int) -> float:
    """Q: [ncols, n] (each row one column vector)."""
    ncols, n = Q.shape
    return lib().orc_orthogonality_error(n, n, _d(Q).reshape(-1), search)


def block_inverse(a: np.ndarray) -> np.ndarray:
    bs = a.shape[0]
    out = np.zeros(bs * bs)
    rc = lib().orc_block_inverse(bs, _d(a).reshape(-1), out)
    if rc != 0:
        raise ZeroDivisionError("zero pivot")
    return out.reshape(bs, bs)


# ------------------------------------------------------------- BCSR

@dataclass
class BlockFactors:
    L: Tri          # block CSRL: identity diagonal blocks last; val [nblkL, bs*bs]
    U: Tri          # block CSCU: diagonal block last per block column; blocks untransposed
    bs: int
    steps: list

    def U_rows(self) -> Tri:
        nb = len(self.U.ptr) - 1
        ptr, idx, _, perm = transpose(self.U.ptr, self.U.idx, None, nb)
        return Tri(ptr, idx, self.U.val[perm])

    def dinv(self) -> np.ndarray:
        """inverses of U's diagonal blocks (block row order)."""
        Ur = self.U_rows()
        nb = len(Ur.ptr) - 1
        out = np.zeros((nb, self.bs * self.bs))
        for I in range(nb):
            out[I] = block_inverse(Ur.val[Ur.ptr[I]].reshape(self.bs, self.bs)).ravel()
        return out


def bcsr_parilu(B, sweeps: int, mode: str = "sync", stop_below: float | None = None) -> BlockFactors:
    """Block ParILU(0) from the A-initial guess (BCSRL with identity diagonal
    blocks, BCSCU), src/parilu_v0_3_bcsr.cpp:22-32 and :118-254.  stop_below:
    LACE's BCSR stop (un-normalised step <= reduction, :118)."""
    bs, ld = B.bs, B.bs * B.bs
    rid = B.rowidx()
    A = np.ascontiguousarray(np.asarray(B.val).reshape(B.nblk, ld))
    keepL = B.col <= rid
    Lptr = np.zeros(B.nb + 1, dtype=np.int32)
    np.cumsum(np.bincount(rid[keepL], minlength=B.nb), out=Lptr[1:])
    Lidx = _i(B.col[keepL])
    Lval = A[keepL].copy()
    Lval[B.col[keepL] == rid[keepL]] = np.eye(bs).ravel()
    keepU = B.col >= rid
    Urp = np.zeros(B.nb + 1, dtype=np.int32)
    np.cumsum(np.bincount(rid[keepU], minlength=B.nb), out=Urp[1:])
    up, ui, _, perm = transpose(Urp, _i(B.col[keepU]), None, B.nb)
    Uval = A[keepU][perm].copy()
    F = BlockFactors(Tri(Lptr, Lidx, Lval), Tri(up, ui, Uval), bs, [])
    lb = lib()
    Lc, Uc = Lval.ravel().copy(), Uval.ravel().copy()
    Ln, Un = Lc.copy(), Uc.copy()
    it = 0
    while it < sweeps:
        if mode == "async":
            s = lb.orc_bcsr_parilu_sweep(0, bs, B.nblk, rid, _i(B.col), A.ravel().copy(), Lptr, Lidx, Lc, Lc,
                                         up, ui, Uc, Uc)
        else:
            s = lb.orc_bcsr_parilu_sweep(1, bs, B.nblk, rid, _i(B.col), A.ravel().copy(), Lptr, Lidx, Lc, Ln,
                                         up, ui, Uc, Un)
            Lc, Ln = Ln, Lc
            Uc, Un = Un, Uc
            Ln[:] = Lc
            Un[:] = Uc
        F.steps.append(s)
        it += 1
        if stop_below is not None and not s > stop_below:
            break
    F.L.val = Lc.reshape(-1, ld)
    F.U.val = Uc.reshape(-1, ld)
    return F


def bcsr_precond(F: BlockFactors, f32: bool = False) -> dict:
    Ur = F.U_rows()
    return {"kind": "bcsr_f32" if f32 else "bcsr", "t1": F.L, "t2": Ur, "bdinv": F.dinv()}


# ------------------------------------------------------------ FGMRES

@dataclass
class GmresResult:
    x: np.ndarray
    info: int
    restarts: int
    search_directions: int
    total_iterations: int
    initial_residual: float
    final_residual: float
    converged: bool
    lost_update: bool
    resid_hist: np.ndarray
    orth_hist: np.ndarray | None


PREC = {"trsv": 0, "partrsv": 1, "none": 2, "trsv_f32": 3, "jacobi": 4, "bcsr": 5, "bcsr_f32": 6}


def _gmres_inputs(op: dict, prec: dict, keep: list):
    """The operator and preconditioner structs of the C oracle (arrays kept
    alive in `keep`)."""

    def ptr(a, dt):
        if a is None:
            return None
        a = np.ascontiguousarray(a, dtype=dt)
        keep.append(a)
        return a.ctypes.data

    if op["kind"] == "csr":
        n = len(op["row"]) - 1
        o = OrcOperator(0, n, 1, ptr(op["row"], np.int32), ptr(op["col"], np.int32),
                        ptr(op["val"], np.float64))
    else:
        bs = op["bs"]
        n = (len(op["row"]) - 1) * bs
        o = OrcOperator(1, n, bs, ptr(op["row"], np.int32), ptr(op["col"], np.int32),
                        ptr(np.asarray(op["val"]).reshape(-1), np.float64))
    kind = PREC[prec["kind"]]
    p = OrcPrecond()
    p.kind = kind
    f32 = prec["kind"] in ("trsv_f32", "bcsr_f32")
    for t in ("t1", "t2"):
        tri = prec.get(t)
        if tri is None:
            continue
        setattr(p, t + "_row", ptr(tri.ptr, np.int32))
        setattr(p, t + "_col", ptr(tri.idx, np.int32))
        v = np.asarray(tri.val).reshape(-1)
        if f32:
            setattr(p, t + "_val32", ptr(v, np.float32))
        else:
            setattr(p, t + "_val", ptr(v, np.float64))
        setattr(p, t + "_lower", int(prec.get(t + "_lower", t == "t1")))
        setattr(p, t + "_unit", int(prec.get(t + "_unit", t == "t1")))
    if "bdinv" in prec:
        bd = np.asarray(prec["bdinv"]).reshape(-1)
        if f32:
            p.bdinv32 = ptr(bd, np.float32)
        else:
            p.bdinv = ptr(bd, np.float64)
    p.tol = float(prec.get("tol", 1.0))
    p.max_sweeps = int(prec.get("max_sweeps", 100))
    return o, p, n


def _gmres_result(x, info, log, rh, oh) -> GmresResult:
    t = log.total_iterations
    return GmresResult(x, info, log.restarts, log.search_directions, t, log.initial_residual,
                       log.final_residual, bool(log.converged), bool(log.lost_update), rh[:t].copy(),
                       oh[:t].copy() if oh is not None else None)


def fgmres(op: dict, prec: dict, b, x0=None, search_max=30, restart_max=20, rtol=1e-10,
           tol_type=1, monitor_orthog=False) -> GmresResult:
    """FGMRES-Householder mirror (src/fgmres_householder_restart.cpp:63-788).

    op: {'kind': 'csr', 'row','col','val'} or {'kind': 'bcsr', 'bs', 'row','col','val'}.
    prec: {'kind': one of PREC, 't1': Tri, 't1_lower', 't1_unit', 't2': Tri, ...,
           'bdinv': array, 'tol', 'max_sweeps'}."""
    keep = []
    o, p, n = _gmres_inputs(op, prec, keep)
    par = OrcGmresPar(search_max, restart_max, tol_type, rtol, int(monitor_orthog), 0)
    log = OrcGmresLog()
    x = np.zeros(n) if x0 is None else _d(x0).copy()
    rh = np.zeros(search_max * restart_max)
    oh = np.zeros(search_max * restart_max) if monitor_orthog else None
    info = lib().orc_fgmres_householder(C.byref(o), C.byref(p), _d(b), x, C.byref(par), C.byref(log),
                                         rh.ctypes.data, oh.ctypes.data if oh is not None else None)
    return _gmres_result(x, info, log, rh, oh)


def fgmres_mgs(op: dict, prec: dict, b, x0=None, search_max=30, restart_max=20, rtol=1e-10,
               tol_type=1, monitor_orthog=False, reorth=0, restarted=True) -> GmresResult:
    """FGMRES with modified Gram-Schmidt Arnoldi: src/fgmres_restart.cpp:63-532
    (restarted) or src/fgmres.cpp:64-517 (one cycle).  Arguments as fgmres();
    reorth: 0 Brown/Hindmarsh test, 1 never, 2 always (sparse_types.h:164-166)."""
    keep = []
    o, p, n = _gmres_inputs(op, prec, keep)
    par = OrcGmresPar(search_max, restart_max if restarted else 1, tol_type, rtol, int(monitor_orthog),
                      int(reorth))
    log = OrcGmresLog()
    x = np.zeros(n) if x0 is None else _d(x0).copy()
    nc = restart_max if restarted else 1
    rh = np.zeros(search_max * nc)
    oh = np.zeros(search_max * nc) if monitor_orthog else None
    info = lib().orc_fgmres_mgs(C.byref(o), C.byref(p), _d(b), x, C.byref(par), int(bool(restarted)),
                                C.byref(log), rh.ctypes.data, oh.ctypes.data if oh is not None else None)
    return _gmres_result(x, info, log, rh, oh)


def ilu_precond(F: Factors, kind: str = "trsv", **kw) -> dict:
    """Forward preconditioner M = LU: t1 = L (lower, unit), t2 = U (CSR)."""
    Ur = F.U_csr()
    d = {"kind": kind, "t1": F.L, "t1_lower": True, "t1_unit": True,
         "t2": Ur, "t2_lower": False, "t2_unit": False}
    d.update(kw)
    return d


def ilu_precond_adjoint(F: Factors, kind: str = "trsv") -> dict:
    """Transposed preconditioner (LU)^T = U^T L^T: t1 = U^T (U's CSC image read
    as CSR: lower, non-unit, diagonal last), t2 = L^T (L's CSC image: upper,
    unit, diagonal first)."""
    n = len(F.L.ptr) - 1
    lp, li, lv, _ = transpose(F.L.ptr, F.L.idx, F.L.val, n)
    return {"kind": kind, "t1": F.U, "t1_lower": True, "t1_unit": False,
            "t2": Tri(lp, li, lv), "t2_lower": False, "t2_unit": True}


# ------------------------------------------------------------ orderings

def cuthill_mckee(n: int, row, col, reverse: bool = False) -> np.ndarray:
    """nn_map[old] = new, the Cuthill-McKee numbering of A's row graph as
    src/cuthill_mckee.cpp states it: degree = off-diagonal entries of a row
    (:98-113), the seed a node of maximum degree (:128-139), breadth first,
    each node's unnumbered neighbours in order of decreasing degree
    (compare_degree, :31-41, popped in that order :192-207), nn_map[old] = new
    (:224-225).  The cases LACE's routine leaves undefined are fixed as the
    library fixes them: ties to the lower index, a new component from the
    next node of maximum degree, new' = n - 1 - new when reversed."""
    row = np.asarray(row, dtype=np.int64)
    col = np.asarray(col, dtype=np.int64)
    deg = [int(np.count_nonzero(col[row[i]:row[i + 1]] != i)) for i in range(n)]
    key = lambda v: (-deg[v], v)  # noqa: E731
    seeds = sorted(range(n), key=key)
    seen = [False] * n
    order: list[int] = []
    head = nxt = 0
    while len(order) < n:
        if head == len(order):
            while seen[seeds[nxt]]:
                nxt += 1
            seen[seeds[nxt]] = True
            order.append(seeds[nxt])
        v = order[head]
        head += 1
        nb = []
        for u in col[row[v]:row[v + 1]]:
            u = int(u)
            if u != v and not seen[u]:
                seen[u] = True
                nb.append(u)
        order.extend(sorted(nb, key=key))
    nn_map = np.empty(n, dtype=np.int64)
    for k, v in enumerate(order):
        nn_map[v] = n - 1 - k if reverse else k
    return nn_map


def permute_csr(row, col, val, P, Pinv, ld: int = 1):
    """src/reorder.cpp:86-122 then :127-165: row i of the result is row P[i]
    of A with columns c -> Pinv[c], each row sorted by column (ld values per
    entry)."""
    row = np.asarray(row)
    n = len(row) - 1
    val = np.asarray(val).reshape(-1, ld)
    r2, c2, v2 = [0], [], []
    for i in range(n):
        o = P[i]
        cols = np.asarray(Pinv)[np.asarray(col[row[o]:row[o + 1]], dtype=np.int64)]
        order = np.argsort(cols, kind="stable")
        c2.extend(cols[order].tolist())
        v2.append(val[row[o]:row[o + 1]][order])
        r2.append(r2[-1] + len(cols))
    vals = np.concatenate(v2).reshape(-1) if v2 else np.zeros(0)
    return np.array(r2, dtype=np.int32), np.array(c2, dtype=np.int32), vals
