"""LACE-named entry points called through LACE's data_d_matrix container.

These mirror how LACE's own tests drive the path (testing/test_iLU.cpp,
testing/test_linearSolver.cpp): build host containers, call
data_PariLU_v0_3*, convert, call data_fgmres_householder_restart, check the
residual.  The library allocates the output factor arrays with
posix_memalign (as LACE_CALLOC does); `free_matrix` releases them with free().
"""
from __future__ import annotations

import ctypes as C
import weakref

import numpy as np

from . import DataMatrix, GmresLog, GmresParam, PrecondLog, lib

# data_storage_t / data_diagorder_t / data_uplo_t (include/dense_types.h)
Magma_CSR, Magma_DENSE, Magma_BCSR, Magma_CSC = 611, 614, 615, 616
Magma_CSRL, Magma_CSRU, Magma_CSCU, Magma_BCSCU = 627, 628, 635, 646
Magma_UNITY, Magma_VALUE = 593, 594
MagmaUpper, MagmaLower, MagmaFull = 121, 122, 123
MagmaRowMajor, MagmaColMajor = 101, 102

_libc = C.CDLL(None)
_libc.free.argtypes = [C.c_void_p]
_libc.malloc.restype = C.c_void_p
_libc.malloc.argtypes = [C.c_size_t]


def set_options(precision: str = "fp64", trsv: str = "syncfree", jacobi_sweeps: int = 8,
                use_graph: bool = True) -> None:
    """lace_gpu_dropin_set_options: how the LACE-named calls run."""
    from . import PREC, TRSV, GpuOptions
    o = GpuOptions()
    f = lib()
    f.lace_gpu_default_options(C.byref(o))
    o.precision = PREC[precision]
    o.trsv_mode = TRSV[trsv]
    o.jacobi_sweeps = jacobi_sweeps
    o.use_graph = int(use_graph)
    rc = f.lace_gpu_dropin_set_options(C.byref(o))
    if rc:
        from . import LaceError
        raise LaceError(rc, "lace_gpu_dropin_set_options")


class Mat:
    """A DataMatrix plus the numpy arrays it points into."""

    def __init__(self):
        self.m = DataMatrix()
        self.keep = []

    @property
    def ref(self):
        return C.byref(self.m)

    def _own(self, a, dt):
        a = np.ascontiguousarray(a, dtype=dt)
        self.keep.append(a)
        return a.ctypes.data


def csr(row, col, val, n, storage=Magma_CSR) -> Mat:
    M = Mat()
    M.m.storage_type = storage
    M.m.num_rows = n
    M.m.num_cols = n
    M.m.nnz = len(col)
    M.m.true_nnz = len(col)
    M.m.major = MagmaRowMajor
    M.m.fill_mode = MagmaFull
    M.m.row = M._own(row, np.int32)
    M.m.col = M._own(col, np.int32)
    M.m.val = M._own(val, np.float64)
    return M


def bcsr(A) -> Mat:
    """problems.BCSR -> Magma_BCSR container (row-major blocks)."""
    M = Mat()
    M.m.storage_type = Magma_BCSR
    M.m.num_rows = A.nb
    M.m.num_cols = A.nb
    M.m.blocksize = A.bs
    M.m.ldblock = A.bs * A.bs
    M.m.numblocks = A.nblk
    M.m.nnz = A.nblk * A.bs * A.bs
    M.m.row = M._own(A.row, np.int32)
    M.m.col = M._own(A.col, np.int32)
    M.m.val = M._own(np.asarray(A.val).reshape(-1), np.float64)
    return M


def dense(v, copy: bool = True) -> Mat:
    """A Magma_DENSE column; copy=False wraps a float64 array the call only
    reads (no copy when it is already contiguous)."""
    v = np.asarray(v, dtype=np.float64)
    M = Mat()
    M.m.storage_type = Magma_DENSE
    M.m.num_rows = len(v)
    M.m.num_cols = 1
    M.m.nnz = len(v)
    M.m.ld = len(v)
    M.m.major = MagmaColMajor
    M.m.val = M._own(v.copy() if copy else v, np.float64)
    return M


def vector_values(M: Mat) -> np.ndarray:
    return np.ctypeslib.as_array(C.cast(M.m.val, C.POINTER(C.c_double)), shape=(M.m.num_rows,)).copy()


def matrix_arrays(m: DataMatrix):
    """(ptr, idx, val) copies of a library-filled container."""
    n = m.num_rows
    nidx = m.numblocks if m.blocksize > 0 and m.numblocks > 0 else m.nnz
    nval = m.nnz
    ptr = np.ctypeslib.as_array(C.cast(m.row, C.POINTER(C.c_int)), shape=(n + 1,)).copy()
    idx = np.ctypeslib.as_array(C.cast(m.col, C.POINTER(C.c_int)), shape=(nidx,)).copy()
    val = np.ctypeslib.as_array(C.cast(m.val, C.POINTER(C.c_double)), shape=(nval,)).copy()
    return ptr, idx, val


def free_matrix(m: DataMatrix) -> None:
    """data_zmfree for library-allocated members."""
    for name in ("val", "col", "row", "rowidx", "diag", "list", "blockinfo"):
        p = getattr(m, name)
        if p:
            _libc.free(p)
            setattr(m, name, None)


def parilu(A: Mat, reduction: float = 1e-15, max_sweeps: int | None = None, gpu_name: bool = False):
    """data_PariLU_v0_3[_gpu] (max_sweeps None) or the prescribed-sweeps
    variants.  Returns (L arrays, U arrays (CSC), log dict)."""
    L = DataMatrix()
    U = DataMatrix()
    L.storage_type = Magma_CSRL
    U.storage_type = Magma_CSCU
    log = PrecondLog()
    f = lib()
    if max_sweeps is None:
        if gpu_name:
            f.data_PariLU_v0_3_gpu(A.ref, C.byref(L), C.byref(U), reduction, C.byref(log), 0)
        else:
            f.data_PariLU_v0_3(A.ref, C.byref(L), C.byref(U), reduction, C.byref(log))
    else:
        log.maxSweeps = max_sweeps
        if gpu_name:
            f.data_PariLU_v0_3_gpu_prescribedSweeps(A.ref, C.byref(L), C.byref(U), reduction, C.byref(log))
        else:
            f.data_PariLU_v0_3_prescribedSweeps(A.ref, C.byref(L), C.byref(U), reduction, C.byref(log))
    if log.sweeps < 0:
        from . import LaceError
        raise LaceError(f.lace_gpu_last_error(), "data_PariLU_v0_3")
    la = matrix_arrays(L)
    ua = matrix_arrays(U)
    info = {k: getattr(log, k) for k in ("sweeps", "tol", "finalStep", "A_Frobenius", "precond_generation_time",
                                         "initial_residual", "initial_nonlinear_residual",
                                         "nonlinear_residual", "omp_num_threads")}
    info["L_storage"] = L.storage_type
    info["U_storage"] = U.storage_type
    free_matrix(L)
    free_matrix(U)
    return la, ua, info


class LibMat(Mat):
    """A container the library filled (ParILU's L or U); its arrays are
    released with free(), as data_zmfree does, when the object goes away."""

    def __init__(self, m: DataMatrix):
        super().__init__()
        self.m = m
        weakref.finalize(self, free_matrix, m)

    def arrays(self):
        return matrix_arrays(self.m)


def parilu_mats(A: Mat, reduction: float = 1e-15, max_sweeps: int | None = None):
    """data_PariLU_v0_3 (max_sweeps None) or data_PariLU_v0_3_prescribedSweeps,
    returning the filled containers themselves (L in CSRL, U in CSCU) to pass
    on to fgmres_householder_restart as a C caller would, without copies."""
    L = DataMatrix()
    U = DataMatrix()
    L.storage_type = Magma_CSRL
    U.storage_type = Magma_CSCU
    log = PrecondLog()
    f = lib()
    if max_sweeps is None:
        f.data_PariLU_v0_3(A.ref, C.byref(L), C.byref(U), reduction, C.byref(log))
    else:
        log.maxSweeps = max_sweeps
        f.data_PariLU_v0_3_prescribedSweeps(A.ref, C.byref(L), C.byref(U), reduction, C.byref(log))
    if log.sweeps < 0:
        from . import LaceError
        raise LaceError(f.lace_gpu_last_error(), "data_PariLU_v0_3")
    info = {k: getattr(log, k) for k in ("sweeps", "tol", "finalStep", "A_Frobenius", "precond_generation_time",
                                         "initial_residual", "initial_nonlinear_residual",
                                         "nonlinear_residual", "omp_num_threads")}
    return LibMat(L), LibMat(U), info


def fgmres_householder_restart(A: Mat, b, x0, L: Mat | None, U: Mat | None, search_max=20, restart_max=20,
                               rtol=1e-3, tol_type=0, choice=0, monitor_orthog=0, single_cycle=False,
                               x0_inplace=False):
    """data_fgmres_householder_restart (or data_fgmres_householder).
    x0_inplace: the solution overwrites x0 (a contiguous float64 array), as
    LACE overwrites its caller's x0 container; otherwise x0 is copied first."""
    f = lib()
    fn = f.data_fgmres_householder if single_cycle else f.data_fgmres_householder_restart
    return _fgmres_call(fn, A, b, x0, L, U, search_max, restart_max, rtol, tol_type, choice, monitor_orthog, 0,
                        x0_inplace)


def fgmres_restart(A: Mat, b, x0, L: Mat | None, U: Mat | None, search_max=20, restart_max=20,
                   rtol=1e-3, tol_type=0, choice=0, monitor_orthog=0, reorth=0, single_cycle=False):
    """data_fgmres_restart, FGMRES with modified Gram-Schmidt (or data_fgmres:
    one cycle)."""
    f = lib()
    fn = f.data_fgmres if single_cycle else f.data_fgmres_restart
    return _fgmres_call(fn, A, b, x0, L, U, search_max, restart_max, rtol, tol_type, choice, monitor_orthog,
                        reorth)


def _fgmres_call(fn, A: Mat, b, x0, L, U, search_max, restart_max, rtol, tol_type, choice, monitor_orthog,
                 reorth, x0_inplace=False):
    bv = dense(b, copy=False)
    if x0_inplace and not (isinstance(x0, np.ndarray) and x0.dtype == np.float64 and x0.flags.c_contiguous):
        raise ValueError("x0_inplace needs a contiguous float64 array")
    xv = dense(x0, copy=not x0_inplace)
    par = GmresParam()
    par.search_max = search_max
    par.restart_max = restart_max
    par.rtol = rtol
    par.tol_type = tol_type
    par.user_csrtrsv_choice = choice
    par.monitorOrthog = monitor_orthog
    par.precondition = 1
    par.reorth = reorth
    log = GmresLog()
    Lr = L.ref if L is not None else None
    Ur = U.ref if U is not None else None
    rc = fn(A.ref, bv.ref, xv.ref, Lr, Ur, C.byref(par), C.byref(log))
    # the solution is written into x0's array in place: hand that array back
    own = xv.keep[-1]
    x = own if xv.m.val == own.ctypes.data else vector_values(xv)
    return x, rc, {k: getattr(log, k) for k in ("restarts", "search_directions", "solve_time",
                                                 "initial_residual", "final_residual")}


def read_mtx(path: str, coo: bool = False):
    """read_z_csr_from_mtx (or read_z_coo_from_mtx): (rc, n_rows, n_cols,
    row (pointers, or indices), col, val) as numpy arrays (copies; the
    library's arrays are released)."""
    st, nr, nc, nz = C.c_int(), C.c_int(), C.c_int(), C.c_int()
    val, row, col = C.c_void_p(), C.c_void_p(), C.c_void_p()
    fn = lib().read_z_coo_from_mtx if coo else lib().read_z_csr_from_mtx
    rc = fn(C.byref(st), C.byref(nr), C.byref(nc), C.byref(nz), C.byref(val), C.byref(row), C.byref(col),
            path.encode())
    if rc != 0:
        return rc, 0, 0, None, None, None
    n, z = nr.value, nz.value
    nrow = max(z, 1) if coo else n + 1
    r = np.ctypeslib.as_array(C.cast(row, C.POINTER(C.c_int)), shape=(nrow,))[:(z if coo else n + 1)].copy()
    c = np.ctypeslib.as_array(C.cast(col, C.POINTER(C.c_int)), shape=(max(z, 1),))[:z].copy()
    v = np.ctypeslib.as_array(C.cast(val, C.POINTER(C.c_double)), shape=(max(z, 1),))[:z].copy()
    libc = C.CDLL(None)
    for p in (val, row, col):
        libc.free(p)
    return rc, n, nc.value, r, c, v


def write_mtx(A: "Mat", path: str, major: int = 101) -> int:
    """data_zwrite_csr_mtx (major 101 row-major, 102 column-major)."""
    return lib().data_zwrite_csr_mtx(A.m, int(major), path.encode())


def spmv(alpha: float, A: Mat, x, beta: float = 0.0, y=None):
    nout = A.m.num_rows * (A.m.blocksize if A.m.storage_type == Magma_BCSR else 1)
    xv = dense(x)
    yv = dense(np.zeros(nout) if y is None else y)
    rc = lib().data_z_spmv(alpha, A.ref, xv.ref, beta, yv.ref)
    return vector_values(yv), rc


def parcsrtrsv(uplo, storage, diag, ptr, idx, val, rhs, y0=None, tol=1.0):
    n = len(ptr) - 1
    ptr = np.ascontiguousarray(ptr, dtype=np.int32)
    idx = np.ascontiguousarray(idx, dtype=np.int32)
    val = np.ascontiguousarray(val, dtype=np.float64)
    rhs = np.ascontiguousarray(rhs, dtype=np.float64)
    y = np.zeros(n) if y0 is None else np.ascontiguousarray(y0, dtype=np.float64).copy()
    it = C.c_int()
    rc = lib().data_parcsrtrsv(uplo, storage, diag, n, val.ctypes.data, ptr.ctypes.data, idx.ctypes.data,
                               rhs.ctypes.data, y.ctypes.data, tol, C.byref(it))
    return y, it.value, rc


def zilures(A: Mat, L: Mat, U: Mat):
    res = C.c_double()
    nl = C.c_double()
    LU = DataMatrix()
    rc = lib().data_zilures(A.m, L.m, U.m, C.byref(LU), C.byref(res), C.byref(nl))
    return res.value, nl.value, rc


def zilures_bcsr(A: Mat, L: Mat, U: Mat):
    """data_zilures_bcsr: A a scalar CSR container, L and U BCSR containers."""
    res = C.c_double()
    nl = C.c_double()
    LU = DataMatrix()
    rc = lib().data_zilures_bcsr(A.m, L.m, U.m, C.byref(LU), C.byref(res), C.byref(nl))
    return res.value, nl.value, rc


def cuthill_mckee(n: int, row, col, reverse: bool = False) -> np.ndarray:
    """data_reorder_cuthill_mckee on a CSR pattern: nn_map[old] = new."""
    A = csr(row, col, np.zeros(len(col)), n)
    nn_map = np.empty(n, dtype=np.int32)
    f = lib()
    f.data_reorder_cuthill_mckee(A.ref, nn_map.ctypes.data_as(C.POINTER(C.c_int)), bool(reverse))
    rc = f.lace_gpu_last_error()
    if rc:
        from . import LaceError
        raise LaceError(rc, "data_reorder_cuthill_mckee")
    return nn_map


def sparse_reorder(n: int, row, col, val, reorder: int, blocksize: int = 0):
    """data_sparse_reorder on a copy of A (CSR, or BCSR of n block rows when
    blocksize > 0): (row, col, val) of A in the new numbering, P (new ->
    old) and Pinv (old -> new).  The call replaces the container's arrays,
    so they are handed over in memory of the C allocator."""
    ld = blocksize * blocksize if blocksize else 1
    M = DataMatrix()
    M.storage_type = Magma_BCSR if blocksize else Magma_CSR
    M.num_rows = M.num_cols = n
    arrs = (np.ascontiguousarray(row, dtype=np.int32), np.ascontiguousarray(col, dtype=np.int32),
            np.ascontiguousarray(val, dtype=np.float64).reshape(-1))
    for name, a in zip(("row", "col", "val"), arrs):
        p = _libc.malloc(max(a.nbytes, 8))
        if not p:
            raise MemoryError("malloc")
        C.memmove(p, a.ctypes.data, a.nbytes)
        setattr(M, name, p)
    if blocksize:
        M.blocksize, M.ldblock, M.numblocks = blocksize, ld, len(arrs[1])
    M.nnz = len(arrs[1]) * ld
    P = np.empty(max(n, 1), dtype=np.int32)
    Pinv = np.empty(max(n, 1), dtype=np.int32)
    ip = C.POINTER(C.c_int)
    try:
        rc = lib().data_sparse_reorder(C.byref(M), P.ctypes.data_as(ip), Pinv.ctypes.data_as(ip), int(reorder))
        if rc:
            from . import LaceError
            raise LaceError(rc, "data_sparse_reorder")
        nz = int(np.ctypeslib.as_array(C.cast(M.row, C.POINTER(C.c_int)), shape=(n + 1,))[n])
        out = (np.ctypeslib.as_array(C.cast(M.row, C.POINTER(C.c_int)), shape=(n + 1,)).copy(),
               np.ctypeslib.as_array(C.cast(M.col, C.POINTER(C.c_int)), shape=(max(nz, 1),)).copy()[:nz],
               np.ctypeslib.as_array(C.cast(M.val, C.POINTER(C.c_double)), shape=(max(nz * ld, 1),)).copy()[:nz * ld])
    finally:
        for name in ("row", "col", "val"):
            _libc.free(getattr(M, name))
    return out + (P[:n], Pinv[:n])
