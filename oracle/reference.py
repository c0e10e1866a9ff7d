"""ctypes access to LACE's own implementation, compiled unmodified from the
LACE sources by `make -C oracle ref` into oracle/_ref/ (TEST INFRASTRUCTURE).

Only available where the LACE source tree is present (oracle/Makefile names
where it reads it; LACE_REF_SRC overrides); callers must skip when
`available()` is False.
Used to pin the C restatement and to generate the golden fixtures in
tests/golden/.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))


def _ref_src() -> str:
    """The LACE source tree the oracle's Makefile reads (LACE_REF_SRC, else the
    recipe's default)."""
    env = os.environ.get("LACE_REF_SRC")
    if env:
        return env
    try:
        r = subprocess.run(["make", "-s", "-C", HERE, "print-ref"], capture_output=True, text=True, check=True)
        return r.stdout.strip()
    except (subprocess.CalledProcessError, OSError):
        return ""


REF_SRC = _ref_src()
LIB = os.path.join(HERE, "_ref", "liblace_ref.so")
LIB_BCSR = os.path.join(HERE, "_ref", "liblace_ref_bcsr.so")

# data_storage_t / data_diagorder_t values (include/dense_types.h:308-383)
Magma_CSR, Magma_DENSE, Magma_BCSR, Magma_CSC = 611, 614, 615, 616
Magma_CSRL, Magma_CSRU, Magma_CSCU = 627, 628, 635
Magma_BCSRL, Magma_BCSCU = 641, 646
Magma_UNITY, Magma_VALUE = 593, 594
MagmaUpper, MagmaLower = 121, 122

_libs: dict = {}


def available() -> bool:
    if os.path.exists(LIB) and os.path.exists(LIB_BCSR):
        return True
    if not os.path.isdir(os.path.join(REF_SRC, "src")):
        return False
    try:
        subprocess.run(["make", "-s", "-C", HERE, "ref", f"REF={REF_SRC}", "-j8"], check=True,
                       stdout=subprocess.DEVNULL)
    except (subprocess.CalledProcessError, OSError):
        return False
    return os.path.exists(LIB) and os.path.exists(LIB_BCSR)


def _load(path: str) -> C.CDLL:
    if path not in _libs:
        L = C.CDLL(path)
        vp = C.c_void_p
        L.ref_mat_new.restype = vp
        L.ref_mat_new.argtypes = [C.c_int, C.c_int, C.c_int, C.c_int, vp, vp, vp, C.c_int]
        L.ref_mat_info.argtypes = [vp, vp]
        L.ref_mat_copy.argtypes = [vp, C.c_int, C.c_int, C.c_int, vp, vp, vp]
        L.ref_mat_free.argtypes = [vp]
        L.ref_convert.restype = vp
        L.ref_convert.argtypes = [vp, C.c_int, C.c_int, C.c_int]
        L.ref_convert_bs.restype = vp
        L.ref_convert_bs.argtypes = [vp, C.c_int, C.c_int, C.c_int, C.c_int]
        L.ref_coo_new.restype = vp
        L.ref_coo_new.argtypes = [C.c_int, C.c_int, C.c_int, vp, vp, vp]
        L.ref_transpose.restype = vp
        L.ref_transpose.argtypes = [vp]
        if path == LIB:
            L.ref_parilu.argtypes = [vp, C.c_double, C.c_int, C.POINTER(vp), C.POINTER(vp), vp]
            L.ref_zilures.argtypes = [vp, vp, vp, C.POINTER(C.c_double), C.POINTER(C.c_double)]
            L.ref_zilures_bcsr.argtypes = [vp, vp, vp, C.POINTER(C.c_double), C.POINTER(C.c_double)]
            L.ref_spmv.argtypes = [C.c_double, vp, vp, C.c_double, vp]
            L.ref_parcsrtrsv.argtypes = [C.c_int, C.c_int, C.c_int, C.c_int, vp, vp, vp, vp, vp,
                                         C.c_double, C.POINTER(C.c_int)]
            L.ref_fgmres_householder_restart.argtypes = [vp, vp, vp, vp, vp, vp, vp]
            L.ref_fgmres_mgs.argtypes = [vp, vp, vp, vp, vp, vp, vp, C.c_int]
            L.ref_givens.argtypes = [C.c_double, C.c_double, C.c_double, C.POINTER(C.c_double),
                                     C.POINTER(C.c_double)]
            L.ref_orthogonality_error.restype = C.c_double
            L.ref_orthogonality_error.argtypes = [C.c_int, C.c_int, vp, C.c_int]
            L.ref_csrilu0.argtypes = [vp]
            L.ref_read_csr_mtx.restype = vp
            L.ref_read_csr_mtx.argtypes = [C.c_char_p, C.POINTER(C.c_int)]
            L.ref_write_csr_mtx.argtypes = [vp, C.c_int, C.c_char_p]
            L.ref_read_coo_mtx.argtypes = [C.c_char_p, vp, C.c_int, vp, vp, vp]
        else:
            L.ref_bcsr_parilu.argtypes = [vp, C.c_double, C.POINTER(vp), C.POINTER(vp), vp]
            L.ref_dense_inverse.argtypes = [C.c_int, vp, vp]
        _libs[path] = L
    return _libs[path]


def lib() -> C.CDLL:
    return _load(LIB)


def lib_bcsr() -> C.CDLL:
    return _load(LIB_BCSR)


def _p(a):
    return a.ctypes.data


class Mat:
    """Owning wrapper of a LACE data_d_matrix handle."""

    def __init__(self, handle, L):
        self.h = C.c_void_p(handle)
        self.L = L

    @classmethod
    def from_arrays(cls, storage, nrows, ncols, row, col, val, blocksize=0, L=None):
        L = L or lib()
        row = np.ascontiguousarray(row, dtype=np.int32)
        col = np.ascontiguousarray(col, dtype=np.int32)
        val = np.ascontiguousarray(val, dtype=np.float64).reshape(-1)
        h = L.ref_mat_new(storage, nrows, ncols, len(col), _p(row), _p(col), _p(val), blocksize)
        return cls(h, L)

    def info(self):
        out = np.zeros(6, dtype=np.int32)
        self.L.ref_mat_info(self.h, _p(out))
        return dict(storage=int(out[0]), nrows=int(out[1]), ncols=int(out[2]), nnz=int(out[3]),
                    numblocks=int(out[4]), blocksize=int(out[5]))

    def arrays(self, nptr=None):
        """(ptr, idx, val).  ptr has num_rows+1 entries (for a CSC/BCSC
        matrix num_rows is the number of columns of the original)."""
        inf = self.info()
        nptr = inf["nrows"] + 1 if nptr is None else nptr
        if inf["blocksize"] > 0 and inf["numblocks"] > 0:
            nidx = inf["numblocks"]
            nval = inf["numblocks"] * inf["blocksize"] ** 2
        else:
            nidx = inf["nnz"]
            nval = inf["nnz"]
        row = np.zeros(nptr, dtype=np.int32)
        col = np.zeros(nidx, dtype=np.int32)
        val = np.zeros(nval)
        self.L.ref_mat_copy(self.h, nptr, nidx, nval, _p(row), _p(col), _p(val))
        return row, col, val

    def free(self):
        if self.h:
            self.L.ref_mat_free(self.h)
            self.h = C.c_void_p(None)

    def __del__(self):
        try:
            self.free()
        except Exception:
            pass


def set_storage(A: Mat, storage: int) -> None:
    """A->storage_type = storage (the first member of data_d_matrix)."""
    C.cast(A.h, C.POINTER(C.c_int))[0] = storage


def convert(A: Mat, old, new, diagorder=0) -> Mat:
    return Mat(A.L.ref_convert(A.h, old, new, diagorder), A.L)


def transpose(A: Mat) -> Mat:
    """LACE's data_zmtranspose into a fresh matrix."""
    return Mat(A.L.ref_transpose(A.h), A.L)


def parilu(A: Mat, reduction: float, max_sweeps: int = -1):
    """data_PariLU_v0_3 (max_sweeps < 0) or data_PariLU_v0_3_prescribedSweeps.
    Returns (L CSRL Mat, U CSCU Mat, log dict)."""
    L = lib()
    hl = C.c_void_p()
    hu = C.c_void_p()
    log = np.zeros(8)
    L.ref_parilu(A.h, reduction, max_sweeps, C.byref(hl), C.byref(hu), _p(log))
    keys = ["sweeps", "tol", "finalStep", "A_Frobenius", "generation_time", "initial_residual",
            "initial_nonlinear_residual", "omp_threads"]
    return Mat(hl.value, L), Mat(hu.value, L), dict(zip(keys, log.tolist()))


def zilures(A: Mat, Lm: Mat, Um: Mat):
    r = C.c_double()
    nl = C.c_double()
    lib().ref_zilures(A.h, Lm.h, Um.h, C.byref(r), C.byref(nl))
    return r.value, nl.value


def zilures_bcsr(A: Mat, Lm: Mat, Um: Mat):
    """LACE's data_zilures_bcsr (control/norms.cpp:409-468): A scalar CSR,
    L and U BCSR handles."""
    r = C.c_double()
    nl = C.c_double()
    lib().ref_zilures_bcsr(A.h, Lm.h, Um.h, C.byref(r), C.byref(nl))
    return r.value, nl.value


def spmv(A: Mat, x, alpha=1.0, beta=0.0, y=None):
    n = A.info()["nrows"]
    x = np.ascontiguousarray(x, dtype=np.float64)
    y = np.zeros(n) if y is None else np.ascontiguousarray(y, dtype=np.float64).copy()
    info = lib().ref_spmv(alpha, A.h, _p(x), beta, _p(y))
    return y, info


def parcsrtrsv(uplo, storage, diag, ptr, idx, val, rhs, y0=None, tol=1.0):
    n = len(ptr) - 1
    ptr = np.ascontiguousarray(ptr, dtype=np.int32)
    idx = np.ascontiguousarray(idx, dtype=np.int32)
    val = np.ascontiguousarray(val, dtype=np.float64)
    rhs = np.ascontiguousarray(rhs, dtype=np.float64)
    y = np.zeros(n) if y0 is None else np.ascontiguousarray(y0, dtype=np.float64).copy()
    it = C.c_int()
    info = lib().ref_parcsrtrsv(uplo, storage, diag, n, _p(val), _p(ptr), _p(idx), _p(rhs), _p(y),
                                tol, C.byref(it))
    return y, it.value, info


def fgmres_householder_restart(A: Mat, b, x0, Lm: Mat, Um: Mat, search_max=20, restart_max=20,
                               rtol=1e-3, tol_type=0, choice=0, monitor_orthog=0):
    b = np.ascontiguousarray(b, dtype=np.float64)
    x = np.ascontiguousarray(x0, dtype=np.float64).copy()
    par = np.array([search_max, tol_type, rtol, choice, monitor_orthog, restart_max, 1, 0],
                   dtype=np.float64)
    log = np.zeros(7)
    info = lib().ref_fgmres_householder_restart(A.h, _p(b), _p(x), Lm.h, Um.h, _p(par), _p(log))
    keys = ["restarts", "search_directions", "solve_time", "initial_residual", "final_residual",
            "scaled_residual", "original_residual"]
    return x, info, dict(zip(keys, log.tolist()))


def fgmres_mgs(A: Mat, b, x0, Lm: Mat, Um: Mat, search_max=20, restart_max=20, rtol=1e-3,
               tol_type=0, choice=0, monitor_orthog=0, reorth=0, restarted=True):
    """data_fgmres_restart (restarted) or data_fgmres, LACE's own code."""
    b = np.ascontiguousarray(b, dtype=np.float64)
    x = np.ascontiguousarray(x0, dtype=np.float64).copy()
    par = np.array([search_max, tol_type, rtol, choice, monitor_orthog, restart_max, 1, reorth],
                   dtype=np.float64)
    log = np.zeros(7)
    info = lib().ref_fgmres_mgs(A.h, _p(b), _p(x), Lm.h, Um.h, _p(par), _p(log), int(bool(restarted)))
    keys = ["restarts", "search_directions", "solve_time", "initial_residual", "final_residual",
            "scaled_residual", "original_residual"]
    return x, info, dict(zip(keys, log.tolist()))


def givens(a, b, tol):
    c = C.c_double()
    s = C.c_double()
    lib().ref_givens(a, b, tol, C.byref(c), C.byref(s))
    return c.value, s.value


def orthogonality_error(Q: np.ndarray, search: int) -> float:
    ncols, n = Q.shape
    Q = np.ascontiguousarray(Q, dtype=np.float64)
    return lib().ref_orthogonality_error(n, ncols, _p(Q), search)


def csrilu0(A: Mat) -> None:
    lib().ref_csrilu0(A.h)


def bcsr_parilu(A: Mat, reduction: float):
    L = lib_bcsr()
    hl = C.c_void_p()
    hu = C.c_void_p()
    log = np.zeros(2)
    L.ref_bcsr_parilu(A.h, reduction, C.byref(hl), C.byref(hu), _p(log))
    return Mat(hl.value, L), Mat(hu.value, L), {"sweeps": log[0], "generation_time": log[1]}


def dense_inverse(a: np.ndarray) -> np.ndarray:
    bs = a.shape[0]
    a = np.ascontiguousarray(a, dtype=np.float64)
    out = np.zeros((bs, bs))
    lib_bcsr().ref_dense_inverse(bs, _p(a), _p(out))
    return out


def read_csr_mtx(path: str):
    """LACE's own read_z_csr_from_mtx: (info, n_rows, n_cols, row, col, val)."""
    info = C.c_int()
    h = lib().ref_read_csr_mtx(path.encode(), C.byref(info))
    M = Mat(h, lib())
    if info.value != 0:
        return info.value, 0, 0, None, None, None
    d = M.info()
    r, c, v = M.arrays()
    return info.value, d["nrows"], d["ncols"], r.copy(), c.copy(), v.copy()


def read_coo_mtx(path: str, cap: int = 1 << 22):
    """LACE's own read_z_coo_from_mtx (non-symmetric files):
    (info, n_rows, n_cols, row, col, val)."""
    dims = np.zeros(3, dtype=np.int32)
    r = np.zeros(cap, dtype=np.int32)
    c = np.zeros(cap, dtype=np.int32)
    v = np.zeros(cap)
    info = lib().ref_read_coo_mtx(path.encode(), _p(dims), cap, _p(r), _p(c), _p(v))
    z = int(dims[2])
    return info, int(dims[0]), int(dims[1]), r[:z].copy(), c[:z].copy(), v[:z].copy()


def write_csr_mtx(A: Mat, path: str, major: int = 101) -> int:
    """LACE's own data_zwrite_csr_mtx (major 101 row-major, 102 column-major)."""
    return lib().ref_write_csr_mtx(A.h, int(major), path.encode())


def read_mtx(path: str):
    """Read a Matrix Market file through LACE's own reader (data_z_csr_mtx is
    not wrapped; this parses the coordinate file in numpy the same way:
    symmetric entries mirrored, zero-based, columns sorted per row)."""
    with open(path) as f:
        header = f.readline().lower()
        line = f.readline()
        while line.startswith("%"):
            line = f.readline()
        nr, nc, nz = (int(t) for t in line.split())
        data = np.loadtxt(f, ndmin=2)
    r = data[:, 0].astype(np.int64) - 1
    c = data[:, 1].astype(np.int64) - 1
    v = data[:, 2].astype(np.float64) if data.shape[1] > 2 else np.ones(len(r))
    if "symmetric" in header:
        off = r != c
        r, c, v = np.concatenate([r, c[off]]), np.concatenate([c, r[off]]), np.concatenate([v, v[off]])
    order = np.lexsort((c, r))
    r, c, v = r[order], c[order], v[order]
    row = np.zeros(nr + 1, dtype=np.int32)
    np.cumsum(np.bincount(r, minlength=nr), out=row[1:])
    return nr, nc, row, c.astype(np.int32), v
