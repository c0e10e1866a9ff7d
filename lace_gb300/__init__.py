"""lace_gb300 - GB300 (sm_103a) preconditioned-solve path of LACE.

The compute path is liblace_gb300.so (hand-written CUDA kernels behind a C
ABI, include/lace_gb300.h).  This module is the Python host mirror of LACE's
interface for that path:

* ``Context`` - the GPU-resident API (lace_gpu_*): upload a CSR/BCSR
  matrix once, run ParILU(0) sweeps, SpMV, SpTRSV, FGMRES-Householder and
  its adjoint on device vectors (torch CUDA tensors or raw pointers).
* ``dropin`` - the LACE-named entry points (data_PariLU_v0_3,
  data_fgmres_householder_restart, data_z_spmv, data_parcsrtrsv,
  data_zilures) called through LACE's own data_d_matrix container.

There is no CPU fallback: importing works without a GPU (so bindings and the
ABI can be inspected), but every compute call goes to the CUDA library and
fails loudly when it, or a GPU, is missing.
"""
from __future__ import annotations

import ctypes as C
import os

from . import problems  # noqa: F401  (workload generators)

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "liblace_gb300.so")

# error codes (include/dense_types.h:134-160)
DEV_SUCCESS = 0
DEV_ERR_NOT_INITIALIZED = -101
DEV_ERR_NOT_SUPPORTED = -103
DEV_ERR_ILLEGAL_VALUE = -104
DEV_ERR_INTERNAL_LIMIT = -107
DEV_ERR_DEVICE_ALLOC = -113
DEV_ERR_INVALID_PTR = -115
DEV_ERR_UNKNOWN = -116
DEV_ERR_NOT_IMPLEMENTED = -117
DEV_ERR_BADPRECOND = -204
DEV_NOTCONVERGED = -205

PREC = {"fp64": 0, "fp32": 1, "bf16": 2}
TRSV = {"syncfree": 0, "levels": 1, "jacobi": 2, "none": 3}

_lib = None


class LaceError(RuntimeError):
    def __init__(self, code: int, what: str = ""):
        msg = lib().lace_gpu_error_string(code).decode() if _lib is not None else str(code)
        super().__init__(f"{what}: {msg} ({code})" if what else f"{msg} ({code})")
        self.code = code


def lib() -> C.CDLL:
    """Load liblace_gb300.so (built by build(); never a Python fallback)."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise RuntimeError(f"{LIB_PATH} is missing: run lace_gb300.build.build() "
                               "(python -c 'import __graft_entry__ as g; g.build()')")
        _lib = C.CDLL(LIB_PATH)
        _declare(_lib)
    return _lib


# --------------------------------------------------------------- C structs

class GpuOptions(C.Structure):
    _fields_ = [("precision", C.c_int), ("trsv_mode", C.c_int), ("jacobi_sweeps", C.c_int),
                ("jacobi_tol", C.c_double), ("use_graph", C.c_int), ("spmv_lanes", C.c_int),
                ("trsv_rows_per_lane", C.c_int), ("monitor_orthog", C.c_int),
                ("trsv_chunks_per_block", C.c_int), ("trsv_warps", C.c_int), ("trsv_cluster", C.c_int)]


def _padded(fields):
    """ctypes fields with explicit padding to the given byte offsets:
    [(name, ctype, offset)], final ('__end__', None, size)."""
    out = []
    pos = 0
    k = 0
    for name, ct, off in fields:
        if off > pos:
            out.append((f"_pad{k}", C.c_char * (off - pos)))
            k += 1
            pos = off
        if ct is None:
            break
        out.append((name, ct))
        pos += C.sizeof(ct)
    return out


_vp = C.c_void_p
# LACE's data_d_matrix (include/sparse_types.h:14-41): pointer members and
# the struct are 64-byte aligned
DATA_D_MATRIX_LAYOUT = [
    ("storage_type", C.c_int, 0), ("sym", C.c_int, 4), ("diagorder_type", C.c_int, 8),
    ("fill_mode", C.c_int, 12), ("num_rows", C.c_int, 16), ("num_cols", C.c_int, 20),
    ("nnz", C.c_int, 24), ("max_nnz_row", C.c_int, 28), ("diameter", C.c_int, 32),
    ("true_nnz", C.c_int, 36), ("val", _vp, 64), ("diag", _vp, 128), ("row", _vp, 192),
    ("rowidx", _vp, 256), ("col", _vp, 320), ("list", _vp, 328), ("blockinfo", _vp, 336),
    ("blocksize", C.c_int, 344), ("ldblock", C.c_int, 348), ("numblocks", C.c_int, 352),
    ("alignment", C.c_int, 356), ("major", C.c_int, 360), ("ld", C.c_int, 364),
    ("pad_rows", C.c_int, 368), ("pad_cols", C.c_int, 372), ("__end__", None, 384)]


class DataMatrix(C.Structure):
    _fields_ = _padded(DATA_D_MATRIX_LAYOUT)


PRECOND_LOG_LAYOUT = [
    ("sweeps", C.c_int, 0), ("maxSweeps", C.c_int, 4), ("tol", C.c_double, 8),
    ("finalStep", C.c_double, 16), ("A_Frobenius", C.c_double, 24),
    ("precond_generation_time", C.c_double, 32), ("initial_residual", C.c_double, 40),
    ("initial_nonlinear_residual", C.c_double, 48), ("residual", C.c_double, 56),
    ("nonlinear_residual", C.c_double, 64), ("omp_num_threads", C.c_int, 72), ("__end__", None, 128)]


class PrecondLog(C.Structure):
    _fields_ = _padded(PRECOND_LOG_LAYOUT)


GMRES_LOG_LAYOUT = [
    ("restarts", C.c_int, 0), ("search_directions", C.c_int, 4), ("solve_time", C.c_double, 8),
    ("initial_residual", C.c_double, 16), ("final_residual", C.c_double, 24),
    ("scaled_residual", C.c_double, 32), ("original_residual", C.c_double, 40), ("__end__", None, 64)]


class GmresLog(C.Structure):
    _fields_ = _padded(GMRES_LOG_LAYOUT)


GMRES_PARAM_LAYOUT = [
    ("search_max", C.c_int, 0), ("tol_type", C.c_int, 4), ("rtol", C.c_double, 8),
    ("reorth", C.c_int, 16), ("user_csrtrsv_choice", C.c_int, 20), ("monitorOrthog", C.c_int, 24),
    ("restart_max", C.c_int, 28), ("precondition", C.c_int, 32), ("parilu_reduction", C.c_double, 40),
    ("reorder", C.c_int, 48), ("__end__", None, 64)]


class GmresParam(C.Structure):
    _fields_ = _padded(GMRES_PARAM_LAYOUT)


# every function the public header declares, with its ctypes signature
_i, _d, _p = C.c_int, C.c_double, C.c_void_p
_DM = C.POINTER(DataMatrix)
SIGNATURES = {
    "data_PariLU_v0_3": (None, [_DM, _DM, _DM, _d, C.POINTER(PrecondLog)]),
    "data_PariLU_v0_3_prescribedSweeps": (None, [_DM, _DM, _DM, _d, C.POINTER(PrecondLog)]),
    "data_PariLU_v0_3_gpu": (None, [_DM, _DM, _DM, _d, C.POINTER(PrecondLog), _i]),
    "data_PariLU_v0_3_gpu_prescribedSweeps": (None, [_DM, _DM, _DM, _d, C.POINTER(PrecondLog)]),
    "data_parcsrtrsv": (_i, [_i, _i, _i, _i, _p, _p, _p, _p, _p, _d, C.POINTER(_i)]),
    "data_z_spmv": (_i, [_d, _DM, _DM, _d, _DM]),
    "data_fgmres_householder_restart": (_i, [_DM, _DM, _DM, _DM, _DM, C.POINTER(GmresParam),
                                             C.POINTER(GmresLog)]),
    "data_fgmres_householder": (_i, [_DM, _DM, _DM, _DM, _DM, C.POINTER(GmresParam), C.POINTER(GmresLog)]),
    "data_fgmres_restart": (_i, [_DM, _DM, _DM, _DM, _DM, C.POINTER(GmresParam), C.POINTER(GmresLog)]),
    "data_fgmres": (_i, [_DM, _DM, _DM, _DM, _DM, C.POINTER(GmresParam), C.POINTER(GmresLog)]),
    "data_zilures": (_i, [DataMatrix, DataMatrix, DataMatrix, _DM, C.POINTER(_d), C.POINTER(_d)]),
    "data_zilures_bcsr": (_i, [DataMatrix, DataMatrix, DataMatrix, _DM, C.POINTER(_d), C.POINTER(_d)]),
    "read_z_csr_from_mtx": (_i, [C.POINTER(_i), C.POINTER(_i), C.POINTER(_i), C.POINTER(_i), C.POINTER(_p),
                                 C.POINTER(_p), C.POINTER(_p), C.c_char_p]),
    "data_z_csr_mtx": (_i, [_DM, C.c_char_p]),
    "read_z_coo_from_mtx": (_i, [C.POINTER(_i), C.POINTER(_i), C.POINTER(_i), C.POINTER(_i), C.POINTER(_p),
                                 C.POINTER(_p), C.POINTER(_p), C.c_char_p]),
    "data_z_coo_mtx": (_i, [_DM, C.c_char_p]),
    "data_zmconvert": (_i, [DataMatrix, _DM, _i, _i]),
    "data_zmtranspose": (_i, [DataMatrix, _DM]),
    "data_rowindex": (_i, [_DM, C.POINTER(_p)]),
    "data_reorder_cuthill_mckee": (None, [_DM, C.POINTER(_i), C.c_bool]),
    "data_sparse_reorder": (_i, [_DM, C.POINTER(_i), C.POINTER(_i), _i]),
    "data_zwrite_csr_mtx": (_i, [DataMatrix, _i, C.c_char_p]),
    "lace_gpu_default_options": (None, [C.POINTER(GpuOptions)]),
    "lace_gpu_dropin_set_options": (_i, [C.POINTER(GpuOptions)]),
    "lace_gpu_ctx_create": (_i, [C.POINTER(_p), _i, _p]),
    "lace_gpu_ctx_destroy": (_i, [_p]),
    "lace_gpu_set_options": (_i, [_p, C.POINTER(GpuOptions)]),
    "lace_gpu_stream": (_p, [_p]),
    "lace_gpu_upload_csr_host": (_i, [_p, _i, _i, _p, _p, _p]),
    "lace_gpu_upload_csr_device": (_i, [_p, _i, _i, _p, _p, _p]),
    "lace_gpu_upload_bcsr_host": (_i, [_p, _i, _i, _i, _p, _p, _p]),
    "lace_gpu_update_values_device": (_i, [_p, _p]),
    "lace_gpu_parilu0": (_i, [_p, _i, C.POINTER(_d), C.POINTER(_d)]),
    "lace_gpu_spmv": (_i, [_p, _d, _p, _d, _p]),
    "lace_gpu_apply_precond": (_i, [_p, _p, _p]),
    "lace_gpu_precond_enqueue": (_i, [_p, _p, _p]),
    "lace_gpu_get_trsv_schedule": (_i, [_p, _p]),
    "lace_gpu_parcsrtrsv_noalloc": (_i, [_i, _i, _i, _i, _p, _p, _p, _p, _p, _d, _p, _p]),
    "lace_gpu_sptrsv": (_i, [_p, _i, _p, _p]),
    "lace_gpu_fgmres_householder": (_i, [_p, _p, _p, C.POINTER(GmresParam), C.POINTER(GmresLog),
                                         C.POINTER(_i)]),
    "lace_gpu_fgmres_mgs": (_i, [_p, _p, _p, C.POINTER(GmresParam), _i, C.POINTER(GmresLog), C.POINTER(_i)]),
    "lace_gpu_get_solve_stats": (_i, [_p, _p]),
    "lace_gpu_time_arnoldi_step": (_i, [_p, _i, _i, _i, C.POINTER(_d)]),
    "lace_gpu_solve_backward": (_i, [_p, _p, _p, C.POINTER(GmresParam), _p, _p, C.POINTER(_i)]),
    "lace_gpu_last_error": (_i, []),
    "lace_gpu_selftest_wait_limit": (_i, [_i, C.POINTER(_i)]),
    "lace_gpu_inject_alloc_failure": (None, [_i]),
    "lace_gpu_get_orthog_history": (_i, [_p, _p, _i, C.POINTER(_i)]),
    "lace_gpu_error_string": (C.c_char_p, [_i]),
    "lace_gpu_rowindex_device": (_i, [_p, _i, _p, _p]),
    "lace_gpu_csr_split_device": (_i, [_p, _i, _p, _p, _p, _i, _i, C.POINTER(_i), _p, _p, _p]),
    "lace_gpu_csr_transpose_device": (_i, [_p, _i, _i, _p, _p, _p, _p, _p, _p]),
    "lace_gpu_csr_to_bcsr_device": (_i, [_p, _i, _p, _p, _p, _i, C.POINTER(_i), _p, _p, _p]),
    "lace_gpu_batch_create": (_i, [C.POINTER(_p), _p, _i, _p, _p, _p, _p, _p, _p, _i]),
    "lace_gpu_batch_destroy": (_i, [_p]),
    "lace_gpu_batch_solve": (_i, [_p, _i, _i, _i, _d, _p, _p, _p]),
    "lace_gpu_abi_layout": (_i, [C.POINTER(_i), _i]),
}


def _declare(L: C.CDLL) -> None:
    for name, (res, args) in SIGNATURES.items():
        f = getattr(L, name)
        f.restype = res
        f.argtypes = args


def abi_layout() -> list[int]:
    buf = (C.c_int * 64)()
    n = lib().lace_gpu_abi_layout(buf, 64)
    return list(buf[:n])


def expected_abi_layout() -> list[int]:
    """The same quantities from the ctypes mirrors above."""
    DM, PL, GL, GP = DataMatrix, PrecondLog, GmresLog, GmresParam
    return [C.sizeof(DM), DM.num_rows.offset, DM.nnz.offset, DM.val.offset, DM.diag.offset,
            DM.row.offset, DM.rowidx.offset, DM.col.offset, DM.list.offset, DM.blockinfo.offset,
            DM.blocksize.offset, DM.ldblock.offset, DM.numblocks.offset, DM.major.offset, DM.ld.offset,
            DM.pad_cols.offset, C.sizeof(PL), PL.tol.offset, PL.omp_num_threads.offset, C.sizeof(GL),
            GL.solve_time.offset, GL.original_residual.offset, C.sizeof(GP), GP.rtol.offset,
            GP.restart_max.offset, GP.parilu_reduction.offset, GP.reorder.offset]


from .context import Context, GmresResult  # noqa: E402,F401
from . import dropin  # noqa: E402,F401
