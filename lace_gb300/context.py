"""GPU-resident solver context (the lace_gpu_* half of include/lace_gb300.h).

Vectors are torch CUDA float64 tensors (or raw device pointers as ints);
matrices are uploaded once from host numpy arrays (lace_gb300.problems.CSR /
BCSR) and stay in HBM with their factors and the Krylov workspace.
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass, field

import numpy as np

from . import (DEV_NOTCONVERGED, DEV_SUCCESS, PREC, TRSV, GmresLog, GmresParam, GpuOptions, LaceError,
               lib)


def _ptr(t) -> int:
    if t is None:
        return 0
    if isinstance(t, int):
        return t
    if hasattr(t, "data_ptr"):
        if not t.is_cuda:
            raise ValueError("device tensor expected")
        if not t.is_contiguous():
            raise ValueError("contiguous tensor expected")
        return t.data_ptr()
    raise TypeError(type(t))


def _chk(rc: int, what: str) -> int:
    if rc != DEV_SUCCESS:
        raise LaceError(rc, what)
    return rc


@dataclass
class GmresResult:
    converged: bool
    restarts: int            # index of the final cycle (LACE's gmres_log.restarts)
    search_directions: int   # directions of the final cycle
    total_iterations: int    # directions over all cycles
    initial_residual: float
    final_residual: float
    solve_time: float
    code: int
    hist: list = field(default_factory=list)


class Context:
    def __init__(self, device: int = 0, stream=None):
        self._lib = lib()
        self.h = C.c_void_p()
        sp = 0
        if stream is not None:
            sp = stream if isinstance(stream, int) else stream.cuda_stream
        _chk(self._lib.lace_gpu_ctx_create(C.byref(self.h), device, sp or None), "ctx_create")
        self.n = 0
        self.opts = GpuOptions()
        self._lib.lace_gpu_default_options(C.byref(self.opts))

    # -------------------------------------------------------------- setup
    def stream_ptr(self) -> int:
        return self._lib.lace_gpu_stream(self.h) or 0

    def set_options(self, precision: str | None = None, trsv: str | None = None,
                    jacobi_sweeps: int | None = None, use_graph: bool | None = None,
                    spmv_lanes: int | None = None, rows_per_lane: int | None = None,
                    monitor_orthog: bool | None = None, schedule: tuple | None = None) -> "Context":
        """schedule: (chunks per block, warps, cluster) pins the sync-free
        solve's schedule (see lace_gpu_options); (0, 0, 0) returns it to the
        autotune."""
        o = self.opts
        if precision is not None:
            o.precision = PREC[precision]
        if trsv is not None:
            o.trsv_mode = TRSV[trsv]
        if jacobi_sweeps is not None:
            o.jacobi_sweeps = int(jacobi_sweeps)
        if use_graph is not None:
            o.use_graph = int(bool(use_graph))
        if spmv_lanes is not None:
            o.spmv_lanes = int(spmv_lanes)
        if rows_per_lane is not None:
            o.trsv_rows_per_lane = int(rows_per_lane)
        if monitor_orthog is not None:
            o.monitor_orthog = int(bool(monitor_orthog))
        if schedule is not None:
            o.trsv_chunks_per_block, o.trsv_warps, o.trsv_cluster = (int(v) for v in schedule)
        _chk(self._lib.lace_gpu_set_options(self.h, C.byref(o)), "set_options")
        return self

    def upload(self, A) -> "Context":
        """A: problems.CSR or problems.BCSR (host arrays)."""
        row = np.ascontiguousarray(A.row, dtype=np.int32)
        col = np.ascontiguousarray(A.col, dtype=np.int32)
        val = np.ascontiguousarray(A.val, dtype=np.float64)
        if hasattr(A, "bs"):
            _chk(self._lib.lace_gpu_upload_bcsr_host(self.h, A.nb, A.bs, A.nblk, row.ctypes.data,
                                                     col.ctypes.data, val.ctypes.data), "upload_bcsr")
            self.n = A.nb * A.bs
        else:
            _chk(self._lib.lace_gpu_upload_csr_host(self.h, A.n, A.nnz, row.ctypes.data, col.ctypes.data,
                                                    val.ctypes.data), "upload_csr")
            self.n = A.n
        return self

    def upload_device(self, n: int, nnz: int, row, col, val) -> "Context":
        _chk(self._lib.lace_gpu_upload_csr_device(self.h, n, nnz, _ptr(row), _ptr(col), _ptr(val)),
             "upload_csr_device")
        self.n = n
        return self

    def update_values(self, val) -> None:
        _chk(self._lib.lace_gpu_update_values_device(self.h, _ptr(val)), "update_values")

    # ------------------------------------------------------------ kernels
    def parilu0(self, sweeps: int, residual: bool = True) -> tuple[float, float]:
        """`sweeps` synchronous sweeps; returns (last normalised step,
        ||(A-LU)|_S||_F/||A||_F), the residual only when asked for (it is one
        more kernel over A's pattern; NaN otherwise)."""
        step = C.c_double()
        nl = C.c_double(float("nan"))
        _chk(self._lib.lace_gpu_parilu0(self.h, int(sweeps), C.byref(step), C.byref(nl) if residual else None),
             "parilu0")
        return step.value, nl.value

    def spmv(self, x, y, alpha: float = 1.0, beta: float = 0.0) -> None:
        _chk(self._lib.lace_gpu_spmv(self.h, alpha, _ptr(x), beta, _ptr(y)), "spmv")

    def sptrsv(self, which: int, b, x) -> None:
        """which: 0 L, 1 U, 2 U^T, 3 L^T."""
        _chk(self._lib.lace_gpu_sptrsv(self.h, int(which), _ptr(b), _ptr(x)), "sptrsv")

    def apply_precond(self, q, z) -> None:
        _chk(self._lib.lace_gpu_apply_precond(self.h, _ptr(q), _ptr(z)), "apply_precond")

    def trsv_schedule(self) -> tuple:
        """(rows per lane, chunks per block, warps per CTA, CTAs per cluster)
        of the sync-free solves, once the first solve has tuned it."""
        out = (C.c_int * 4)()
        _chk(self._lib.lace_gpu_get_trsv_schedule(self.h, out), "get_trsv_schedule")
        return tuple(out)

    def precond_enqueue(self, q, z) -> None:
        """z = M^{-1} q as the FGMRES cycle applies it (q, z in the factor
        precision's vector type: float32 unless precision is fp64), enqueued
        on the context's stream without waiting - for timing."""
        _chk(self._lib.lace_gpu_precond_enqueue(self.h, _ptr(q), _ptr(z)), "precond_enqueue")

    def fgmres(self, b, x, search_max: int = 30, restart_max: int = 20, rtol: float = 1e-10,
               tol_type: int = 1, orthogonalization: str = "householder", reorth: int = 0,
               restarted: bool = True) -> GmresResult:
        """FGMRES on device vectors b, x (x: initial guess in, solution out).
        orthogonalization "householder" (LACE's data_fgmres_householder_restart)
        or "mgs" (modified Gram-Schmidt: data_fgmres_restart, or data_fgmres
        when restarted is False; reorth as LACE's gmres_par->reorth)."""
        par = GmresParam()
        par.search_max = search_max
        par.restart_max = restart_max
        par.rtol = rtol
        par.tol_type = tol_type
        par.reorth = reorth
        log = GmresLog()
        tot = C.c_int()
        if orthogonalization == "mgs":
            rc = self._lib.lace_gpu_fgmres_mgs(self.h, _ptr(b), _ptr(x), C.byref(par), int(bool(restarted)),
                                               C.byref(log), C.byref(tot))
        elif orthogonalization == "householder":
            rc = self._lib.lace_gpu_fgmres_householder(self.h, _ptr(b), _ptr(x), C.byref(par), C.byref(log),
                                                       C.byref(tot))
        else:
            raise ValueError(f"orthogonalization {orthogonalization!r}: 'householder' or 'mgs'")
        if rc not in (DEV_SUCCESS, DEV_NOTCONVERGED):
            raise LaceError(rc, "fgmres_" + orthogonalization)
        return GmresResult(rc == DEV_SUCCESS, log.restarts, log.search_directions, tot.value,
                           log.initial_residual, log.final_residual, log.solve_time, rc)

    def solve_stats(self) -> dict:
        """The last FGMRES solve: directions the Gram-Schmidt variant
        reorthogonalised, and whether its second pass is a conditional graph
        node."""
        out = (C.c_int * 4)()
        rc = self._lib.lace_gpu_get_solve_stats(self.h, out)
        if rc != DEV_SUCCESS:
            raise LaceError(rc, "get_solve_stats")
        return {"reorthogonalised": out[0], "conditional_nodes": bool(out[1]), "one_kernel_step": bool(out[2]),
                "one_kernel_householder_step": bool(out[3])}

    def orthog_history(self) -> np.ndarray:
        """||I - Q^T Q||_inf after every direction of the last solve (the
        monitor_orthog option)."""
        cnt = C.c_int()
        _chk(self._lib.lace_gpu_get_orthog_history(self.h, None, 0, C.byref(cnt)), "get_orthog_history")
        out = np.zeros(max(1, cnt.value))
        _chk(self._lib.lace_gpu_get_orthog_history(self.h, out.ctypes.data, cnt.value, C.byref(cnt)),
             "get_orthog_history")
        return out[:cnt.value]

    def time_arnoldi_step(self, orthogonalization: str = "householder", j: int = 15, reps: int = 20) -> float:
        """Seconds per launch of the one-kernel Arnoldi step j, replayed on the
        basis of the last solve (overwrites that solve's cycle state)."""
        t = C.c_double()
        rc = self._lib.lace_gpu_time_arnoldi_step(self.h, 1 if orthogonalization == "mgs" else 0, int(j),
                                                  int(reps), C.byref(t))
        if rc != DEV_SUCCESS:
            raise LaceError(rc, "time_arnoldi_step")
        return t.value

    def backward(self, x, dLdx, dLdb=None, dLdA=None, search_max: int = 30, restart_max: int = 20,
                 rtol: float = 1e-10, tol_type: int = 1) -> int:
        par = GmresParam()
        par.search_max = search_max
        par.restart_max = restart_max
        par.rtol = rtol
        par.tol_type = tol_type
        tot = C.c_int()
        rc = self._lib.lace_gpu_solve_backward(self.h, _ptr(x), _ptr(dLdx), C.byref(par), _ptr(dLdb) or None,
                                               _ptr(dLdA) or None, C.byref(tot))
        if rc not in (DEV_SUCCESS, DEV_NOTCONVERGED):
            raise LaceError(rc, "solve_backward")
        return tot.value

    def close(self) -> None:
        if self.h:
            self._lib.lace_gpu_ctx_destroy(self.h)
            self.h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()
