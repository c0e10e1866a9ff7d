"""CPU tests of the C-ABI boundary: the library loads without a GPU, exports
every symbol include/lace_gb300.h declares, its structs are byte-compatible
with LACE's, and host-side argument checks answer like LACE does."""
import ctypes as C
import os
import re
import subprocess

import numpy as np
import pytest

import lace_gb300 as lg
from lace_gb300 import dropin
from oracle import reference as ref

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADER = os.path.join(ROOT, "include", "lace_gb300.h")


def declared_functions():
    txt = open(HEADER).read()
    txt = re.sub(r"/\*.*?\*/", "", txt, flags=re.S)
    names = re.findall(r"^\s*(?:const\s+)?[A-Za-z_][\w\s\*]*?\b([A-Za-z_]\w*)\s*\([^;{]*\)\s*;", txt,
                       flags=re.M)
    return sorted(set(n for n in names if n.startswith(("data_", "lace_gpu_", "read_z_"))))


def test_library_exports_every_declared_symbol():
    L = lg.lib()
    names = declared_functions()
    assert len(names) >= 30
    for n in names:
        assert hasattr(L, n), n
    # and the Python mirror binds exactly these
    assert sorted(lg.SIGNATURES) == names


def test_exported_symbols_by_nm():
    out = subprocess.run(["nm", "-D", "--defined-only", lg.LIB_PATH], capture_output=True, text=True).stdout
    exported = {l.split()[-1] for l in out.splitlines() if " T " in l}
    for n in declared_functions():
        assert n in exported, n


def test_struct_layout_matches_python_mirror():
    assert lg.abi_layout() == lg.expected_abi_layout()
    assert C.sizeof(lg.DataMatrix) == 384
    assert C.sizeof(lg.PrecondLog) == 128
    assert C.sizeof(lg.GmresLog) == 64
    assert C.sizeof(lg.GmresParam) == 64


@pytest.mark.skipif(not os.path.isdir(os.path.join(ref.REF_SRC, "include")), reason="LACE tree not present")
def test_struct_layout_matches_lace_headers(tmp_path):
    """Compile against LACE's own include/sparse_types.h and compare."""
    src = tmp_path / "layout.cpp"
    src.write_text(r'''
#include <cstdio>
#include <cstddef>
#include "sparse_types.h"
int main() {
  printf("%zu %zu %zu %zu %zu %zu %zu %zu %zu %zu %zu %zu %zu %zu %zu %zu ",
    sizeof(data_d_matrix), offsetof(data_d_matrix, num_rows), offsetof(data_d_matrix, nnz),
    offsetof(data_d_matrix, val), offsetof(data_d_matrix, diag), offsetof(data_d_matrix, row),
    offsetof(data_d_matrix, rowidx), offsetof(data_d_matrix, col), offsetof(data_d_matrix, list),
    offsetof(data_d_matrix, blockinfo), offsetof(data_d_matrix, blocksize), offsetof(data_d_matrix, ldblock),
    offsetof(data_d_matrix, numblocks), offsetof(data_d_matrix, major), offsetof(data_d_matrix, ld),
    offsetof(data_d_matrix, pad_cols));
  printf("%zu %zu %zu %zu %zu %zu %zu %zu %zu %zu %zu\n",
    sizeof(data_d_preconditioner_log), offsetof(data_d_preconditioner_log, tol),
    offsetof(data_d_preconditioner_log, omp_num_threads), sizeof(data_d_gmres_log),
    offsetof(data_d_gmres_log, solve_time), offsetof(data_d_gmres_log, original_residual),
    sizeof(data_d_gmres_param), offsetof(data_d_gmres_param, rtol), offsetof(data_d_gmres_param, restart_max),
    offsetof(data_d_gmres_param, parilu_reduction), offsetof(data_d_gmres_param, reorder));
}
''')
    exe = tmp_path / "layout"
    subprocess.run(["g++", "-w", "-I", os.path.join(ROOT, "oracle", "mkl_shim"), "-I",
                    os.path.join(ref.REF_SRC, "include"), str(src), "-o", str(exe)], check=True)
    vals = [int(v) for v in subprocess.run([str(exe)], capture_output=True, text=True).stdout.split()]
    assert vals == lg.abi_layout()


@pytest.mark.skipif(not os.path.isdir(os.path.join(ref.REF_SRC, "include")), reason="LACE tree not present")
def test_header_compiles_next_to_lace_headers(tmp_path):
    """A LACE caller includes both headers: every function both declare
    (the drop-ins, the Matrix Market files) must be declared alike."""
    src = tmp_path / "both.cpp"
    src.write_text('#include "sparse.h"\n#include "lace_gb300.h"\nint main() { return 0; }\n')
    r = subprocess.run(["g++", "-fsyntax-only", "-Werror", "-I", os.path.join(ref.REF_SRC, "include"), "-I",
                        os.path.join(ROOT, "oracle", "mkl_shim"), "-I", os.path.join(ROOT, "include"), str(src)],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr[-2000:]


def test_context_without_gpu_fails_loudly():
    import torch
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    with pytest.raises(lg.LaceError) as e:
        lg.Context(0)
    assert e.value.code == lg.DEV_ERR_NOT_INITIALIZED


def test_dropin_argument_checks_match_lace():
    """Checks that LACE makes before touching data answer the same way."""
    A = lg.problems.laplace2d(4)
    Am = dropin.csr(A.row, A.col, A.val, A.n)
    # data_z_spmv: dimension mismatch -> DEV_ERR_NOT_SUPPORTED (blas/zspmv.cpp:71-75)
    x = dropin.dense(np.ones(A.n + 1))
    y = dropin.dense(np.zeros(A.n))
    assert lg.lib().data_z_spmv(1.0, Am.ref, x.ref, 0.0, y.ref) == lg.DEV_ERR_NOT_SUPPORTED
    # unsupported storage -> DEV_ERR_NOT_SUPPORTED (:65-68)
    D = dropin.csr(A.row, A.col, A.val, A.n, storage=dropin.Magma_DENSE)
    x = dropin.dense(np.ones(A.n))
    assert lg.lib().data_z_spmv(1.0, D.ref, x.ref, 0.0, y.ref) == lg.DEV_ERR_NOT_SUPPORTED
    # data_parcsrtrsv: wrong storage / fill combinations -> -1 (src/trisolve.cpp:298-344)
    y, it, rc = dropin.parcsrtrsv(dropin.MagmaLower, dropin.Magma_CSRU, dropin.Magma_UNITY, A.row, A.col, A.val,
                                  np.ones(A.n))
    assert rc == -1
    y, it, rc = dropin.parcsrtrsv(dropin.MagmaUpper, dropin.Magma_CSRL, dropin.Magma_VALUE, A.row, A.col, A.val,
                                  np.ones(A.n))
    assert rc == -1


def test_new_entry_points_reject_null_arguments():
    """The Gram-Schmidt FGMRES, the solve facts and the step timing answer
    DEV_ERR_INVALID_PTR for missing arguments before any GPU work."""
    L = lg.lib()
    par = lg.GmresParam()
    log = lg.GmresLog()
    assert L.lace_gpu_fgmres_mgs(None, None, None, C.byref(par), 1, C.byref(log), None) == lg.DEV_ERR_INVALID_PTR
    assert L.lace_gpu_get_solve_stats(None, None) == lg.DEV_ERR_INVALID_PTR
    t = C.c_double()
    assert L.lace_gpu_time_arnoldi_step(None, 0, 1, 1, C.byref(t)) == lg.DEV_ERR_INVALID_PTR
    assert L.data_fgmres(None, None, None, None, None, None, None) == lg.DEV_ERR_INVALID_PTR
    assert L.data_fgmres_restart(None, None, None, None, None, None, None) == lg.DEV_ERR_INVALID_PTR
    assert L.read_z_csr_from_mtx(None, None, None, None, None, None, None, b"x.mtx") == lg.DEV_ERR_INVALID_PTR
    assert L.data_z_csr_mtx(None, b"x.mtx") == lg.DEV_ERR_INVALID_PTR
    assert L.read_z_coo_from_mtx(None, None, None, None, None, None, None, b"x.mtx") == lg.DEV_ERR_INVALID_PTR
    assert L.data_z_coo_mtx(None, b"x.mtx") == lg.DEV_ERR_INVALID_PTR


def test_error_strings():
    L = lg.lib()
    for code in (0, -101, -103, -104, -107, -113, -115, -116, -204, -205):
        assert len(L.lace_gpu_error_string(code)) > 3
