"""The setup conversions (data_zmconvert, data_zmtranspose, data_rowindex)
against LACE's: every field and array of the output, on generated matrices
(golden digests of LACE's own outputs; live when LACE's tree is present)."""
import ctypes as C

import numpy as np
import pytest

import lace_gb300 as lg
from lace_gb300 import dropin
from oracle import reference as ref
import convert_cases as CC

G = np.load(__import__("os").path.join(__import__("os").path.dirname(__file__), "golden", "lace_golden.npz"))
_libc = C.CDLL(None)
_libc.free.argtypes = [C.c_void_p]
JOBS = {j[0]: j for j in CC.jobs()}


def ours_input(spec):
    st, n, m, r, c, v, bs = CC.job_input(spec)
    A = dropin.Mat()
    A.m.storage_type = st
    A.m.num_rows, A.m.num_cols = n, m
    A.m.fill_mode = dropin.MagmaFull
    A.m.major = dropin.MagmaRowMajor
    if bs:
        A.m.blocksize, A.m.ldblock, A.m.numblocks = bs, bs * bs, len(c)
        A.m.nnz = len(c) * bs * bs
    else:
        A.m.nnz = len(c)
    A.m.true_nnz = A.m.nnz
    A.m.row = A._own(r, np.int32)
    A.m.col = A._own(c, np.int32)
    A.m.val = A._own(v, np.float64)
    return A


def release(m):
    for f in ("val", "row", "col", "rowidx"):
        p = getattr(m, f)
        if p:
            _libc.free(p)


def run_ours(key):
    _, spec, old, new, d, bs = JOBS[key]
    A = ours_input(spec)
    B = lg.DataMatrix()
    B.diagorder_type = d
    B.blocksize = bs
    if new is None:
        rc = lg.lib().data_zmtranspose(A.m, C.byref(B))
    else:
        rc = lg.lib().data_zmconvert(A.m, C.byref(B), old, new)
    assert rc == 0, (key, rc)
    snap = CC.snapshot(B, CC.nptr_of(B))
    release(B)
    return snap


def run_lace(key):
    _, spec, old, new, d, bs = JOBS[key]
    st, n, m, r, c, v, bsi = CC.job_input(spec)
    if st == CC.COO:
        L = ref.lib()
        r, c, v = (np.ascontiguousarray(x, dtype=t) for x, t in ((r, np.int32), (c, np.int32), (v, np.float64)))
        A = ref.Mat(L.ref_coo_new(n, m, len(c), r.ctypes.data, c.ctypes.data, v.ctypes.data), L)
    else:
        A = ref.Mat.from_arrays(st, n, m, r, c, v, blocksize=bsi)
    if spec.startswith("csrl0:"):
        C.cast(A.h, C.POINTER(lg.DataMatrix))[0].nnz = len(c)
    if new is None:
        B = ref.transpose(A)
    else:
        B = ref.Mat(A.L.ref_convert_bs(A.h, old, new, d, bs), A.L) if bs else ref.convert(A, old, new, d)
    m_ = lg.DataMatrix.from_address(B.h.value)
    return CC.snapshot(m_, CC.nptr_of(m_))


@pytest.mark.parametrize("key", sorted(JOBS))
def test_conversion_equals_lace(key):
    s = run_ours(key)
    assert CC.digest(s) == str(G[key][0]), s["fields"]


@pytest.mark.skipif(not ref.available(), reason="LACE source tree not present")
@pytest.mark.parametrize("key", [k for k in sorted(JOBS) if "large" not in k][::3])
def test_conversion_live(key):
    a, b = run_ours(key), run_lace(key)
    assert a["fields"] == b["fields"]
    for k in ("row", "col", "val", "rowidx"):
        assert np.array_equal(a[k], b[k]), k


def test_rowindex():
    n, m, r, c, v = CC.matrices()["empty_rows"]
    A = ours_input("empty_rows")
    p = C.c_void_p()
    assert lg.lib().data_rowindex(C.byref(A.m), C.byref(p)) == 0
    got = np.ctypeslib.as_array(C.cast(p, C.POINTER(C.c_int)), (len(c),)).copy()
    _libc.free(p)
    assert np.array_equal(got, np.repeat(np.arange(n), np.diff(r)))


def test_unsupported_pairs_leave_the_output_alone():
    A = ours_input("square")
    B = lg.DataMatrix()
    B.num_rows = 7
    assert lg.lib().data_zmconvert(A.m, C.byref(B), CC.CSR, 614) == lg.DEV_ERR_NOT_SUPPORTED  # dense
    assert lg.lib().data_zmconvert(A.m, C.byref(B), CC.CSR, CC.BCSR) == lg.DEV_ERR_NOT_SUPPORTED  # no block size
    assert B.num_rows == 7 and not B.val and not B.row
    assert lg.lib().data_zmconvert(A.m, None, CC.CSR, CC.CSRL) == lg.DEV_ERR_INVALID_PTR
    assert lg.lib().data_rowindex(None, None) == lg.DEV_ERR_INVALID_PTR
