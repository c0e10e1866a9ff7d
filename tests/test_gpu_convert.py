"""GPU-side setup conversions (lace_gpu_*_device) against the host forms
(data_zmconvert / data_zmtranspose / data_rowindex, which tests/test_convert.py
pins to LACE's own outputs): array for array on the same seeded matrices,
every diagonal order of the split, the transpose of square and rectangular
matrices, CSR -> BCSR for several block sizes; malformed row pointers answer
DEV_ERR_ILLEGAL_VALUE."""
import ctypes as C

import numpy as np
import pytest

import convert_cases as CC

pytestmark = pytest.mark.gpu

NAMES = ["square", "no_diagonal", "empty_rows", "tall", "large"]


@pytest.fixture(scope="module")
def env(torch_cuda):
    import lace_gb300 as lg
    from lace_gb300 import dropin
    ctx = lg.Context(0)
    yield lg, dropin, torch_cuda, ctx
    ctx.close()


def host_convert(lg, dropin, n, m, r, c, v, old, new, diag=0, bs=0):
    A = dropin.csr(r, c, v, n)
    A.m.num_cols = m
    B = lg.DataMatrix()
    B.diagorder_type = diag
    B.blocksize = bs
    if new is None:
        assert lg.lib().data_zmtranspose(A.m, C.byref(B)) == 0
    else:
        assert lg.lib().data_zmconvert(A.m, C.byref(B), old, new) == 0
    nptr = B.num_rows + 1 if new is not None else max(B.num_rows, B.num_cols) + 1
    nidx = B.numblocks if bs else B.nnz
    ptr = np.ctypeslib.as_array(C.cast(B.row, C.POINTER(C.c_int)), shape=(nptr,)).copy()
    idx = np.ctypeslib.as_array(C.cast(B.col, C.POINTER(C.c_int)), shape=(max(nidx, 1),)).copy()[:nidx]
    nval = nidx * (bs * bs if bs else 1)
    val = np.ctypeslib.as_array(C.cast(B.val, C.POINTER(C.c_double)), shape=(max(nval, 1),)).copy()[:nval]
    dropin.free_matrix(B)
    return ptr, idx, val


def dev(torch, a, dtype):
    return torch.tensor(np.asarray(a), dtype=dtype, device="cuda")


@pytest.mark.parametrize("name", NAMES)
@pytest.mark.parametrize("lower,diag", [(1, CC.UNITY), (1, CC.VALUE), (1, CC.ZERO), (1, CC.NODIAG), (1, 0),
                                        (0, CC.UNITY), (0, CC.VALUE), (0, CC.ZERO), (0, CC.NODIAG), (0, 0)])
def test_split_equals_host(env, name, lower, diag):
    lg, dropin, torch, ctx = env
    n, m, r, c, v = CC.matrices()[name]
    hp, hi, hv = host_convert(lg, dropin, n, m, r, c, v, CC.CSR, CC.CSRL if lower else CC.CSRU, diag)
    dr, dc, dv = dev(torch, r, torch.int32), dev(torch, c, torch.int32), dev(torch, v, torch.float64)
    L = lg.lib()
    cnt = C.c_int()
    brow = torch.zeros(n + 1, dtype=torch.int32, device="cuda")
    assert L.lace_gpu_csr_split_device(ctx.h, n, dr.data_ptr(), dc.data_ptr(), dv.data_ptr(), lower, diag,
                                       C.byref(cnt), brow.data_ptr(), None, None) == 0
    bcol = torch.zeros(max(cnt.value, 1), dtype=torch.int32, device="cuda")
    bval = torch.zeros(max(cnt.value, 1), dtype=torch.float64, device="cuda")
    assert L.lace_gpu_csr_split_device(ctx.h, n, dr.data_ptr(), dc.data_ptr(), dv.data_ptr(), lower, diag,
                                       C.byref(cnt), brow.data_ptr(), bcol.data_ptr(), bval.data_ptr()) == 0
    k = cnt.value
    assert np.array_equal(brow.cpu().numpy(), hp)
    assert np.array_equal(bcol.cpu().numpy()[:k], hi[:k]) and np.array_equal(bval.cpu().numpy()[:k], hv[:k])
    # LACE's nnz may also count a lower split's default diagonal, which no row holds
    assert hp[-1] == k


@pytest.mark.parametrize("name", NAMES)
def test_transpose_and_rowindex_equal_host(env, name):
    lg, dropin, torch, ctx = env
    n, m, r, c, v = CC.matrices()[name]
    hp, hi, hv = host_convert(lg, dropin, n, m, r, c, v, None, None)
    dr, dc, dv = dev(torch, r, torch.int32), dev(torch, c, torch.int32), dev(torch, v, torch.float64)
    nnz = len(c)
    tptr = torch.zeros(m + 1, dtype=torch.int32, device="cuda")
    tidx = torch.zeros(max(nnz, 1), dtype=torch.int32, device="cuda")
    tval = torch.zeros(max(nnz, 1), dtype=torch.float64, device="cuda")
    L = lg.lib()
    assert L.lace_gpu_csr_transpose_device(ctx.h, n, m, dr.data_ptr(), dc.data_ptr(), dv.data_ptr(),
                                           tptr.data_ptr(), tidx.data_ptr(), tval.data_ptr()) == 0
    assert np.array_equal(tptr.cpu().numpy(), hp[:m + 1])
    assert np.array_equal(tidx.cpu().numpy()[:nnz], hi) and np.array_equal(tval.cpu().numpy()[:nnz], hv)
    ridx = torch.zeros(max(nnz, 1), dtype=torch.int32, device="cuda")
    assert L.lace_gpu_rowindex_device(ctx.h, n, dr.data_ptr(), ridx.data_ptr()) == 0
    assert np.array_equal(ridx.cpu().numpy()[:nnz], np.repeat(np.arange(n), np.diff(r)))


@pytest.mark.parametrize("name", ["square", "empty_rows", "large"])
@pytest.mark.parametrize("bs", [2, 3, 5])
def test_bcsr_equals_host(env, name, bs):
    lg, dropin, torch, ctx = env
    n, m, r, c, v = CC.matrices()[name]
    hp, hi, hv = host_convert(lg, dropin, n, m, r, c, v, CC.CSR, CC.BCSR, bs=bs)
    dr, dc, dv = dev(torch, r, torch.int32), dev(torch, c, torch.int32), dev(torch, v, torch.float64)
    nbr = (n + bs - 1) // bs
    L = lg.lib()
    nb = C.c_int()
    brow = torch.zeros(nbr + 1, dtype=torch.int32, device="cuda")
    assert L.lace_gpu_csr_to_bcsr_device(ctx.h, n, dr.data_ptr(), dc.data_ptr(), dv.data_ptr(), bs, C.byref(nb),
                                         brow.data_ptr(), None, None) == 0
    bcol = torch.zeros(max(nb.value, 1), dtype=torch.int32, device="cuda")
    bval = torch.zeros(max(nb.value, 1) * bs * bs, dtype=torch.float64, device="cuda")
    assert L.lace_gpu_csr_to_bcsr_device(ctx.h, n, dr.data_ptr(), dc.data_ptr(), dv.data_ptr(), bs, C.byref(nb),
                                         brow.data_ptr(), bcol.data_ptr(), bval.data_ptr()) == 0
    k = nb.value
    assert np.array_equal(brow.cpu().numpy(), hp)
    assert np.array_equal(bcol.cpu().numpy()[:k], hi) and np.array_equal(bval.cpu().numpy()[:k * bs * bs], hv)


def test_malformed_rows_are_rejected(env):
    lg, dropin, torch, ctx = env
    n, m, r, c, v = CC.matrices()["square"]
    bad = r.copy()
    bad[10] = bad[9] - 1  # decreasing
    dr, dc, dv = dev(torch, bad, torch.int32), dev(torch, c, torch.int32), dev(torch, v, torch.float64)
    L = lg.lib()
    cnt = C.c_int()
    out = torch.zeros(len(c), dtype=torch.int32, device="cuda")
    assert L.lace_gpu_csr_split_device(ctx.h, n, dr.data_ptr(), dc.data_ptr(), dv.data_ptr(), 1, CC.UNITY,
                                       C.byref(cnt), None, None, None) == lg.DEV_ERR_ILLEGAL_VALUE
    assert L.lace_gpu_rowindex_device(ctx.h, n, dr.data_ptr(), out.data_ptr()) == lg.DEV_ERR_ILLEGAL_VALUE
    # a column outside the matrix in the transpose
    cc = c.copy()
    cc[3] = m + 5
    dr2, dc2 = dev(torch, r, torch.int32), dev(torch, cc, torch.int32)
    tptr = torch.zeros(m + 1, dtype=torch.int32, device="cuda")
    tval = torch.zeros(len(c), dtype=torch.float64, device="cuda")
    assert L.lace_gpu_csr_transpose_device(ctx.h, n, m, dr2.data_ptr(), dc2.data_ptr(), dv.data_ptr(),
                                           tptr.data_ptr(), out.data_ptr(), tval.data_ptr()) == lg.DEV_ERR_ILLEGAL_VALUE
