"""Cuthill-McKee orderings (data_reorder_cuthill_mckee, src/cuthill_mckee.cpp:53)
and the reorder dispatch (data_sparse_reorder, src/reorder.cpp:167) against
the oracle's restatement of the ordering LACE's source describes (LACE's own
routine reads outside its arrays on ordinary meshes, so it gives no
reproducible result to compare with): the numbering array for array on
meshes, random and unsymmetric patterns, several components and isolated
nodes; the permuted matrix against a dense permutation; errors."""
import ctypes as C

import numpy as np
import pytest

import lace_gb300 as lg
from lace_gb300 import dropin
from lace_gb300 import problems as P
from oracle import oracle as orc

_libc = C.CDLL(None)
_libc.posix_memalign.argtypes = [C.POINTER(C.c_void_p), C.c_size_t, C.c_size_t]
_libc.free.argtypes = [C.c_void_p]


def random_pattern(n, per_row, seed, symmetric=True, components=1, isolated=0):
    """A random pattern with the diagonal, over `components` disconnected
    groups of nodes, plus `isolated` nodes with only their diagonal."""
    rng = np.random.default_rng(seed)
    groups = np.array_split(rng.permutation(n - isolated), components)
    ent = {(i, i) for i in range(n)}
    for g in groups:
        for i in g:
            for j in rng.choice(g, size=min(per_row, len(g)), replace=False):
                ent.add((int(i), int(j)))
                if symmetric:
                    ent.add((int(j), int(i)))
    ent = sorted(ent)
    row = np.zeros(n + 1, dtype=np.int32)
    np.cumsum(np.bincount([e[0] for e in ent], minlength=n), out=row[1:])
    return row, np.array([e[1] for e in ent], dtype=np.int32)


def cases():
    A = P.convdiff3d(6)
    L = P.laplace2d(13, 9)
    T = P.trefethen(19)
    out = {"convdiff6": (A.n, A.row, A.col), "laplace13x9": (L.n, L.row, L.col), "trefethen19": (T.n, T.row, T.col)}
    out["random"] = (300,) + random_pattern(300, 4, 1)
    out["unsymmetric"] = (257,) + random_pattern(257, 3, 2, symmetric=False)
    out["components"] = (400,) + random_pattern(400, 3, 3, components=5, isolated=7)
    out["one"] = (1, np.array([0, 1], dtype=np.int32), np.array([0], dtype=np.int32))
    # unsorted rows with a repeated column
    out["unsorted"] = (4, np.array([0, 3, 5, 7, 9], dtype=np.int32),
                       np.array([2, 0, 2, 1, 0, 3, 2, 3, 1], dtype=np.int32))
    return out


def container(n, row, col, val=None, storage=dropin.Magma_CSR, bs=0):
    """A LACE container whose arrays come from posix_memalign, as LACE's do
    (data_sparse_reorder frees and replaces them)."""
    m = lg.DataMatrix()
    m.storage_type = storage
    m.num_rows = m.num_cols = n
    ld = bs * bs if bs else 1
    nz = int(row[n])
    if val is None:
        val = np.arange(1, nz * ld + 1, dtype=np.float64)
    for name, arr in (("row", np.ascontiguousarray(row, dtype=np.int32)),
                      ("col", np.ascontiguousarray(col, dtype=np.int32)),
                      ("val", np.ascontiguousarray(val, dtype=np.float64))):
        p = C.c_void_p()
        assert _libc.posix_memalign(C.byref(p), 64, max(arr.nbytes, 64)) == 0
        C.memmove(p, arr.ctypes.data, arr.nbytes)
        setattr(m, name, p.value)
    if bs:
        m.blocksize, m.ldblock, m.numblocks = bs, ld, nz
    m.nnz = nz * ld
    return m


def arrays(m, n, ld=1):
    nz = np.ctypeslib.as_array(C.cast(m.row, C.POINTER(C.c_int)), shape=(n + 1,))[n]
    row = np.ctypeslib.as_array(C.cast(m.row, C.POINTER(C.c_int)), shape=(n + 1,)).copy()
    col = np.ctypeslib.as_array(C.cast(m.col, C.POINTER(C.c_int)), shape=(max(nz, 1),)).copy()[:nz]
    val = np.ctypeslib.as_array(C.cast(m.val, C.POINTER(C.c_double)), shape=(max(nz * ld, 1),)).copy()[:nz * ld]
    return row, col, val


def release(m):
    for f in ("row", "col", "val"):
        _libc.free(getattr(m, f))


@pytest.mark.parametrize("reverse", [False, True])
@pytest.mark.parametrize("name", sorted(cases()))
def test_cuthill_mckee_equals_oracle(name, reverse):
    n, row, col = cases()[name]
    m = container(n, row, col)
    nn_map = np.full(n, -1, dtype=np.int32)
    lg.lib().data_reorder_cuthill_mckee(C.byref(m), nn_map.ctypes.data_as(C.POINTER(C.c_int)), reverse)
    release(m)
    assert lg.lib().lace_gpu_last_error() == 0
    assert np.array_equal(np.sort(nn_map), np.arange(n))
    assert np.array_equal(nn_map, orc.cuthill_mckee(n, row, col, reverse))


def bandwidth(row, col):
    rid = np.repeat(np.arange(len(row) - 1), np.diff(row))
    return int(np.max(np.abs(rid - col))) if len(col) else 0


def test_reverse_cuthill_mckee_recovers_the_band():
    """A 5-point 40 x 25 grid numbered at random: RCM brings the bandwidth
    back to within twice the natural ordering's (40)."""
    L = P.laplace2d(40, 25)
    perm = np.random.default_rng(5).permutation(L.n)
    inv = np.argsort(perm)
    row, col, _ = orc.permute_csr(L.row, L.col, L.val, perm, inv)
    assert bandwidth(row, col) > 10 * 40
    m = container(L.n, row, col)
    Pv = np.zeros(L.n, dtype=np.int32)
    Pi = np.zeros(L.n, dtype=np.int32)
    ip = C.POINTER(C.c_int)
    assert lg.lib().data_sparse_reorder(C.byref(m), Pv.ctypes.data_as(ip), Pi.ctypes.data_as(ip), 2) == 0
    r2, c2, _ = arrays(m, L.n)
    release(m)
    assert bandwidth(r2, c2) <= 2 * 40


@pytest.mark.parametrize("reorder", [0, 1, 2, 7])
@pytest.mark.parametrize("name", ["convdiff6", "unsymmetric", "components", "unsorted"])
def test_sparse_reorder_permutes_a(name, reorder):
    n, row, col = cases()[name]
    rng = np.random.default_rng(reorder)
    val = rng.standard_normal(int(row[n]))
    m = container(n, row, col, val)
    Pv = np.full(n, -1, dtype=np.int32)
    Pi = np.full(n, -1, dtype=np.int32)
    ip = C.POINTER(C.c_int)
    assert lg.lib().data_sparse_reorder(C.byref(m), Pv.ctypes.data_as(ip), Pi.ctypes.data_as(ip), reorder) == 0
    r2, c2, v2 = arrays(m, n)
    release(m)
    if reorder in (1, 2):
        want_inv = orc.cuthill_mckee(n, row, col, reorder == 2)
    else:
        want_inv = np.arange(n)
    assert np.array_equal(Pi, want_inv)
    assert np.array_equal(Pv[Pi], np.arange(n))
    er, ec, ev = orc.permute_csr(row, col, val, Pv, Pi)
    assert np.array_equal(r2, er) and np.array_equal(c2, ec) and np.array_equal(v2, ev)
    # and as a dense matrix: B = A[P][:, P] (repeated columns summed)
    D = np.zeros((n, n))
    rid = np.repeat(np.arange(n), np.diff(row))
    np.add.at(D, (rid, col), val)
    E = np.zeros((n, n))
    np.add.at(E, (np.repeat(np.arange(n), np.diff(r2)), c2), v2)
    assert np.array_equal(E, D[np.ix_(Pv, Pv)])


def test_sparse_reorder_bcsr_moves_blocks():
    B = P.bcsr3d(3, seed=2)
    m = container(B.nb, B.row, B.col, np.asarray(B.val).reshape(-1), storage=dropin.Magma_BCSR, bs=B.bs)
    Pv = np.zeros(B.nb, dtype=np.int32)
    Pi = np.zeros(B.nb, dtype=np.int32)
    ip = C.POINTER(C.c_int)
    assert lg.lib().data_sparse_reorder(C.byref(m), Pv.ctypes.data_as(ip), Pi.ctypes.data_as(ip), 2) == 0
    r2, c2, v2 = arrays(m, B.nb, B.bs * B.bs)
    release(m)
    assert np.array_equal(Pi, orc.cuthill_mckee(B.nb, B.row, B.col, True))
    er, ec, ev = orc.permute_csr(B.row, B.col, np.asarray(B.val).reshape(-1), Pv, Pi, ld=B.bs * B.bs)
    assert np.array_equal(r2, er) and np.array_equal(c2, ec) and np.array_equal(v2, ev)


def test_amd_is_not_supported_and_leaves_a():
    n, row, col = cases()["convdiff6"]
    m = container(n, row, col)
    before = arrays(m, n)
    Pv = np.zeros(n, dtype=np.int32)
    ip = C.POINTER(C.c_int)
    assert lg.lib().data_sparse_reorder(C.byref(m), Pv.ctypes.data_as(ip), Pv.ctypes.data_as(ip), 3) == \
        lg.DEV_ERR_NOT_SUPPORTED
    after = arrays(m, n)
    release(m)
    assert all(np.array_equal(a, b) for a, b in zip(before, after))


def test_argument_errors():
    L = lg.lib()
    ip = C.POINTER(C.c_int)
    n, row, col = cases()["random"]
    nn_map = np.full(n, -7, dtype=np.int32)
    L.data_reorder_cuthill_mckee(None, nn_map.ctypes.data_as(ip), False)
    assert L.lace_gpu_last_error() == lg.DEV_ERR_INVALID_PTR
    bad = col.copy()
    bad[5] = n + 3
    m = container(n, row, bad)
    L.data_reorder_cuthill_mckee(C.byref(m), nn_map.ctypes.data_as(ip), True)
    assert L.lace_gpu_last_error() == lg.DEV_ERR_ILLEGAL_VALUE
    assert (nn_map == -7).all()
    assert L.data_sparse_reorder(C.byref(m), nn_map.ctypes.data_as(ip), nn_map.ctypes.data_as(ip), 2) == \
        lg.DEV_ERR_ILLEGAL_VALUE
    release(m)
    m = container(n, row, col, storage=dropin.Magma_CSCU)
    assert L.data_sparse_reorder(C.byref(m), nn_map.ctypes.data_as(ip), nn_map.ctypes.data_as(ip), 2) == \
        lg.DEV_ERR_NOT_SUPPORTED
    assert L.data_sparse_reorder(C.byref(m), None, nn_map.ctypes.data_as(ip), 2) == lg.DEV_ERR_INVALID_PTR
    release(m)


def test_empty_matrix():
    """n = 0: nothing to number or permute, no error."""
    L = lg.lib()
    ip = C.POINTER(C.c_int)
    m = container(0, np.zeros(1, dtype=np.int32), np.zeros(0, dtype=np.int32))
    nn_map = np.zeros(1, dtype=np.int32)
    L.data_reorder_cuthill_mckee(C.byref(m), nn_map.ctypes.data_as(ip), True)
    assert L.lace_gpu_last_error() == 0
    assert L.data_sparse_reorder(C.byref(m), nn_map.ctypes.data_as(ip), nn_map.ctypes.data_as(ip), 2) == 0
    release(m)


def test_python_wrappers():
    """dropin.cuthill_mckee / dropin.sparse_reorder: the same results as the
    entry points, LaceError for what the entry points refuse."""
    n, row, col = cases()["components"]
    for rev in (False, True):
        assert np.array_equal(dropin.cuthill_mckee(n, row, col, rev), orc.cuthill_mckee(n, row, col, rev))
    val = np.random.default_rng(3).standard_normal(len(col))
    r2, c2, v2, Pv, Pi = dropin.sparse_reorder(n, row, col, val, 1)
    er, ec, ev = orc.permute_csr(row, col, val, Pv, Pi)
    assert np.array_equal(r2, er) and np.array_equal(c2, ec) and np.array_equal(v2, ev)
    B = P.bcsr3d(3, seed=5)
    r2, c2, v2, Pv, Pi = dropin.sparse_reorder(B.nb, B.row, B.col, np.asarray(B.val), 2, blocksize=B.bs)
    er, ec, ev = orc.permute_csr(B.row, B.col, np.asarray(B.val).reshape(-1), Pv, Pi, ld=B.bs * B.bs)
    assert np.array_equal(r2, er) and np.array_equal(c2, ec) and np.array_equal(v2, ev)
    with pytest.raises(lg.LaceError):
        dropin.sparse_reorder(n, row, col, val, 3)
    bad = col.copy()
    bad[0] = n
    with pytest.raises(lg.LaceError):
        dropin.cuthill_mckee(n, row, bad)
