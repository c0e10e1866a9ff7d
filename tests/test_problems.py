"""CPU tests of the synthetic workload generators (sizes of the benchmark
configurations, structure, seeding)."""
import numpy as np
import pytest

from lace_gb300 import problems as P


def _sorted_with_diag(A):
    for i in range(A.n):
        c = A.col[A.row[i]:A.row[i + 1]]
        assert np.all(np.diff(c) > 0)
        assert i in c


def test_laplace_config_sizes():
    A = P.laplace2d(64)
    assert (A.n, A.nnz) == (4096, 20224)
    _sorted_with_diag(P.laplace2d(8))
    d = P.laplace2d(5).to_dense()
    assert np.allclose(d, d.T) and np.all(np.diag(d) == 4)


@pytest.mark.parametrize("shape", [(6, 5, 4), (9, 9, 9), (32, 32, 32)])
def test_convdiff_sizes_and_structure(shape):
    nx, ny, nz = shape
    A = P.convdiff3d(nx, ny, nz)
    assert A.n == nx * ny * nz
    assert A.nnz == 7 * A.n - 2 * (nx * ny + ny * nz + nx * nz)
    if A.n < 500:
        _sorted_with_diag(A)
        d = A.to_dense()
        assert not np.allclose(d, d.T)  # upwind convection: nonsymmetric
        # rows are weakly diagonally dominant (strictly at the boundary)
        off = np.sum(np.abs(d), axis=1) - np.abs(np.diag(d))
        assert np.all(np.abs(np.diag(d)) >= off - 1e-12)
    # 128^3 (the benchmark): n = 2,097,152, nnz = 14,581,760 by the same formula
    n128 = 128 ** 3
    assert 7 * n128 - 6 * 128 * 128 == 14581760


def test_convdiff_peclet_definition():
    A = P.convdiff3d(4, pe=10.0)
    d = A.to_dense()
    i = 1 + 4 * (1 + 4 * 1)  # interior cell (1,1,1)
    assert d[i, i] == pytest.approx(6 + 10 + 5 + 2.5)
    assert d[i, i - 1] == pytest.approx(-11.0) and d[i, i + 1] == pytest.approx(-1.0)
    assert d[i, i - 4] == pytest.approx(-6.0) and d[i, i - 16] == pytest.approx(-3.5)


def test_bcsr_config_structure():
    B = P.bcsr3d(5, seed=3)
    assert B.nb == 125 and B.bs == 5
    assert B.nblk == 7 * 125 - 6 * 25
    assert 7 * 64 ** 3 - 6 * 64 ** 2 == 1810432
    C = B.to_csr()
    assert C.n == 625 and C.nnz == B.nblk * 25
    d = C.to_dense()
    off = np.sum(np.abs(d), axis=1) - np.abs(np.diag(d))
    assert np.all(np.abs(np.diag(d)) >= 1.05 * off * (1 - 1e-12))
    assert np.array_equal(P.bcsr3d(5, seed=3).val, B.val)


def test_aniso_and_batch():
    A = P.aniso2d(10, 0.01)
    assert A.nnz == 5 * 100 - 40
    batch = P.batch_aniso(count=12, seed=4)
    assert len(batch) == 12
    for s in batch:
        assert 32 <= s.side <= 256 and 1e-3 <= s.eps <= 1.0
        assert s.A.nnz == 5 * s.side ** 2 - 4 * s.side
        assert s.B.shape == (4, s.A.n)
    again = P.batch_aniso(count=12, seed=4)
    assert [s.side for s in again] == [s.side for s in batch]


def test_trefethen_definition():
    T = P.trefethen(19)
    d = T.to_dense()
    assert list(np.diag(d)[:5]) == [3, 5, 7, 11, 13]
    assert d[0, 1] == 1 and d[0, 2] == 1 and d[0, 3] == 0 and d[0, 4] == 1 and d[0, 16] == 1
    assert T.nnz == 147
