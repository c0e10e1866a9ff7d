"""Seeded synthetic systems for the preconditioned-solve path.

LACE itself only reads Matrix Market files (control/magma_zmio.cpp:92-351);
these generators produce the synthetic workloads the solver is measured on,
as zero-based CSR (or row-major-block BCSR) with sorted columns and every
diagonal entry present - the layout LACE's reader produces
(control/magma_zmio.cpp:323-336).  Natural lexicographic ordering, Dirichlet
boundaries eliminated (boundary neighbours are simply not stored).

All generators are vectorised numpy; they allocate int32 indices and float64
values.
"""
from __future__ import annotations

from dataclasses import dataclass

import numpy as np


@dataclass
class CSR:
    """Zero-based CSR matrix, sorted columns (LACE's Magma_CSR)."""

    n: int
    row: np.ndarray  # int32 [n+1]
    col: np.ndarray  # int32 [nnz]
    val: np.ndarray  # float64 [nnz]
    m: int | None = None

    def __post_init__(self):
        if self.m is None:
            self.m = self.n

    @property
    def nnz(self) -> int:
        return int(self.col.shape[0])

    def rowidx(self) -> np.ndarray:
        """COO row ids (control/magma_zmconverter.cpp:145-167)."""
        return np.repeat(np.arange(self.n, dtype=np.int32), np.diff(self.row)).astype(np.int32)

    def to_dense(self) -> np.ndarray:
        d = np.zeros((self.n, self.m))
        d[self.rowidx(), self.col] = self.val
        return d

    def matvec(self, x: np.ndarray) -> np.ndarray:
        prod = self.val * x[self.col]
        return np.add.reduceat(prod, self.row[:-1]) if self.nnz else np.zeros(self.n)


@dataclass
class BCSR:
    """Zero-based block CSR with row-major bs x bs blocks (LACE's Magma_BCSR
    as produced by mkl_dcsrbsr with zero-based indexing,
    control/magma_zmconverter.cpp:640-668)."""

    nb: int
    bs: int
    row: np.ndarray  # int32 [nb+1]
    col: np.ndarray  # int32 [nblk]
    val: np.ndarray  # float64 [nblk, bs, bs]

    @property
    def nblk(self) -> int:
        return int(self.col.shape[0])

    @property
    def n(self) -> int:
        return self.nb * self.bs

    def rowidx(self) -> np.ndarray:
        return np.repeat(np.arange(self.nb, dtype=np.int32), np.diff(self.row)).astype(np.int32)

    def to_csr(self) -> CSR:
        """Scalar CSR with every block entry stored (mkl_dcsrbsr BSR->CSR)."""
        bs = self.bs
        rid = self.rowidx()
        # entry (blk p, r, c) -> scalar (rid[p]*bs + r, col[p]*bs + c)
        srow = (rid[:, None, None] * bs + np.arange(bs)[None, :, None]) * np.ones((1, 1, bs), dtype=np.int64)
        scol = (self.col[:, None, None] * bs + np.arange(bs)[None, None, :]) * np.ones((1, bs, 1), dtype=np.int64)
        srow = srow.ravel()
        scol = scol.ravel()
        sval = self.val.ravel()
        order = np.lexsort((scol, srow))
        counts = np.bincount(srow, minlength=self.n)
        row = np.zeros(self.n + 1, dtype=np.int32)
        np.cumsum(counts, out=row[1:])
        return CSR(self.n, row, scol[order].astype(np.int32), sval[order].astype(np.float64))


def _assemble(n: int, rows: list[np.ndarray], cols: list[np.ndarray], vals: list[np.ndarray]) -> CSR:
    r = np.concatenate(rows).astype(np.int64)
    c = np.concatenate(cols).astype(np.int64)
    v = np.concatenate(vals).astype(np.float64)
    order = np.lexsort((c, r))
    r, c, v = r[order], c[order], v[order]
    counts = np.bincount(r, minlength=n)
    row = np.zeros(n + 1, dtype=np.int32)
    np.cumsum(counts, out=row[1:])
    return CSR(n, row, c.astype(np.int32), v)


def _stencil(shape: tuple[int, ...], coeffs: dict[tuple[int, ...], float]) -> CSR:
    """Constant-coefficient stencil on a lexicographically ordered grid
    (first axis fastest), neighbours outside the grid dropped."""
    dims = len(shape)
    n = int(np.prod(shape))
    idx = np.arange(n, dtype=np.int64)
    coords = []
    rem = idx.copy()
    for d in range(dims):
        coords.append(rem % shape[d])
        rem //= shape[d]
    strides = [int(np.prod(shape[:d])) for d in range(dims)]
    rows, cols, vals = [], [], []
    for off, coef in coeffs.items():
        mask = np.ones(n, dtype=bool)
        delta = 0
        for d in range(dims):
            if off[d] != 0:
                nc = coords[d] + off[d]
                mask &= (nc >= 0) & (nc < shape[d])
                delta += off[d] * strides[d]
        sel = idx[mask]
        rows.append(sel)
        cols.append(sel + delta)
        vals.append(np.full(sel.shape[0], coef))
    return _assemble(n, rows, cols, vals)


def laplace2d(nx: int, ny: int | None = None) -> CSR:
    """2D 5-point Laplacian (4 on the diagonal, -1 off), Dirichlet boundary.
    64x64: n = 4096, nnz = 20,224."""
    ny = nx if ny is None else ny
    return _stencil((nx, ny), {(0, 0): 4.0, (-1, 0): -1.0, (1, 0): -1.0, (0, -1): -1.0, (0, 1): -1.0})


def aniso2d(s: int, eps: float) -> CSR:
    """2D 5-point anisotropic Laplacian -eps*u_xx - u_yy on an s x s grid.
    nnz = 5 s^2 - 4 s."""
    return _stencil((s, s), {(0, 0): 2.0 * (1.0 + eps), (-1, 0): -eps, (1, 0): -eps, (0, -1): -1.0, (0, 1): -1.0})


def convdiff3d(nx: int, ny: int | None = None, nz: int | None = None, pe: float = 10.0,
               velocity: tuple[float, float, float] = (1.0, 0.5, 0.25)) -> CSR:
    """3D 7-point first-order upwind convection-diffusion, D = 1, unit cube.

    Cell Peclet number: Pe = max_d |v_d| h / D = `pe`; per axis
    Pe_d = pe * v_d / max|v|.  Rows are scaled by h^2/D, so the stencil is
    diagonal 6 + sum_d Pe_d, upwind neighbours -1 - Pe_d, downwind -1
    (velocity components are positive).  128^3: n = 2,097,152,
    nnz = 14,581,760."""
    ny = nx if ny is None else ny
    nz = nx if nz is None else nz
    vmax = max(abs(v) for v in velocity)
    ped = [pe * v / vmax for v in velocity]
    coeffs = {(0, 0, 0): 6.0 + sum(abs(p) for p in ped)}
    for d in range(3):
        lo = [0, 0, 0]
        hi = [0, 0, 0]
        lo[d] = -1
        hi[d] = 1
        up, down = (-1.0 - abs(ped[d]), -1.0)
        if ped[d] >= 0:
            coeffs[tuple(lo)] = up
            coeffs[tuple(hi)] = down
        else:
            coeffs[tuple(lo)] = down
            coeffs[tuple(hi)] = up
    return _stencil((nx, ny, nz), coeffs)


def _primes(count: int) -> list[int]:
    out, c = [], 2
    while len(out) < count:
        if all(c % p for p in out if p * p <= c):
            out.append(c)
        c += 1
    return out


def trefethen(n: int = 19) -> CSR:
    """Trefethen matrix (SuiteSparse JGD_Trefethen/Trefethen_20b layout):
    diagonal = the primes 3, 5, 7, ...; a 1 wherever |i-j| is a power of 2."""
    pr = _primes(n + 1)[1:]
    rows, cols, vals = [np.arange(n)], [np.arange(n)], [np.array(pr, dtype=np.float64)]
    k = 1
    while k < n:
        i = np.arange(n - k)
        rows += [i + k, i]
        cols += [i, i + k]
        vals += [np.ones(n - k), np.ones(n - k)]
        k *= 2
    return _assemble(n, rows, cols, vals)


def bcsr3d(nx: int, ny: int | None = None, nz: int | None = None, bs: int = 5, seed: int = 0,
           dominance: float = 1.05) -> BCSR:
    """Block 7-point stencil over an nx*ny*nz cell grid with bs x bs blocks.

    Off-diagonal block entries ~ N(0,1)*0.1; diagonal blocks 5*I + N(0,1)*0.1.
    Then every scalar row is made strictly diagonally dominant: where
    |a_rr| < dominance * sum_{c != r} |a_rc|, a_rr is raised (keeping its
    sign) to that bound.  64^3 cells: 262,144 block rows, 1,810,432 blocks."""
    ny = nx if ny is None else ny
    nz = nx if nz is None else nz
    pattern = _stencil((nx, ny, nz), {(0, 0, 0): 1.0, (-1, 0, 0): 1.0, (1, 0, 0): 1.0,
                                      (0, -1, 0): 1.0, (0, 1, 0): 1.0, (0, 0, -1): 1.0, (0, 0, 1): 1.0})
    rng = np.random.default_rng(seed)
    nblk = pattern.nnz
    val = rng.standard_normal((nblk, bs, bs)) * 0.1
    rid = pattern.rowidx()
    isdiag = rid == pattern.col
    val[isdiag] += 5.0 * np.eye(bs)[None, :, :]
    absrow = np.zeros((pattern.n, bs))
    np.add.at(absrow, rid, np.abs(val).sum(axis=2))
    dvals = val[isdiag][:, np.arange(bs), np.arange(bs)]  # [nb, bs]
    off = absrow - np.abs(dvals)
    need = dominance * off
    newd = np.where(np.abs(dvals) < need, np.sign(dvals + (dvals == 0)) * need, dvals)
    dblocks = val[isdiag]
    dblocks[:, np.arange(bs), np.arange(bs)] = newd
    val[isdiag] = dblocks
    return BCSR(pattern.n, bs, pattern.row.copy(), pattern.col.copy(), val)


def rhs_normal(n: int, seed: int, nrhs: int = 1) -> np.ndarray:
    rng = np.random.default_rng(seed)
    if nrhs == 1:
        return rng.standard_normal(n)
    return rng.standard_normal((nrhs, n))


@dataclass
class BatchSystem:
    side: int
    eps: float
    A: CSR
    B: np.ndarray  # [nrhs, n]


def batch_aniso(count: int = 256, side_lo: int = 32, side_hi: int = 256, eps_lo: float = 1e-3,
                eps_hi: float = 1.0, nrhs: int = 4, seed: int = 0) -> list[BatchSystem]:
    """Independent 2D anisotropic Laplacians: side ~ U{side_lo..side_hi},
    eps log-uniform in [eps_lo, eps_hi], nrhs right-hand sides ~ N(0,1)."""
    rng = np.random.default_rng(seed)
    sides = rng.integers(side_lo, side_hi + 1, size=count)
    epss = np.exp(rng.uniform(np.log(eps_lo), np.log(eps_hi), size=count))
    out = []
    for s, e in zip(sides, epss):
        A = aniso2d(int(s), float(e))
        out.append(BatchSystem(int(s), float(e), A, rng.standard_normal((nrhs, A.n))))
    return out
