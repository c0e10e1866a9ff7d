"""Inputs for the setup-conversion parity tests (data_zmconvert,
data_zmtranspose, data_rowindex), generated from seeds, and a snapshot of a
data_d_matrix (its fields and the arrays they describe) to compare LACE's
output with the library's."""
from __future__ import annotations

import ctypes as C
import functools
import hashlib

import numpy as np

# storage and diagonal codes (include/sparse_types.h)
CSR, BCSR, CSC, COO = 611, 615, 616, 618
CSRL, CSRU, CSRCOO, CUCSR = 627, 628, 629, 630
CSCL, CSCU, CSCCOO = 634, 635, 636
BCSRL, BCSRU, BCSCU = 641, 642, 646
UNITY, VALUE, ZERO, NODIAG = 593, 594, 595, 596

CSR_TARGETS = [CSR, CUCSR, CSRL, CSRU, COO, CSRCOO, CSC, CSCL, CSCU, CSCCOO]
DIAGS = [0, UNITY, VALUE, ZERO, NODIAG]


def random_csr(n, m, per_row, seed, diag=True, empty_rows=False):
    """Sorted CSR rows with random columns (the diagonal in every row when
    `diag`), values from a seeded normal."""
    rng = np.random.default_rng(seed)
    row, col = [0], []
    for i in range(n):
        k = 0 if (empty_rows and i % 7 == 3) else int(rng.integers(1, per_row + 1))
        cols = set(int(c) for c in rng.integers(0, m, k))
        if diag and i < m and not (empty_rows and i % 7 == 3):
            cols.add(i)
        col += sorted(cols)
        row.append(len(col))
    # dyadic values: the same bits on every platform
    val = rng.integers(-2 ** 20, 2 ** 20, len(col)) / 1024.0
    return np.array(row, np.int32), np.array(col, np.int32), val


@functools.lru_cache(maxsize=None)
def matrices():
    """name -> (n_rows, n_cols, row, col, val)"""
    out = {}
    for name, (n, m, k, seed, diag, empty) in {
        "square": (300, 300, 9, 1, True, False),
        "no_diagonal": (120, 120, 6, 2, False, False),
        "empty_rows": (150, 150, 5, 3, True, True),
        "tall": (80, 60, 7, 4, True, False),
        "large": (40000, 40000, 12, 5, True, False),
    }.items():
        r, c, v = random_csr(n, m, k, seed, diag, empty)
        out[name] = (n, m, r, c, v)
    return out


def block_matrix(nb=60, bs=3, seed=6):
    """A BCSR pattern with a diagonal block in every block row: (block rows,
    bs, row, col, val (numblocks * bs * bs, row-major blocks))."""
    r, c, _ = random_csr(nb, nb, 5, seed, True, False)
    rng = np.random.default_rng(seed + 100)
    return nb, bs, r, c, rng.integers(-2 ** 20, 2 ** 20, len(c) * bs * bs) / 1024.0


def jobs():
    """(key, input, old, new, diagorder, blocksize) for every conversion
    checked; input names a matrix of matrices(), "blocks" the block matrix,
    "onebased:<name>" that matrix with one-based indices; new None is a
    transpose."""
    out = []
    for name in matrices():
        for new in CSR_TARGETS:
            for d in (DIAGS if new in (CSRL, CSRU, CSCL, CSCU) else [0]):
                out.append((f"conv_{name}_{new}_{d}", name, CSR, new, d, 0))
        out.append((f"conv_{name}_t", name, CSR, None, 0, 0))
    for bs in (2, 3, 4):
        out.append((f"conv_square_bcsr{bs}", "square", CSR, BCSR, 0, bs))
    out.append(("conv_tall_bcsr3", "tall", CSR, BCSR, 0, 3))
    for new in (BCSRL, BCSRU, BCSCU):
        for d in DIAGS:
            out.append((f"conv_blocks_{new}_{d}", "blocks", BCSR, new, d, 0))
    out.append(("conv_blocks_t", "blocks", BCSR, None, 0, 0))
    out.append(("conv_onebased_square_t", "onebased:square", CSR, None, 0, 0))
    for name in ("square", "empty_rows", "large"):
        out.append((f"conv_coo_{name}", "coo:" + name, COO, CSR, 0, 0))
    # LACE's CSRL with the default diagonal order, transposed again
    out.append(("conv_square_csrl0_t", "csrl0:square", CSRL, None, 0, 0))
    return out


@functools.lru_cache(maxsize=None)
def job_input(spec):
    """(storage, n_rows, n_cols, row, col, val, blocksize) of a job's input"""
    if spec == "blocks":
        nb, bs, r, c, v = block_matrix()
        return BCSR, nb, nb, r, c, v, bs
    if spec.startswith("onebased:"):
        n, m, r, c, v = matrices()[spec.split(":")[1]]
        return CSR, n, m, r + 1, c + 1, v, 0
    if spec.startswith("coo:"):
        # the entries in a shuffled order, a tenth of them repeated (equal
        # columns in a row: the sort's own order decides between them)
        n, m, r, c, v = matrices()[spec.split(":")[1]]
        rows = np.repeat(np.arange(n, dtype=np.int32), np.diff(r))
        rng = np.random.default_rng(n)
        dup = rng.choice(len(c), len(c) // 10, replace=False)
        rows = np.concatenate([rows, rows[dup]])
        cols = np.concatenate([c, c[dup]])
        vals = np.concatenate([v, v[dup] + 0.5])
        order = rng.permutation(len(cols))
        return COO, n, m, rows[order], cols[order], vals[order], 0
    if spec.startswith("csrl0:"):
        # rows with their diagonal dropped and nnz counting it (LACE's CSRL
        # under diagorder 0): the tail holds zero entries in column 0
        n, m, r, c, v = matrices()[spec.split(":")[1]]
        keep = [[k for k in range(r[i], r[i + 1]) if c[k] < i] for i in range(n)]
        rr = np.cumsum([0] + [len(x) for x in keep]).astype(np.int32)
        cc = np.array([c[k] for x in keep for k in x], np.int32)
        vv = np.array([v[k] for x in keep for k in x])
        ndiag = sum(1 for i in range(n) for k in range(r[i], r[i + 1]) if c[k] == i)
        return CSRL, n, m, rr, np.concatenate([cc, np.zeros(ndiag, np.int32)]), \
            np.concatenate([vv, np.zeros(ndiag)]), 0
    n, m, r, c, v = matrices()[spec]
    return CSR, n, m, r, c, v, 0


FIELDS = ("storage_type", "fill_mode", "num_rows", "num_cols", "nnz", "true_nnz", "max_nnz_row", "diameter",
          "blocksize", "ldblock", "numblocks", "major", "pad_rows", "pad_cols")


def snapshot(m, nptr: int) -> dict:
    """A data_d_matrix's fields and arrays: `nptr` row entries (the row
    index array's length for COO), the index and value arrays by nnz (by
    numblocks for a block matrix), rowidx when present."""
    f = {k: int(getattr(m, k)) for k in FIELDS}
    blocks = f["blocksize"] > 0 and f["numblocks"] > 0
    nidx = f["numblocks"] if blocks else f["nnz"]
    nval = f["nnz"]

    def arr(p, n, t):
        if not p or n <= 0:
            return np.zeros(0, t)
        return np.ctypeslib.as_array(C.cast(p, C.POINTER(C.c_int if t == np.int32 else C.c_double)), (n,)).copy()

    return dict(fields=f, row=arr(m.row, nptr, np.int32), col=arr(m.col, nidx, np.int32),
                val=arr(m.val, nval, np.float64),
                rowidx=arr(m.rowidx, f["nnz"], np.int32) if m.rowidx else np.zeros(0, np.int32))


def nptr_of(m) -> int:
    """row entries LACE's conversion allocates: rows + 1, or nnz for COO"""
    if int(m.storage_type) == COO:
        return int(m.nnz)
    return max(int(m.num_rows), int(m.num_cols)) + 1 if int(m.storage_type) in (CSC, CSCL, CSCU, CSCCOO) \
        else int(m.num_rows) + 1


def digest(s: dict) -> str:
    h = hashlib.sha256()
    h.update(repr(sorted(s["fields"].items())).encode())
    for k in ("row", "col", "val", "rowidx"):
        h.update(np.ascontiguousarray(s[k]).tobytes())
    return h.hexdigest()
