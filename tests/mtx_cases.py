"""Matrix Market files for the reader/writer parity tests, generated from
seeds (no files are stored): every kind of coordinate file LACE's reader
accepts, layouts fscanf tolerates, and a few it rejects."""
from __future__ import annotations

import numpy as np

# values with every printf %.16g shape: exponents, subnormals, integers,
# negative zero, long mantissas
TRICKY = [1.5, -2.25e-3, 3e10, 0.1, 123456789.12345679, 7.0, -0.0, 1e-310, 1.7976931348623157e308,
          2.2250738585072014e-308, 1 / 3, -1e-5, 0.1 + 0.2, 1e16, 123456789012345678.0, 5e-324]


def _fmt(v: float, rng) -> str:
    """a value as a file might hold it (several spellings)"""
    k = int(rng.integers(0, 4))
    if k == 0:
        return repr(float(v))
    if k == 1:
        return "%.17g" % v
    if k == 2:
        return "%.6e" % v
    return "%.10G" % v


def _entries(rng, m, n, count, lower=False):
    out = set()
    while len(out) < count:
        i, j = int(rng.integers(0, m)), int(rng.integers(0, n))
        if lower and j > i:
            i, j = j, i
        out.add((i, j))
    out = list(out)
    rng.shuffle(out)
    return out


def cases() -> dict[str, str]:
    rng = np.random.default_rng(2024)
    c = {}

    def coord(banner, m, n, ents, fields, sep="\n", comments=(), per_line=1, blank_every=0):
        lines = [banner] + ["%" + t for t in comments] + ["%d %d %d" % (m, n, len(ents))]
        body = []
        for k, (i, j) in enumerate(ents):
            vals = []
            if fields >= 3:
                vals.append(_fmt(TRICKY[k % len(TRICKY)] * (1 + k) if k % 3 else float(rng.standard_normal()),
                                 rng))
            if fields == 4:
                vals.append(_fmt(float(rng.standard_normal()), rng))
            body.append(" ".join([str(i + 1), str(j + 1)] + vals))
        rows = []
        for k in range(0, len(body), per_line):
            rows.append("   ".join(body[k:k + per_line]))
            if blank_every and k % blank_every == 0:
                rows.append("")
        return sep.join(lines + rows) + sep

    c["general_real"] = coord("%%MatrixMarket matrix coordinate real general", 30, 30,
                              _entries(rng, 30, 30, 160), 3)
    c["symmetric_real"] = coord("%%MatrixMarket matrix coordinate real symmetric", 25, 25,
                                _entries(rng, 25, 25, 90, lower=True) + [(k, k) for k in (3, 7)], 3)
    c["pattern_general"] = coord("%%MatrixMarket matrix coordinate pattern general", 20, 20,
                                 _entries(rng, 20, 20, 70), 2)
    c["pattern_symmetric"] = coord("%%MatrixMarket matrix coordinate pattern symmetric", 20, 20,
                                   _entries(rng, 20, 20, 50, lower=True), 2)
    c["integer_general"] = coord("%%MatrixMarket matrix coordinate integer general", 15, 15,
                                 _entries(rng, 15, 15, 40), 2)
    # integer values: append an integer field per entry line
    lines = c["integer_general"].splitlines()
    c["integer_general"] = "\n".join(lines[:2] + [ln + " " + str(int(rng.integers(-99, 99))) for ln in lines[2:]]) + "\n"
    c["complex_general"] = coord("%%MatrixMarket matrix coordinate complex general", 18, 18,
                                 _entries(rng, 18, 18, 60), 4)
    c["complex_hermitian"] = coord("%%MatrixMarket matrix coordinate complex hermitian", 18, 18,
                                   _entries(rng, 18, 18, 45, lower=True), 4)
    c["skew_symmetric"] = coord("%%MatrixMarket matrix coordinate real skew-symmetric", 16, 16,
                                [e for e in _entries(rng, 16, 16, 40, lower=True) if e[0] != e[1]], 3)
    c["comments_blank_lines"] = coord("%%MatrixMarket matrix coordinate real general", 22, 22,
                                      _entries(rng, 22, 22, 80), 3, comments=("a comment", "", "another one"),
                                      blank_every=7)
    c["two_entries_per_line"] = coord("%%MatrixMarket matrix coordinate real general", 24, 24,
                                      _entries(rng, 24, 24, 75), 3, per_line=2)
    c["crlf"] = coord("%%MatrixMarket matrix coordinate real general", 12, 12, _entries(rng, 12, 12, 30), 3,
                      sep="\r\n")
    c["rectangular"] = coord("%%MatrixMarket matrix coordinate real general", 20, 35,
                             _entries(rng, 20, 35, 90), 3)
    c["upper_case_banner"] = coord("%%MatrixMarket MATRIX Coordinate REAL General", 10, 10,
                                   _entries(rng, 10, 10, 25), 3)
    dup = _entries(rng, 14, 14, 40)
    dup = dup + dup[:12] + dup[3:9]  # repeated (row, column) pairs: kept, as LACE keeps them
    c["duplicates"] = coord("%%MatrixMarket matrix coordinate real general", 14, 14, dup, 3)
    # a larger one: the parallel path (several line-aligned chunks)
    big = [(i, j) for i in range(3000) for j in (i - 40, i - 1, i, i + 1, i + 40) if 0 <= j < 3000]
    rng.shuffle(big)
    c["large_general"] = coord("%%MatrixMarket matrix coordinate real general", 3000, 3000, big, 3)
    # rejected by LACE's reader
    c["array_format"] = "%%MatrixMarket matrix array real general\n3 3\n1\n2\n3\n4\n5\n6\n7\n8\n9\n"
    c["bad_banner"] = "%%NotMatrixMarket matrix coordinate real general\n2 2 1\n1 1 1.0\n"
    return c


REJECTED = {"array_format", "bad_banner"}


def write_values_matrix():
    """A CSR matrix whose values exercise every %.16g shape (writer tests)."""
    n = 12
    row = [0]
    col, val = [], []
    k = 0
    for i in range(n):
        for j in sorted({i, (i * 5 + 3) % n, (i * 7 + 1) % n}):
            col.append(j)
            val.append(TRICKY[k % len(TRICKY)] * (-1) ** k)
            k += 1
        row.append(len(col))
    return n, np.array(row, np.int32), np.array(col, np.int32), np.array(val, np.float64)


def large_text() -> str:
    """A 256 x 256 five-point operator in shuffled entry order (~9 MB): enough
    lines for the reader's and the writer's parallel paths."""
    rng = np.random.default_rng(7)
    s = 256
    n = s * s
    ents = []
    for i in range(n):
        x, y = i % s, i // s
        for j, ok in ((i - s, y > 0), (i - 1, x > 0), (i, True), (i + 1, x < s - 1), (i + s, y < s - 1)):
            if ok:
                ents.append((i, j))
    order = rng.permutation(len(ents))
    # exact power-of-two scales: the file text must not depend on the
    # platform's exp (numpy's differs in the last bit between x86 and Arm)
    vals = np.ldexp(rng.standard_normal(len(ents)), rng.integers(-30, 30, len(ents)))
    lines = ["%%MatrixMarket matrix coordinate real general", "%d %d %d" % (n, n, len(ents))]
    lines += ["%d %d %r" % (ents[k][0] + 1, ents[k][1] + 1, float(vals[k])) for k in order]
    return "\n".join(lines) + "\n"


def digest_arrays(nr, nc, row, col, val) -> str:
    import hashlib
    h = hashlib.sha256()
    h.update(np.array([nr, nc], np.int64).tobytes())
    for a in (row, col, val):
        h.update(np.ascontiguousarray(a).tobytes())
    return h.hexdigest()


def digest_file(path: str) -> str:
    import hashlib
    return hashlib.sha256(open(path, "rb").read()).hexdigest()
