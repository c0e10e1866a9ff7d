"""CPU tests: the library's Matrix Market reader and writer against LACE's
own (control/magma_zmio.cpp), through the golden digests of LACE's outputs
on generated files (tests/mtx_cases.py, tests/golden/make_golden.py) and,
where the LACE tree is present, side by side."""
import os

import numpy as np
import pytest

import mtx_cases as MC
from lace_gb300 import dropin
from oracle import reference as ref

G = np.load(os.path.join(os.path.dirname(__file__), "golden", "lace_golden.npz"))
CASES = MC.cases()
DEV_ERR_NOT_FOUND = -105


def _file(tmp_path, name, text):
    fn = str(tmp_path / (name + ".mtx"))
    with open(fn, "w", newline="") as f:
        f.write(text)
    return fn


def _read_and_check(fn, name):
    rc, nr, nc, r, c, v = dropin.read_mtx(fn)
    assert rc == int(G[f"mtx_{name}_info"][0])
    if rc == 0:
        assert MC.digest_arrays(nr, nc, r, c, v) == str(G[f"mtx_{name}_read"][0])
    return rc, nr, nc, r, c, v


@pytest.mark.parametrize("name", sorted(CASES))
def test_read_equals_lace(tmp_path, name):
    """Entries, order and values bit for bit as LACE's read_z_csr_from_mtx
    (symmetric/hermitian expansion, skew-symmetric kept as is, blank lines,
    CRLF, two entries a line, duplicates, rejected banners)."""
    _read_and_check(_file(tmp_path, name, CASES[name]), name)


@pytest.mark.parametrize("name", sorted(set(CASES) - MC.REJECTED))
def test_coo_read_equals_lace(tmp_path, name):
    """read_z_coo_from_mtx: the entries in file order as LACE reads them
    (symmetric files: LACE returns freed arrays; here the expansion, which
    must equal the CSR reader's entries before the row fill)."""
    fn = _file(tmp_path, name, CASES[name])
    rc, nr, nc, r, c, v = dropin.read_mtx(fn, coo=True)
    assert rc == 0
    key = f"mtx_{name}_coo"
    if key in G.files:
        assert MC.digest_arrays(nr, nc, r, c, v) == str(G[key][0])
    # the CSR reader's arrays are these entries stably bucketed by row, each
    # row then sorted by column
    rc2, nr2, nc2, rp, ci, cv = dropin.read_mtx(fn)
    order = np.argsort(r, kind="stable")
    assert np.array_equal(np.diff(rp), np.bincount(r, minlength=nr))
    assert sorted(zip(r[order].tolist(), c[order].tolist())) == sorted(
        zip(np.repeat(np.arange(nr), np.diff(rp)).tolist(), ci.tolist()))


@pytest.mark.parametrize("name", sorted(set(CASES) - MC.REJECTED))
@pytest.mark.parametrize("major", [101, 102])
def test_write_equals_lace(tmp_path, name, major):
    """data_zwrite_csr_mtx writes LACE's bytes, row- and column-major."""
    key = f"mtx_{name}_write{major}"
    if key not in G.files:
        pytest.skip("LACE's own transpose rejects a non-square matrix (column-major output)")
    rc, nr, nc, r, c, v = _read_and_check(_file(tmp_path, name, CASES[name]), name)
    A = dropin.csr(r, c, v, nr)
    A.m.num_cols = nc
    out = str(tmp_path / "out.mtx")
    assert dropin.write_mtx(A, out, major) == 0
    assert MC.digest_file(out) == str(G[key][0])


@pytest.mark.parametrize("major", [101, 102])
def test_write_values_equal_lace(tmp_path, major):
    """%.16g of subnormals, -0, the largest double, long mantissas."""
    n, r, c, v = MC.write_values_matrix()
    out = str(tmp_path / "v.mtx")
    assert dropin.write_mtx(dropin.csr(r, c, v, n), out, major) == 0
    assert MC.digest_file(out) == str(G[f"mtx_values_write{major}"][0])


def test_large_file_parallel_paths(tmp_path):
    """~9 MB: the reader's line-aligned chunks and the writer's per-thread
    buffers, still LACE's arrays and bytes; then read back what was written."""
    fn = _file(tmp_path, "large", MC.large_text())
    rc, nr, nc, r, c, v = _read_and_check(fn, "large")
    rcc, cnr, cnc, cr, cc, cv = dropin.read_mtx(fn, coo=True)
    assert rcc == 0 and MC.digest_arrays(cnr, cnc, cr, cc, cv) == str(G["mtx_large_coo"][0])
    A = dropin.csr(r, c, v, nr)
    for major in (101, 102):
        out = str(tmp_path / ("w%d.mtx" % major))
        assert dropin.write_mtx(A, out, major) == 0
        assert MC.digest_file(out) == str(G[f"mtx_large_write{major}"][0])
    # LACE's %.16g keeps 16 significant digits (a double needs 17 to round-trip)
    rc2, nr2, nc2, r2, c2, v2 = dropin.read_mtx(str(tmp_path / "w101.mtx"))
    assert rc2 == 0 and np.array_equal(r2, r) and np.array_equal(c2, c)
    assert np.all(np.abs(v2 - v) <= 1e-15 * np.abs(v))


def test_missing_file():
    assert dropin.read_mtx("/nonexistent/dir/none.mtx")[0] == DEV_ERR_NOT_FOUND
    assert dropin.read_mtx("/nonexistent/dir/none.mtx", coo=True)[0] == DEV_ERR_NOT_FOUND


needs_ref = pytest.mark.skipif(not ref.available(), reason="LACE source tree not present")


@needs_ref
def test_live_lace_reader_on_random_files(tmp_path):
    """Fresh files, both readers side by side."""
    rng = np.random.default_rng(11)
    for k in range(3):
        n = int(rng.integers(50, 400))
        m = int(rng.integers(n, 8 * n))
        ents = sorted({(int(rng.integers(0, n)), int(rng.integers(0, n))) for _ in range(m)},
                      key=lambda e: rng.random())
        lines = ["%%MatrixMarket matrix coordinate real " + ("symmetric" if k == 1 else "general"),
                 "%d %d %d" % (n, n, len(ents))]
        lines += ["%d %d %.17g" % (max(i, j) + 1 if k == 1 else i + 1, min(i, j) + 1 if k == 1 else j + 1,
                                   rng.standard_normal() * 10.0 ** rng.integers(-30, 30)) for i, j in ents]
        fn = _file(tmp_path, "r%d" % k, "\n".join(lines) + "\n")
        ours = dropin.read_mtx(fn)
        theirs = ref.read_csr_mtx(fn)
        assert ours[0] == theirs[0] == 0
        for a, b in zip(ours[3:], theirs[3:]):
            assert np.array_equal(a, b)
        if k != 1:  # LACE's COO reader returns released arrays for symmetric files
            ours, theirs = dropin.read_mtx(fn, coo=True), ref.read_coo_mtx(fn)
            assert ours[0] == theirs[0] == 0 and ours[1:3] == theirs[1:3]
            for a, b in zip(ours[3:], theirs[3:]):
                assert np.array_equal(a, b)
