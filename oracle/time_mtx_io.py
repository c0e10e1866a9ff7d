"""Times LACE's own Matrix Market reader and writer (oracle/_ref, built from
the LACE tree) against the library's on a generated convection-diffusion
system; test infrastructure, run where the LACE tree is present:

    python oracle/time_mtx_io.py [grid side, default 64]
"""
from __future__ import annotations

import os
import sys
import tempfile
import time

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(HERE))
sys.path.insert(0, os.path.join(os.path.dirname(HERE), "tests", "golden"))

import numpy as np  # noqa: E402

from lace_gb300 import dropin, problems as P  # noqa: E402
from oracle import reference as ref  # noqa: E402
from make_golden import CaptureStdout  # noqa: E402


def main():
    side = int(sys.argv[1]) if len(sys.argv) > 1 else 64
    A = P.convdiff3d(side)
    tmp = tempfile.mkdtemp()
    f_ours, f_lace = os.path.join(tmp, "ours.mtx"), os.path.join(tmp, "lace.mtx")
    Am = dropin.csr(A.row, A.col, A.val, A.n)
    t0 = time.perf_counter()
    assert dropin.write_mtx(Am, f_ours) == 0
    t_write = time.perf_counter() - t0
    Rm = ref.Mat.from_arrays(ref.Magma_CSR, A.n, A.n, A.row, A.col, A.val)
    t0 = time.perf_counter()
    with CaptureStdout():
        ref.write_csr_mtx(Rm, f_lace)
    t_write_lace = time.perf_counter() - t0
    same_bytes = open(f_ours, "rb").read() == open(f_lace, "rb").read()
    t0 = time.perf_counter()
    ours = dropin.read_mtx(f_ours)
    t_read = time.perf_counter() - t0
    t0 = time.perf_counter()
    with CaptureStdout():
        lace = ref.read_csr_mtx(f_ours)
    t_read_lace = time.perf_counter() - t0
    same_arrays = all(np.array_equal(a, b) for a, b in zip(ours[3:], lace[3:]))
    mb = os.path.getsize(f_ours) / 1e6
    print(f"{side}^3: n={A.n} nnz={A.nnz} file {mb:.1f} MB, {os.cpu_count()} host threads")
    print(f"  write: library {t_write:.3f} s, LACE {t_write_lace:.3f} s ({t_write_lace / t_write:.1f}x), "
          f"identical bytes: {same_bytes}")
    print(f"  read:  library {t_read:.3f} s, LACE {t_read_lace:.3f} s ({t_read_lace / t_read:.1f}x), "
          f"identical arrays: {same_arrays}")


if __name__ == "__main__":
    main()
