"""Times LACE's own setup conversions (oracle/_ref, built from the LACE tree)
against the library's on a generated convection-diffusion system: the L/U
split the factorisation starts from (CSR -> CSRL with a unit diagonal,
CSR -> CSCU) and the transpose; test infrastructure, run where the LACE tree
is present:

    python oracle/time_convert.py [grid side, default 96]
"""
from __future__ import annotations

import ctypes as C
import os
import sys
import time

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(HERE))

import numpy as np  # noqa: E402

import lace_gb300 as lg  # noqa: E402
from lace_gb300 import dropin, problems as P  # noqa: E402
from oracle import reference as ref  # noqa: E402

CSR, CSRL, CSCU, UNITY = 611, 627, 635, 593


def main():
    side = int(sys.argv[1]) if len(sys.argv) > 1 else 96
    A = P.convdiff3d(side)
    Am = dropin.csr(A.row, A.col, A.val, A.n)
    Ar = ref.Mat.from_arrays(CSR, A.n, A.n, A.row, A.col, A.val)
    libc = C.CDLL(None)
    libc.free.argtypes = [C.c_void_p]
    print("%d rows, %d entries, %d host threads" % (A.n, len(A.col), os.cpu_count()))
    for name, new, d in (("CSR -> CSRL (unit)", CSRL, UNITY), ("CSR -> CSCU", CSCU, 0), ("transpose", None, 0)):
        t_ours, t_lace = [], []
        for _ in range(3):
            B = lg.DataMatrix()
            B.diagorder_type = d
            t0 = time.perf_counter()
            if new is None:
                rc = lg.lib().data_zmtranspose(Am.m, C.byref(B))
            else:
                rc = lg.lib().data_zmconvert(Am.m, C.byref(B), CSR, new)
            t_ours.append(time.perf_counter() - t0)
            assert rc == 0
            for f in ("val", "row", "col"):
                libc.free(getattr(B, f))
            t0 = time.perf_counter()
            R = ref.transpose(Ar) if new is None else ref.convert(Ar, CSR, new, d)
            t_lace.append(time.perf_counter() - t0)
            R.free()
        print("%-20s library %7.1f ms   LACE %7.1f ms" % (name, 1e3 * min(t_ours), 1e3 * min(t_lace)))


if __name__ == "__main__":
    main()
