"""The host thread pool behind the drop-ins' bulk host loops
(lace_gb300/csrc/hostpar.h): tests/hostpool_check.cpp compiled with the host
compiler and run (regions on the parked threads, concurrent and nested
regions, a forked child)."""
import os
import shutil
import subprocess

import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(os.path.dirname(HERE), "lace_gb300", "csrc")


@pytest.mark.skipif(shutil.which("g++") is None, reason="no host C++ compiler")
def test_host_pool(tmp_path):
    exe = str(tmp_path / "hostpool_check")
    subprocess.run(["g++", "-O2", "-std=c++17", "-pthread", "-I", CSRC, os.path.join(HERE, "hostpool_check.cpp"),
                    "-o", exe], check=True)
    r = subprocess.run([exe], capture_output=True, text=True, timeout=120)
    assert r.returncode == 0 and r.stdout.strip() == "ok", (r.returncode, r.stdout, r.stderr)
