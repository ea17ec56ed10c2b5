"""C and C++ programs that use dtFFT as its own integration programs do
(tests/ref_callers/c_caller.c through dtfft.h, cxx_caller.cpp through
dtfft.hpp), built with gcc / g++ against include/, the single-process mpi.h
and libdtfft_gb300.so, and run on the GPU: every plan's round trip passes the
reference's threshold 5 log2(N) eps (tests/test_utils.F90:89-109) and the
transposes of a virtual grid return their input bit for bit."""
import os
import subprocess

import pytest

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("src,plans", [("c_caller.c", 4), ("cxx_caller.cpp", 3)])
def test_caller_program_runs(dt, cuda, tmp_path, src, plans):
    from tests.ref_callers import build_callers as bc
    rc, log, exe = bc.build_program([os.path.join(bc.HERE, src)], str(tmp_path), src + ".bin")
    assert rc == 0, log
    r = subprocess.run([exe], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stdout + r.stderr
    assert r.stdout.count("Test PASSED!") == plans, r.stdout
