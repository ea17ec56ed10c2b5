"""The reference's own C and C++ integration programs (tests/c of dtFFT:
test_c2c_3d_c.c, test_r2r_3d_float_cxx.cpp, ...) compile unchanged against
this library's include/dtfft.h, with the reference's include/dtfft.hpp
unchanged, the single-process include/single_process_mpi/mpi.h and the C
implementation of their helper functions, and link against
libdtfft_gb300.so with every symbol resolved: C entry points and the C++
interface's out-of-line members alike.

The reference's sources exist only where it is checked out; these tests skip
elsewhere.  Running the programs needs a GPU: tests/test_ref_callers_gpu.py
builds and runs this repository's own C and C++ callers there.
"""
import glob
import os

import pytest

REF = "/root/reference"
HAVE_REF = os.path.isdir(os.path.join(REF, "tests", "c"))


@pytest.fixture(scope="module")
def lib_built():
    from dtfft_gb300 import build
    return build.build()


def _ref_programs():
    if not HAVE_REF:
        return []
    return sorted(glob.glob(os.path.join(REF, "tests", "c", "*.c")) +
                  glob.glob(os.path.join(REF, "tests", "c", "*.cpp")))


@pytest.mark.skipif(not HAVE_REF, reason="the reference's sources are not checked out here")
@pytest.mark.parametrize("src", _ref_programs(), ids=os.path.basename)
@pytest.mark.parametrize("hpp", ["reference_hpp", "own_hpp"])
def test_reference_program_compiles_and_links(lib_built, tmp_path, src, hpp):
    from tests.ref_callers import build_callers as bc
    out = str(tmp_path)
    ref_hpp_dir, ref_tests_c = bc.reference_program_dirs(REF, out)
    extra = (ref_hpp_dir, ref_tests_c) if hpp == "reference_hpp" else (ref_tests_c,)
    if hpp == "own_hpp" and src.endswith(".c"):
        pytest.skip("C program: no C++ header involved")
    rc, log, exe = bc.build_program([src], out, os.path.basename(src) + ".bin", extra)
    assert rc == 0, log
    assert os.path.exists(exe)


def test_reference_programs_are_all_found():
    if not HAVE_REF:
        pytest.skip("the reference's sources are not checked out here")
    names = {os.path.basename(p) for p in _ref_programs()}
    assert {"test_c2c_3d_c.c", "test_r2c_3d_c.c", "test_r2r_3d_float_cxx.cpp", "test_c2c_2d_cxx.cpp"} <= names
    assert len(names) == 12


@pytest.mark.parametrize("src", ["c_caller.c", "cxx_caller.cpp"])
def test_own_callers_compile_and_link(lib_built, tmp_path, src):
    from tests.ref_callers import build_callers as bc
    rc, log, exe = bc.build_program([os.path.join(bc.HERE, src)], str(tmp_path), src + ".bin")
    assert rc == 0, log


def test_single_process_mpi_dims_create(lib_built, tmp_path):
    """MPI_Dims_create of the stand-in follows MPI's balanced, non-increasing rule."""
    import subprocess
    from tests.ref_callers import build_callers as bc
    prog = r'''
#include <mpi.h>
#include <stdio.h>
int main(void) {
    int cases[][4] = {{8, 2, 0, 0}, {12, 3, 0, 0}, {1, 2, 0, 0}, {16, 2, 0, 0}, {6, 2, 3, 0}, {7, 2, 0, 0}};
    for (int i = 0; i < 6; ++i) {
        int d[3] = {cases[i][2], cases[i][3], 0};
        if (MPI_Dims_create(cases[i][0], cases[i][1], d) != MPI_SUCCESS) { printf("err\n"); continue; }
        for (int k = 0; k < cases[i][1]; ++k) printf("%d ", d[k]);
        printf("\n");
    }
    return 0;
}
'''
    src = tmp_path / "dims.c"
    src.write_text(prog)
    rc, log, obj = bc.compile_source(str(src), str(tmp_path))
    assert rc == 0, log
    exe = str(tmp_path / "dims")
    rc, log = bc.link([obj], exe)
    assert rc == 0, log
    lines = subprocess.run([exe], capture_output=True, text=True).stdout.split("\n")
    assert lines[:6] == ["4 2 ", "3 2 2 ", "1 1 ", "4 4 ", "3 2 ", "7 1 "]
