"""Drop-in check: the reference's example programs compile unchanged against include/
and link with libcupss.so.

cuPSS user programs include the library either by a path relative to their own file
("../../inc/cupss.h", "../inc/cupss.h") or as <cupss.h> from an include directory, and
the reference builds every source as CUDA (CMakeLists.txt:22).  The test copies each
example into a scratch tree whose inc/ directories point at this repository's
include/, compiles it with nvcc for sm_103a and links it against libcupss.so.  The
programs are not run.

The examples directory of a cuPSS checkout is given by the environment variable
CUPSS_EXAMPLES_DIR; without it the test is skipped.
"""
import concurrent.futures as cf
import glob
import os
import shutil
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
EXAMPLES = os.environ.get("CUPSS_EXAMPLES_DIR", "")


def example_sources():
    if not EXAMPLES or not os.path.isdir(EXAMPLES):
        return []
    return sorted(glob.glob(os.path.join(EXAMPLES, "*", "*.cpp")) + glob.glob(os.path.join(EXAMPLES, "*", "*.cu")))


@pytest.mark.skipif(not example_sources(), reason="CUPSS_EXAMPLES_DIR does not name a cuPSS examples directory")
def test_reference_examples_compile_and_link(built_lib, tmp_path):
    from cupss_gb300 import build
    nvcc = build.nvcc_path()
    include = os.path.join(ROOT, "include")
    libdir = os.path.join(ROOT, "cupss_gb300")
    # scratch/inc and scratch/examples/inc stand where the examples' relative includes look
    os.symlink(include, tmp_path / "inc")
    (tmp_path / "examples").mkdir()
    os.symlink(include, tmp_path / "examples" / "inc")
    jobs = []
    for src in example_sources():
        d = tmp_path / "examples" / os.path.basename(os.path.dirname(src))
        d.mkdir(exist_ok=True)
        dst = d / os.path.basename(src)
        shutil.copyfile(src, dst)
        jobs.append(dst)

    def compile_link(src):
        obj = str(src) + ".o"
        exe = str(src) + ".bin"
        cc = [nvcc, "-std=c++17", "-x", "cu", *build.ARCH, "-I", include, "-c", str(src), "-o", obj]
        r = subprocess.run(cc, capture_output=True, text=True)
        if r.returncode != 0:
            return "%s: compile failed\n%s" % (src.name, r.stderr[-2000:])
        ld = [nvcc, *build.ARCH, obj, "-o", exe, "-L", libdir, "-lcupss", "-Xlinker", "-rpath=" + libdir]
        r = subprocess.run(ld, capture_output=True, text=True)
        if r.returncode != 0:
            return "%s: link failed\n%s" % (src.name, r.stderr[-2000:])
        return None

    with cf.ThreadPoolExecutor(min(8, len(jobs))) as ex:
        errors = [e for e in ex.map(compile_link, jobs) if e]
    assert not errors, "\n".join(errors)
    assert len(jobs) >= 10
