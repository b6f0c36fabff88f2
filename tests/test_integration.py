"""The reference's own `l2c` driver (src/bin/l2c.c), unmodified, compiles and
links against include/leg2cheb.h and libleg2cheb.so.  FFTW and CBLAS, which the
driver uses for its own test modes, come from the oracle's stand-in headers
when the real ones are absent.  Runs only where the reference tree exists
(L2C_REFERENCE, default /root/reference); CPU only: the Lambda self-test mode
(-d11) needs no GPU."""
import os
import subprocess

import pytest

from tests.conftest import PKG, REPO

REF = os.environ.get("L2C_REFERENCE", "/root/reference")
DRIVER = os.path.join(REF, "src", "bin", "l2c.c")


@pytest.fixture(scope="module")
def driver(lib, tmp_path_factory):
    if not os.path.exists(DRIVER):
        pytest.skip("reference tree not present")
    ob = subprocess.run(
        ["python3", "-c", "import glob,os,scipy; d=os.path.join(os.path.dirname(scipy.__file__),"
         "'..','scipy.libs'); g=sorted(glob.glob(os.path.join(d,'libscipy_openblas*.so'))); "
         "print(os.path.realpath(g[0]) if g else '')"], capture_output=True, text=True).stdout.strip()
    if not ob:
        pytest.skip("no OpenBLAS for the driver's own BLAS probe mode")
    out = str(tmp_path_factory.mktemp("l2c") / "l2c")
    libdir = os.path.join(PKG, "lib")
    shim = os.path.join(REPO, "oracle", "ref_shim")
    cmd = ["gcc", "-O1", "-w", "-fopenmp", "-DOMP", "-DTEST", "-I", shim,
           "-I", os.path.join(REPO, "include"), DRIVER, os.path.join(shim, "fftw_stub.c"),
           "-L", libdir, "-l:libleg2cheb.so", f"-Wl,-rpath,{libdir}",
           "-L", os.path.dirname(ob), f"-l:{os.path.basename(ob)}",
           f"-Wl,-rpath,{os.path.dirname(ob)}", "-lm", "-o", out]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stdout + r.stderr
    return out


def test_driver_links_against_library(driver):
    assert os.path.exists(driver)


def test_driver_lambda_mode(driver):
    # test_lambda (src/bin/l2c.c:694-711) asserts Lambda(0..2), Lambda(14.5) vs _LambdaE
    r = subprocess.run([driver, "-d11", "-v2"], capture_output=True, text=True, timeout=60)
    assert r.returncode == 0, r.stdout + r.stderr  # the driver's asserts passed
    assert "Lambda(24.5)       = 2.010024372031780915e-01" in r.stdout
