"""The reference's own front ends, unmodified, against this library.

* src/bin/l2c.c, the reference's test and benchmark driver, compiled against
  include/leg2cheb.h and linked with libleg2cheb.so (`make -C oracle drop-in`;
  FFTW and CBLAS, which the driver uses in its own non-transform modes, come
  from the oracle's stand-in headers).  On the CPU machine: the Lambda
  self-test mode (-d11).  On a GPU: its transform modes, each with the
  driver's own asserts (built with -DTEST): -d2 round trip
  (src/bin/l2c.c:10-66), -d0 / -d1 speed runs (:181-212), -d3 direct round
  trip, -d4 2D against 1D lines, -d5 2D round trip, -d8 known answers.
* src/ctypes/l2ctypes.py, the reference's ctypes wrapper: its own round trip
  (:114-125), with its loader (find_library("leg2cheb")) pointed at this
  library through LD_LIBRARY_PATH.

The reference files come from L2C_REFERENCE (a reference tree) if set, else
from the copy `make -C oracle stage` keeps under oracle/_ref/src (git-ignored;
build() makes it wherever the reference tree is present, and it travels with
the working tree to machines without one).  Without either the tests skip."""
import os
import subprocess
import sys

import pytest

from tests.conftest import PKG, REPO

REF = os.environ.get("L2C_REFERENCE") or os.path.join(REPO, "oracle", "_ref", "src")
DRIVER_SRC = os.path.join(REF, "src", "bin", "l2c.c")
CTYPES_SRC = os.path.join(REF, "src", "ctypes", "l2ctypes.py")
LIBDIR = os.path.join(PKG, "lib")


@pytest.fixture(scope="module")
def driver(lib):
    if not os.path.exists(DRIVER_SRC):
        pytest.skip("reference sources not present")
    r = subprocess.run(["make", "-s", "-C", os.path.join(REPO, "oracle"), "drop-in",
                        f"REF={REF}", f"LIBDIR={LIBDIR}"], capture_output=True, text=True)
    if "no OpenBLAS" in r.stdout + r.stderr:
        pytest.skip("no OpenBLAS for the driver's own BLAS modes")
    assert r.returncode == 0, r.stdout + r.stderr
    return os.path.join(REPO, "oracle", "_ref", "l2c_drop_in")


def run_driver(driver, *args, timeout=300):
    r = subprocess.run([driver, *args], capture_output=True, text=True, timeout=timeout)
    assert r.returncode == 0, (args, r.stdout[-2000:], r.stderr[-2000:])  # its asserts held
    return r.stdout


def test_driver_links_against_library(driver):
    assert os.path.exists(driver)


def test_driver_lambda_mode(driver):
    # test_lambda (src/bin/l2c.c:694-711) asserts Lambda(0..2), Lambda(14.5) vs _LambdaE
    out = run_driver(driver, "-d11", "-v2", timeout=60)
    assert "Lambda(24.5)       = 2.010024372031780915e-01" in out


def _field(out, key):
    for line in out.splitlines():
        if key in line:
            return float(line.split("=")[1].split()[0])
    raise AssertionError(f"{key!r} not in driver output:\n{out}")


@pytest.mark.gpu
@pytest.mark.parametrize("args", [("-N512", "-d2"), ("-N512", "-d2", "-s64"),
                                  ("-N1000", "-d2", "-R1", "-s36"),
                                  ("-N100000", "-d2", "-s64", "-m1")])
def test_driver_round_trip(driver, args):
    out = run_driver(driver, *args, "-v1")
    # the driver asserts error < 1e-10; the relative round trip is far below
    assert _field(out, "L inf Error") < 1e-12, out


@pytest.mark.gpu
@pytest.mark.parametrize("d", ["0", "1"])
def test_driver_speed_mode(lib, driver, d):
    out = run_driver(driver, "-N1000000", f"-d{d}", "-s64", "-r5", "-v0")
    line = [ln for ln in out.splitlines() if ln.startswith("Timing N")][0]
    flops = int(line.rsplit("=", 1)[1])
    assert flops == lib.Plan(1000000, 64).flops(int(d))  # the reference's flop count
    assert float(line.split("=")[1].split("/")[1].split()[0]) > 0.0


@pytest.mark.gpu
@pytest.mark.parametrize("args", [("-N100", "-d3"), ("-N512", "-d4", "-s32"),
                                  ("-N256", "-d5", "-s32"), ("-N512", "-d8", "-s64")])
def test_driver_other_modes(driver, args):
    run_driver(driver, *args, "-v1")


@pytest.mark.gpu
def test_reference_ctypes_wrapper_round_trip(lib):
    if not os.path.exists(CTYPES_SRC):
        pytest.skip("reference sources not present")
    env = dict(os.environ)
    env["LD_LIBRARY_PATH"] = LIBDIR + os.pathsep + env.get("LD_LIBRARY_PATH", "")
    probe = subprocess.run([sys.executable, "-c",
                            "from ctypes.util import find_library; print(find_library('leg2cheb'))"],
                           capture_output=True, text=True, env=env)
    if probe.stdout.strip() != "libleg2cheb.so":
        pytest.skip(f"find_library cannot see the library here: {probe.stdout!r}")
    r = subprocess.run([sys.executable, CTYPES_SRC], capture_output=True, text=True, env=env,
                       timeout=300)
    assert r.returncode == 0, r.stdout + r.stderr  # its assert error < 1e-8 held
    err = float(r.stdout.split(":")[-1])
    assert err < 1e-12, r.stdout
