"""Generated constant tables (csrc/l2c_tables.h) equal the reference's."""
import os
import re
from fractions import Fraction

import numpy as np

from tests.conftest import PKG

HDR = os.path.join(PKG, "csrc", "l2c_tables.h")


def _init(name):
    src = open(HDR).read()
    m = re.search(name + r"_INIT \{ \\\n(.*?)\}", src, re.S)
    vals = m.group(1).replace("\\", "").split(",")
    return np.array([float.fromhex(v.strip()) for v in vals if v.strip()])


def test_lambda_int_table(golden):
    assert np.array_equal(_init("L2C_LAMBDA_INT"), golden["LambdaI"])


def test_binomial_tables(golden):
    assert np.array_equal(_init("L2C_BINOM_LOWER"), golden["BMe"])
    assert np.array_equal(_init("L2C_BINOM_UPPER"), golden["BMeT"])


def test_series_coefficients_exact():
    src = open(HDR).read()
    want = [Fraction(1), Fraction(-1, 64), Fraction(21, 8192), Fraction(-671, 524288),
            Fraction(180323, 134217728), Fraction(-20898423, 8589934592),
            Fraction(7426362705, 1099511627776)]
    for k, w in enumerate(want):
        m = re.search(rf"#define L2C_LAMBDA_C{k} (\S+)", src)
        assert Fraction(float.fromhex(m.group(1))) == w
