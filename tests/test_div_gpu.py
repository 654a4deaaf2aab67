"""The CH smoother's pair of divisions by det (CH/problem.f90:365-366,
:609-610) is evaluated as one correctly rounded reciprocal and two
Markstein-corrected quotients (cellops.cuh div2_rn).  Bit-identity with the
IEEE division `/` is checked here on the GPU over 2^30 seeded random operand
pairs (two quotients each) and over a table of edge cases; the FP64 parity
tests check the smoother itself against the oracle bit for bit."""
import ctypes
import os
import subprocess

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
SRC = os.path.join(ROOT, "tests", "cuda", "div_check.cu")
LIB = os.path.join(ROOT, "bsam1.2_gb300", "_build", "div_check.so")


def _lib():
    os.makedirs(os.path.dirname(LIB), exist_ok=True)
    if not os.path.exists(LIB) or os.path.getmtime(LIB) < max(
            os.path.getmtime(SRC), os.path.getmtime(os.path.join(ROOT, "bsam1.2_gb300", "csrc", "cellops.cuh"))):
        nvcc = os.path.join(os.environ.get("CUDA_HOME", "/usr/local/cuda"), "bin", "nvcc")
        subprocess.run([nvcc, "-gencode", "arch=compute_103a,code=sm_103a", "-O3", "-std=c++17", "-shared",
                        "-Xcompiler", "-fPIC", "-I", os.path.join(ROOT, "bsam1.2_gb300", "csrc"), SRC, "-o", LIB],
                       check=True)
    L = ctypes.CDLL(LIB)
    U, D = ctypes.POINTER(ctypes.c_ulonglong), ctypes.POINTER(ctypes.c_double)
    L.div_check_random.argtypes = [ctypes.c_ulonglong, ctypes.c_ulonglong, U, D]
    L.div_check_table.argtypes = [D, ctypes.c_int, D, ctypes.c_int, U, D]
    return L


def test_markstein_pair_equals_ieee_division_on_random_operands():
    L = _lib()
    bad, first = ctypes.c_ulonglong(), (ctypes.c_double * 3)()
    n = 1 << 30
    assert L.div_check_random(n, 20240503, ctypes.byref(bad), first) == 0
    assert bad.value == 0, (bad.value, list(first))


def test_markstein_pair_equals_ieee_division_on_edge_cases():
    L = _lib()
    ulp = np.spacing
    bs = [1.0, 1.0 + ulp(1.0), 2.0 - ulp(2.0), 2.0, 3.0, 1.5, 7.0, 10.0, 1e6, 2.0**399, 2.0**400 - ulp(2.0**400),
          2.0**400, 0.5, 1.0 - ulp(1.0) / 2, 1e-300, 5e-324, np.inf, np.nan, -1.0, 0.0]
    a_pos = [1.0, 1.0 - ulp(1.0) / 2, 1.0 + ulp(1.0), 3.0, 2.0**-400, 2.0**-400 - ulp(2.0**-400), 2.0**400,
             2.0**401 - ulp(2.0**401), 2.0**401, 0.1, 1 / 3, 2.0**-1074, 2.0**-1022, 1.7976931348623157e308, 0.0,
             np.inf, np.nan, 12345.678, 2.0**52 + 1, 2.0**53 - 1]
    a = np.array(a_pos + [-x for x in a_pos], dtype=np.float64)
    b = np.array(bs, dtype=np.float64)
    bad, first = ctypes.c_ulonglong(), (ctypes.c_double * 3)()
    D = ctypes.POINTER(ctypes.c_double)
    assert L.div_check_table(a.ctypes.data_as(D), len(a), b.ctypes.data_as(D), len(b), ctypes.byref(bad),
                             first) == 0
    # NaN quotients compare by bits, and a NaN's payload may differ between
    # the two forms only when an operand is NaN or Inf, which takes `/`
    assert bad.value == 0, (bad.value, list(first))
