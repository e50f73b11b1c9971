"""Double-float arithmetic of the q_l kernel, on the CPU.

The q_l kernel (compute_order_parameter.c:99-229) runs its Legendre and
angle-addition recurrences in double-float arithmetic (a float pair, about
48 significant bits; hsmc_gb300/csrc/df64.cuh).  The header compiles for the
host: these tests build it with g++ (no contraction) and check each
operation against double arithmetic, and q_l per particle from the same
recurrences in double and in double-float on random bond sets, against the
1e-12 per-particle tolerance the GPU test holds the kernel to against the
oracle.
"""
import ctypes
import os
import shutil
import subprocess

import numpy as np
import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(os.path.dirname(HERE), "hsmc_gb300", "csrc")


@pytest.fixture(scope="module")
def lib(tmp_path_factory):
    cxx = shutil.which("g++")
    if cxx is None:
        pytest.skip("no host C++ compiler")
    out = str(tmp_path_factory.mktemp("df64") / "libdf64check.so")
    subprocess.run([cxx, "-O2", "-std=c++17", "-ffp-contract=off", "-shared", "-fPIC", "-I" + CSRC, "-o", out,
                    os.path.join(HERE, "df64_ql_check.cpp")], check=True)
    lb = ctypes.CDLL(out)
    lb.ql_max_error.restype = ctypes.c_double
    lb.ql_max_error.argtypes = [ctypes.c_int, ctypes.c_long, ctypes.c_ulonglong]
    return lb


def test_operations_carry_about_48_bits(lib):
    out = np.zeros(2)
    lib.op_max_errors(ctypes.c_long(1_000_000), ctypes.c_ulonglong(5), out.ctypes.data_as(ctypes.POINTER(ctypes.c_double)))
    assert out[0] < 2.0**-46 and out[1] < 2.0**-46, out


@pytest.mark.parametrize("l", [4, 6])
def test_ql_recurrences_agree_with_double(lib, l):
    err = lib.ql_max_error(l, 100_000, 7 + l)
    assert err < 1e-13, err
