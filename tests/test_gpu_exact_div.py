"""div_rn_recip (Markstein's reciprocal-based division, used by the
Izhikevich neuron update and the STDP updater) equals CUDA's IEEE double
division bit for bit: exhaustively for the updater's (U - sw) / F over every
finite float sw, and on 2^32 random (numerator, denominator) pairs of the
neuron update's form plus raw doubles over the whole exponent range.  The
integer division by a constant (div_const_rn, used by the STDP updater) is
checked the same way: every finite float sw for (U - sw) / F, plus 2^30 raw
doubles."""
import ctypes
import os
import subprocess

import pytest

pytestmark = pytest.mark.gpu

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


@pytest.fixture(scope="module")
def lib(tmp_path_factory):
    out = str(tmp_path_factory.mktemp("divcheck") / "libdivcheck.so")
    nvcc = os.path.join(os.environ.get("CUDA_HOME", "/usr/local/cuda"), "bin", "nvcc")
    subprocess.run([nvcc, "-std=c++17", "-O3", "--fmad=false", "-shared", "-Xcompiler", "-fPIC",
                    "-gencode", "arch=compute_103a,code=sm_103a",
                    "-I", os.path.join(ROOT, "synaptogenesis_gb300", "csrc"),
                    os.path.join(ROOT, "tests", "gpu_checks", "division_check.cu"), "-o", out],
                   check=True)
    lib = ctypes.CDLL(out)
    lib.check_constant_divisor.argtypes = (ctypes.c_double, ctypes.c_int,
                                           ctypes.POINTER(ctypes.c_ulonglong))
    lib.check_random_pairs.argtypes = (ctypes.c_ulonglong, ctypes.c_ulonglong,
                                       ctypes.POINTER(ctypes.c_ulonglong))
    lib.check_integer_divisor.argtypes = (ctypes.c_double, ctypes.c_int, ctypes.c_ulonglong,
                                          ctypes.c_ulonglong, ctypes.POINTER(ctypes.c_ulonglong))
    return lib


@pytest.mark.parametrize("U,F", [(0.5, 1000), (0.2, 20)])
def test_constant_divisor_exhaustive(lib, U, F):
    out = (ctypes.c_ulonglong * 3)()
    assert lib.check_constant_divisor(U, F, out) == 0
    assert out[1] == (1 << 32) - (1 << 24)          # every finite float
    assert out[0] == 0, "first mismatch at float bits %#x" % out[2]


def test_random_pairs(lib):
    out = (ctypes.c_ulonglong * 3)()
    assert lib.check_random_pairs(1 << 32, 12345, out) == 0
    assert out[1] > 4_000_000_000
    assert out[0] == 0, "first mismatch at sample %d" % out[2]


@pytest.mark.parametrize("U,F", [(0.5, 1000), (0.2, 20), (0.5, 3)])
def test_integer_constant_divisor(lib, U, F):
    out = (ctypes.c_ulonglong * 3)()
    assert lib.check_integer_divisor(U, F, 1 << 30, 99, out) == 0
    assert out[1] > (1 << 32) - (1 << 24) + (1 << 29)
    assert out[0] == 0, "first mismatch at sample %#x" % out[2]
