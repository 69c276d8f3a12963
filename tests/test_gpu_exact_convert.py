"""The integer float <-> double conversions and the float-by-double-constant
product (used by the Izhikevich neuron update and the STDP updater in place of
FP64-pipe conversions) equal the hardware's results bit for bit: exhaustively
over every float bit pattern for (double)f and for (float)((double)f * c) with
the updater's and the neuron update's constants (and the same product kept
in double), and on 2^32 doubles for
(float)d -- raw bit patterns, exact ties and their neighbours in the float
range, and the exponents at the edges of that range."""
import ctypes
import os
import subprocess

import pytest

pytestmark = pytest.mark.gpu

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


@pytest.fixture(scope="module")
def lib(tmp_path_factory):
    out = str(tmp_path_factory.mktemp("convcheck") / "libconvcheck.so")
    nvcc = os.path.join(os.environ.get("CUDA_HOME", "/usr/local/cuda"), "bin", "nvcc")
    subprocess.run([nvcc, "-std=c++17", "-O3", "--fmad=false", "-shared", "-Xcompiler", "-fPIC",
                    "-gencode", "arch=compute_103a,code=sm_103a",
                    "-I", os.path.join(ROOT, "synaptogenesis_gb300", "csrc"),
                    os.path.join(ROOT, "tests", "gpu_checks", "convert_check.cu"), "-o", out],
                   check=True)
    lib = ctypes.CDLL(out)
    lib.check_f2d_all.argtypes = (ctypes.POINTER(ctypes.c_ulonglong),)
    lib.check_mul_all.argtypes = (ctypes.c_double, ctypes.POINTER(ctypes.c_ulonglong))
    lib.check_muld_all.argtypes = (ctypes.c_double, ctypes.POINTER(ctypes.c_ulonglong))
    lib.check_d2f.argtypes = (ctypes.c_ulonglong, ctypes.c_ulonglong,
                              ctypes.POINTER(ctypes.c_ulonglong))
    return lib


def test_float_to_double_every_float(lib):
    out = (ctypes.c_ulonglong * 3)()
    assert lib.check_f2d_all(out) == 0
    assert out[1] == 1 << 32
    assert out[0] == 0, "first mismatch at float bits %#x" % out[2]


@pytest.mark.parametrize("c", [0.933, 0.04, 0.1, 1.0 / 3.0, 7.5e-300, 3.1e+290])
def test_float_times_double_constant_every_float(lib, c):
    out = (ctypes.c_ulonglong * 3)()
    assert lib.check_mul_all(c, out) == 0
    assert out[1] == 1 << 32
    assert out[0] == 0, "first mismatch at float bits %#x" % out[2]


def test_double_to_float(lib):
    out = (ctypes.c_ulonglong * 3)()
    assert lib.check_d2f(1 << 32, 2024, out) == 0
    assert out[1] == 1 << 32
    assert out[0] == 0, "first mismatch at sample %d" % out[2]


@pytest.mark.parametrize("c", [0.04, 0.1, 0.933, 1.0 / 3.0, 7.5e-300, 3.1e+290])
def test_float_times_double_constant_in_double_every_float(lib, c):
    out = (ctypes.c_ulonglong * 3)()
    assert lib.check_muld_all(c, out) == 0
    assert out[1] == 1 << 32
    assert out[0] == 0, "first mismatch at float bits %#x" % out[2]
