"""The float-float evaluations of the Izhikevich model's double expressions
(synaptogenesis_gb300/csrc/ff_exact.cuh) against the same expressions on the
GPU's FP64 pipe: bit for bit wherever the rounding test accepts, over every
float bit pattern for the STDP weight derivative without spike terms, the
presynaptic trace decay product, the float divisions by the integer
constants 60, 700 and 800 (reciprocal and one correction) and short-term w (both opcodes, with and without a source spike), on 2^32
random operand triples with spike terms, and on 2^32 random neuron substeps
(the voltage derivative, the implicit voltage update and the recovery time
constant of a threshold-crossing substep).  The test rejects non-finite
operands, results below 2^-101 and values within the error bound of a
rounding boundary; the rest must be a small fraction."""
import ctypes
import os
import subprocess

import pytest

pytestmark = pytest.mark.gpu

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


@pytest.fixture(scope="module")
def lib(tmp_path_factory):
    out = str(tmp_path_factory.mktemp("ffcheck") / "libffcheck_gpu.so")
    nvcc = os.path.join(os.environ.get("CUDA_HOME", "/usr/local/cuda"), "bin", "nvcc")
    subprocess.run([nvcc, "-std=c++17", "-O3", "--fmad=false", "-shared", "-Xcompiler", "-fPIC",
                    "-gencode", "arch=compute_103a,code=sm_103a",
                    "-I", os.path.join(ROOT, "synaptogenesis_gb300", "csrc"),
                    os.path.join(ROOT, "tests", "gpu_checks", "ff_check.cu"), "-o", out],
                   check=True)
    return ctypes.CDLL(out)


def _out():
    return (ctypes.c_ulonglong * 12)()


def _ok(out, max_fallback):
    assert out[0] == 0, "mismatch at %#x" % out[3]
    assert out[2] <= max_fallback * out[1], (out[2], out[1])


def test_weight_derivative_every_float(lib):
    out = _out()
    assert lib.check_wd_all(out) == 0
    assert out[1] == 1 << 32
    _ok(out, 0.12)        # non-finite and |x| >= 2^100 (11%), results below 2^-101


def test_trace_decay_product_every_float(lib):
    out = _out()
    assert lib.check_product_all(out) == 0
    assert out[1] == 1 << 32
    _ok(out, 0.16)        # non-finite and huge operands, results below 2^-126


@pytest.mark.parametrize("c", [0.95, 0.9])
def test_spnet_decay_products_every_float(lib, c):
    out = _out()
    assert lib.check_product_c_all(ctypes.c_double(c), out) == 0
    assert out[1] == 1 << 32
    _ok(out, 0.16)


@pytest.mark.parametrize("k", [0.01, 0.1])
def test_sum_with_double_constant_every_float(lib, k):
    out = _out()
    assert lib.check_add_const_all(ctypes.c_double(k), out) == 0
    assert out[1] == 1 << 32
    _ok(out, 0.16)


@pytest.mark.parametrize("divisor", [60, 700, 800])
def test_division_by_integer_every_float(lib, divisor):
    out = _out()
    assert lib.check_div_all(divisor, out) == 0
    assert out[1] == 1 << 32
    assert out[0] == 0, "mismatch at %#x" % out[3]


@pytest.mark.parametrize("sub", [0, 1])
@pytest.mark.parametrize("spike", [0, 1])
def test_short_term_w_every_float(lib, sub, spike):
    out = _out()
    assert lib.check_sw_all(sub, spike, out) == 0
    assert out[1] == 1 << 32
    _ok(out, 0.21)


def test_weight_derivative_random_spike_terms(lib):
    out = _out()
    assert lib.check_wd_random(ctypes.c_ulonglong(1 << 32), ctypes.c_ulonglong(3), out) == 0
    assert out[1] == 1 << 32
    _ok(out, 1e-3)


def test_izhikevich_substep_random(lib):
    out = _out()
    assert lib.check_iz_random(ctypes.c_ulonglong(1 << 32), ctypes.c_ulonglong(9), out) == 0
    assert out[1] == out[5] == out[9] == 1 << 32
    _ok(out[:4], 0.05)
    _ok(out[4:8], 1e-3)
    _ok(out[8:], 1e-3)
