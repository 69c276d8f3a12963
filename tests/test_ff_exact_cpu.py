"""Host checks of the float-float evaluations of the Izhikevich model's
double expressions (synaptogenesis_gb300/csrc/ff_exact.cuh): wherever the
rounding test accepts, the float result equals the reference's double
expression evaluated by the host compiler, bit for bit.  The STDP updater's
expressions strided over the float bit patterns here (every one of them on
the GPU) and random with spike terms; the neuron substep's two expressions
on random operands."""
import ctypes
import os
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


class Result(ctypes.Structure):
    _fields_ = [("mismatches", ctypes.c_ulonglong), ("checked", ctypes.c_ulonglong),
                ("fallbacks", ctypes.c_ulonglong), ("first", ctypes.c_ulonglong)]


@pytest.fixture(scope="module")
def lib(tmp_path_factory):
    out = str(tmp_path_factory.mktemp("ffcheck") / "libffcheck.so")
    subprocess.run(["g++", "-std=c++17", "-O2", "-ffp-contract=off", "-fopenmp", "-shared",
                    "-fPIC", "-I", os.path.join(ROOT, "synaptogenesis_gb300", "csrc"),
                    os.path.join(ROOT, "tests", "cpu_checks", "ff_check.cpp"), "-o", out],
                   check=True)
    return ctypes.CDLL(out)


def _check(r, max_fallback):
    assert r.mismatches == 0, "first mismatch at %#x" % r.first
    assert r.fallbacks <= max_fallback * r.checked, (r.fallbacks, r.checked)


def test_weight_derivative_strided(lib):
    r = Result()
    lib.check_wd_strided(ctypes.c_ulonglong(61), ctypes.c_ulonglong(7), ctypes.byref(r))
    assert r.checked == len(range(7, 1 << 32, 61))
    # fallbacks: non-finite and huge operands, results below 2^-101
    _check(r, 0.6)


def test_trace_decay_product_strided(lib):
    r = Result()
    lib.check_product_strided(ctypes.c_ulonglong(61), ctypes.c_ulonglong(5), ctypes.byref(r))
    _check(r, 0.16)       # non-finite and huge operands, results below 2^-126


@pytest.mark.parametrize("c", [0.95, 0.9])
def test_spnet_decay_products_strided(lib, c):
    """spnet's presynaptic trace and weight derivative decays."""
    r = Result()
    lib.check_product_c_strided(ctypes.c_double(c), ctypes.c_ulonglong(61), ctypes.c_ulonglong(11),
                                ctypes.byref(r))
    _check(r, 0.16)


@pytest.mark.parametrize("k", [0.01, 0.1])
def test_sum_with_double_constant_strided(lib, k):
    """spnet's weight step (dw + 0.01) and trace step (p + 0.1)."""
    r = Result()
    lib.check_add_const_strided(ctypes.c_double(k), ctypes.c_ulonglong(61), ctypes.c_ulonglong(13),
                                ctypes.byref(r))
    _check(r, 0.16)       # non-finite operands and results outside the normal range


@pytest.mark.parametrize("divisor", [60, 700, 800])
def test_division_by_integer_strided(lib, divisor):
    r = Result()
    lib.check_div_strided(divisor, ctypes.c_ulonglong(61), ctypes.c_ulonglong(3), ctypes.byref(r))
    _check(r, 0.0)


@pytest.mark.parametrize("sub", [0, 1])
@pytest.mark.parametrize("spike", [0, 1])
def test_short_term_w_strided(lib, sub, spike):
    r = Result()
    lib.check_sw_strided(sub, spike, ctypes.c_ulonglong(61), ctypes.c_ulonglong(11),
                         ctypes.byref(r))
    _check(r, 0.6)


def test_weight_derivative_random_spike_terms(lib):
    r = Result()
    lib.check_wd_random(ctypes.c_ulonglong(20_000_000), ctypes.c_ulonglong(5), ctypes.byref(r))
    assert r.checked == 20_000_000
    _check(r, 1e-3)


def test_izhikevich_substep_random(lib):
    dv, vr, tr = Result(), Result(), Result()
    lib.check_iz_random(ctypes.c_ulonglong(20_000_000), ctypes.c_ulonglong(7), ctypes.byref(dv),
                        ctypes.byref(vr), ctypes.byref(tr))
    assert dv.checked == vr.checked == tr.checked == 20_000_000
    _check(dv, 0.05)
    _check(vr, 1e-3)
    _check(tr, 1e-3)
