"""Init-config noise (uniform, normal, Poisson with fixed or per-neuron
random rates): the library's draws (counter_rng.h, built for the host with the
same float operations as the device kernel) against the oracle's numpy
restatement bit for bit, and the draws' statistics against their
distributions.  The reference's generators are unseeded, so parity with it is
statistical only."""
import ctypes
import os
import subprocess

import numpy as np
import pytest

from oracle import oracle as O

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
N = 200_000


@pytest.fixture(scope="module")
def lib(tmp_path_factory):
    out = str(tmp_path_factory.mktemp("noise") / "libnoise.so")
    subprocess.run(["g++", "-std=c++17", "-O2", "-ffp-contract=off", "-shared", "-fPIC",
                    "-I", os.path.join(ROOT, "synaptogenesis_gb300", "csrc"),
                    os.path.join(ROOT, "tests", "cpu_checks", "noise_check.cpp"), "-o", out],
                   check=True)
    L = ctypes.CDLL(out)
    L.noise_batch.argtypes = (ctypes.c_int, ctypes.c_ulonglong, ctypes.c_ulonglong, ctypes.c_int,
                              ctypes.c_float, ctypes.c_float, ctypes.c_void_p, ctypes.c_void_p)
    return L


def host(lib, kind, seed, step, a, b, rates=None):
    out = np.empty(N, np.float32)
    r = None if rates is None else rates.ctypes.data
    lib.noise_batch({"uniform": 0, "normal": 1, "poisson": 2}[kind], seed, step, N, a, b, r,
                    out.ctypes.data)
    return out


@pytest.mark.parametrize("step", [0, 1, 12345])
def test_uniform_and_normal_match_oracle(lib, step):
    for kind, a, b in (("uniform", -1.5, 2.5), ("normal", 0.5, 2.0)):
        got = host(lib, kind, 99, step, a, b)
        want = O.noise_draw(kind, 99, step, N, a, b)
        assert np.array_equal(got.view(np.uint32), want.view(np.uint32)), kind


def test_poisson_matches_oracle(lib):
    rate = np.float32(0.001) * np.float32(50.0)
    got = host(lib, "poisson", 7, 3, rate, 4.0)
    want = np.where(O.noise_draw("poisson", 7, 3, N, rate, 0.0), np.float32(4.0), np.float32(0.0))
    assert np.array_equal(got, want)
    rates = O.rng_uniform(7, O.RNG_NOISE_RATE, np.arange(N)) * rate
    got = host(lib, "poisson", 7, 3, rate, 4.0, rates)
    want = np.where(O.noise_draw("poisson", 7, 3, N, rate, 0.0, rates), np.float32(4.0),
                    np.float32(0.0))
    assert np.array_equal(got, want)


def test_statistics():
    u = O.noise_draw("uniform", 5, 0, N, -1.0, 3.0)
    assert u.min() >= -1.0 and u.max() <= 3.0
    assert abs(u.mean() - 1.0) < 0.02 and abs(u.var() - 16.0 / 12.0) < 0.02
    g = O.noise_draw("normal", 5, 1, N, 0.5, 2.0).astype(np.float64)
    assert abs(g.mean() - 0.5) < 0.02 and abs(g.std() - 2.0) < 0.02
    z = (g - 0.5) / 2.0
    assert abs((z ** 3).mean()) < 0.03 and abs((z ** 4).mean() - 3.0) < 0.06
    p = O.noise_draw("poisson", 5, 2, N, 0.05, 0.0)
    assert abs(p.mean() - 0.05) < 0.003
    rates = O.rng_uniform(5, O.RNG_NOISE_RATE, np.arange(N)) * np.float32(0.05)
    assert rates.min() >= 0.0 and rates.max() < 0.05 and abs(rates.mean() - 0.025) < 0.001
    fires = np.mean([O.noise_draw("poisson", 5, t, N, 0.05, 0.0, rates).mean() for t in range(5)])
    assert abs(fires - 0.025) < 0.002
