"""The integer-pipe FP64 square root, divisions and compares (fp64_int.cuh)
built for the host, against IEEE binary64 arithmetic, bit for bit, on random operands
over the whole exponent range, on the travel-time range the solvers see, on
the hard cases of each operation (neighbours of exact squares and exact
quotients, mantissa extremes) and on zeros, subnormals, infinities and NaN
(which take the fallback).  The square root and division are also run with their FP32 seeds
degraded to 2^-19 relative error, far worse than the GPU's approximations,
to show that the Newton steps and the remainder correction do not depend on
the seed's accuracy.  CPU only; the kernels that use these operations are
checked bit for bit against the oracle by the GPU parity tests."""
import ctypes
import os
import subprocess

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
CSRC = os.path.join(ROOT, "adtomo.jl_gb300", "csrc")
SRC = os.path.join(ROOT, "tests", "fp64_int_check.cpp")


@pytest.fixture(scope="module")
def lib(tmp_path_factory):
    out = str(tmp_path_factory.mktemp("fi") / "libficheck.so")
    subprocess.run(["g++", "-O2", "-std=c++17", "-ffp-contract=off", "-fno-fast-math", "-shared",
                    "-fPIC", "-I", CSRC, SRC, "-o", out], check=True)
    L = ctypes.CDLL(out)
    L.fi_check_run.restype = ctypes.c_int
    L.fi_check_run.argtypes = [ctypes.c_int, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p,
                               ctypes.c_int64, ctypes.c_double]
    return L


def run(lib, op, a, b=None, perturb=0.0):
    a = np.ascontiguousarray(a, np.float64)
    b = np.ascontiguousarray(a if b is None else b, np.float64)
    out = np.empty_like(a)
    assert lib.fi_check_run(op, a.ctypes.data, b.ctypes.data, out.ctypes.data, a.size,
                            perturb) == 0
    return out


def same_bits(got, want):
    g, w = got.view(np.uint64), want.view(np.uint64)
    ok = (g == w) | (np.isnan(got) & np.isnan(want))
    bad = np.flatnonzero(~ok)
    return bad


def from_bits(u):
    return np.asarray(u, np.uint64).view(np.float64)


def random_doubles(rng, n, lo_exp=1, hi_exp=2046, sign=False):
    e = rng.integers(lo_exp, hi_exp + 1, n, dtype=np.uint64)
    f = rng.integers(0, 1 << 52, n, dtype=np.uint64)
    s = rng.integers(0, 2, n, dtype=np.uint64) if sign else np.zeros(n, np.uint64)
    return from_bits((s << np.uint64(63)) | (e << np.uint64(52)) | f)


def specials():
    v = [0.0, -0.0, np.inf, -np.inf, np.nan, 5e-324, -5e-324, 2.2250738585072014e-308,
         2.225073858507201e-308, 1.7976931348623157e308, 1.0, -1.0, 2.0, 0.5, 3.0, 4.0, 0.25]
    return np.array(v, np.float64)


def neighbours(x):
    x = np.asarray(x, np.float64)
    return np.concatenate([np.nextafter(x, -np.inf), x, np.nextafter(x, np.inf)])


def sqrt_inputs(rng):
    n = 400000
    parts = [random_doubles(rng, n), rng.uniform(1e-6, 1e11, n), specials(),
             random_doubles(rng, 2000, 0, 0), -random_doubles(rng, 2000)]
    y = random_doubles(rng, n, 600, 1400)  # squares and their neighbours: the hard cases
    parts.append(neighbours(y * y))
    m = from_bits((np.uint64(1023) << np.uint64(52)) | np.array([0, 1, (1 << 52) - 1, 1 << 51],
                                                                  np.uint64))
    parts.append(np.concatenate([m, 2 * m]))
    return np.concatenate(parts)


def div_inputs(rng):
    n = 400000
    a = [random_doubles(rng, n, 300, 1700, sign=True), rng.uniform(1e-3, 1e5, n)]
    b = [random_doubles(rng, n, 300, 1700, sign=True), rng.uniform(1e-3, 1e5, n)]
    q, d = random_doubles(rng, n, 900, 1100), random_doubles(rng, n, 900, 1100)
    p = q * d  # exact-ish quotients and their neighbours
    a.append(neighbours(p))
    b.append(np.concatenate([d, d, d]))
    a.append(rng.uniform(0, 10, n) * 3.0)  # divisions by 3 (the three-axis solve)
    b.append(np.full(n, 3.0))
    s = specials()
    a.append(np.repeat(s, s.size))
    b.append(np.tile(s, s.size))
    a.append(random_doubles(rng, 5000, 1, 2046))  # results near under/overflow
    b.append(random_doubles(rng, 5000, 1, 2046))
    mant = from_bits((np.uint64(1023) << np.uint64(52)) | np.array(
        [0, 1, (1 << 52) - 1, (1 << 52) - 2], np.uint64))
    a.append(np.repeat(mant, mant.size))
    b.append(np.tile(mant, mant.size))
    return np.concatenate(a), np.concatenate(b)


@pytest.mark.parametrize("perturb", [0.0, 2.0 ** -19])
def test_sqrt_bit_exact(lib, perturb):
    x = sqrt_inputs(np.random.default_rng(11))
    with np.errstate(invalid="ignore"):
        want = np.sqrt(x)
    bad = same_bits(run(lib, 0, x, perturb=perturb), want)
    assert bad.size == 0, f"{bad.size} mismatches, first x={x[bad[:5]]!r}"


def test_div3_bit_exact(lib):
    rng = np.random.default_rng(15)
    n = 400000
    s = specials()
    x = np.concatenate([random_doubles(rng, n, 0, 2047, sign=True), rng.uniform(0, 1e5, n),
                        3.0 * random_doubles(rng, n, 2, 2040), s, -s,
                        from_bits(np.arange(1 << 52, (1 << 52) + 4096, dtype=np.uint64)),
                        from_bits((np.uint64(1) << np.uint64(52)) * np.arange(1, 5, dtype=np.uint64)
                                  | np.uint64((1 << 52) - 1))])
    with np.errstate(all="ignore"):
        want = x / 3.0
    bad = same_bits(run(lib, 2, x), want)
    assert bad.size == 0, f"{bad.size} mismatches, first x={x[bad[:5]]!r}"


@pytest.mark.parametrize("perturb", [0.0, 2.0 ** -19])
def test_div_bit_exact(lib, perturb):
    a, b = div_inputs(np.random.default_rng(12))
    with np.errstate(all="ignore"):
        want = a / b
    bad = same_bits(run(lib, 1, a, b, perturb), want)
    assert bad.size == 0, f"{bad.size} mismatches, first a={a[bad[:5]]!r} b={b[bad[:5]]!r}"


def test_compares_without_nan(lib):
    """a < b, a <= b, a == b and min(a, b) = (b < a ? b : a) for non-NaN
    doubles: signed values over the whole range, subnormals, infinities, both
    zeros, equal pairs."""
    rng = np.random.default_rng(16)
    n = 300000
    s = specials()
    s = s[~np.isnan(s)]
    a = np.concatenate([random_doubles(rng, n, 0, 2046, sign=True), rng.uniform(0, 1e5, n),
                        np.repeat(s, s.size), np.array([0.0, -0.0, 0.0, -0.0, np.inf, -np.inf])])
    b = np.concatenate([random_doubles(rng, n, 0, 2046, sign=True),
                        np.where(rng.random(n) < 0.3, a[n:2 * n], rng.uniform(0, 1e5, n)),
                        np.tile(s, s.size), np.array([-0.0, 0.0, 0.0, -0.0, np.inf, np.inf])])
    for op, want in ((3, a < b), (4, a <= b), (5, a == b)):
        assert np.array_equal(run(lib, op, a, b) != 0.0, want), op
    assert same_bits(run(lib, 6, a, b), np.where(b < a, b, a)).size == 0
