"""CPU checks of the FP64 white noise's arithmetic: the correctly rounded log and cos that the GPU's
sampleNorm (src/random.c:34-49) uses, through the library's host copies of the device code.

Bit-exactness with the reference: the reference's Gaussians come from the host libm, which
misrounds log and cos by an ulp on a small fraction of inputs (glibc: about 0.1% each).  The GPU
computes the exactly rounded value; these tests show that it equals the reference everywhere else
and that every difference is such a libm misrounding, checked against 60-90 digit decimal
arithmetic."""
import ctypes
import math
import os
import random

import numpy as np
import pytest

import oracle
import mitos_gb300.lib as ml
from oracle.crcheck import exact_cos, exact_log, libm_misrounds, sample_norm_exact, sample_norm_parts

GOLDEN = os.path.join(os.path.dirname(__file__), "golden")
_d = ctypes.c_double


@pytest.fixture(scope="module")
def lib():
    L = ml.load()
    for f in ("mitos_cr_log", "mitos_cr_cos"):
        getattr(L, f).restype = _d
        getattr(L, f).argtypes = [_d]
    L.mitos_sample_norm_cr.restype = _d
    L.mitos_sample_norm_cr.argtypes = [ctypes.c_uint64, ctypes.c_uint64]
    L.mitos_cr_steps.argtypes = [ctypes.c_int, _d, ctypes.POINTER(_d), ctypes.POINTER(_d)]
    return L


def _box_muller_args(n, seed):
    r = random.Random(seed)
    out = []
    for _ in range(n):
        out.append(sample_norm_parts(r.getrandbits(64), r.getrandbits(64)))
    return out


def _edge_logs():
    xs = [(float(A) + 0.5) / 2.0 ** 64 for A in list(range(64)) + [2 ** 64 - 1 - 4093 * i for i in range(64)]]
    xs += [1 - k * 2.0 ** -53 for k in range(1, 200)]
    xs += [math.ldexp(1 + i / 128, e) for i in range(128) for e in (-1, -7, -40, -65)]
    xs += [math.nextafter(math.ldexp(1 + i / 128, -3), 0) for i in range(1, 128)]
    return [x for x in xs if 0 < x <= 1]


def _edge_cos():
    ys = []
    for k in range(5):  # the doubles nearest k pi/2 and their neighbours
        d = k * (math.pi / 2)
        for _ in range(30):
            d = math.nextafter(d, 0)
        for _ in range(61):
            if 0 <= d < 8:
                ys.append(d)
            d = math.nextafter(d, 8)
    ys += [math.ldexp(1, -e) for e in range(1, 66)]
    ys += [j / 128 + s for j in range(101) for s in (-1 / 256, 1 / 256)]
    ys += [2 * 3.14159265358979323846, math.nextafter(2 * 3.14159265358979323846, 0)]
    return ys


def test_cr_log_is_correctly_rounded(lib):
    xs = [u for u, _ in _box_muller_args(3000, 1)] + _edge_logs()
    bad = [x for x in xs if lib.mitos_cr_log(x) != exact_log(x)]
    assert not bad, [x.hex() for x in bad[:5]]
    assert lib.mitos_cr_log(1.0) == 0.0


def test_cr_cos_is_correctly_rounded(lib):
    ys = [y for _, y in _box_muller_args(3000, 2)] + _edge_cos()
    bad = [y for y in ys if lib.mitos_cr_cos(y) != exact_cos(y)]
    assert not bad, [y.hex() for y in bad[:5]]


def test_cr_steps(lib):
    """the accurate step alone is correctly rounded; the fast step, when it decides (all but a few
    in 10^4 inputs), gives the same double"""
    f, a = _d(), _d()
    undecided = 0
    args = _box_muller_args(2000, 3)
    for fn, xs, exact, random_args in ((0, [u for u, _ in args], exact_log, True),
                                       (1, [y for _, y in args], exact_cos, True),
                                       (0, _edge_logs(), exact_log, False), (1, _edge_cos(), exact_cos, False)):
        for x in xs:
            lib.mitos_cr_steps(fn, x, ctypes.byref(f), ctypes.byref(a))
            e = exact(x)
            assert a.value == e, (fn, x.hex())
            if f.value != f.value:
                undecided += random_args
            else:
                assert f.value == e, (fn, x.hex())
    assert undecided < 0.01 * 2 * len(args)  # on the Box-Muller arguments


def test_sample_norm_vs_reference_golden(lib):
    """the reference build's sampleNorm streams (golden, seeds 42, 7, 1000-1002): the library's FP64
    Gaussians equal them bit for bit except where the reference's libm misrounded log or cos, and
    there they are the exactly rounded values"""
    g = np.load(os.path.join(GOLDEN, "sample_norm.npz"))
    total = differ = 0
    for key in g.files:
        seed = int(key.split("_")[1])
        ref = g[key]
        d = oracle.draws(seed, 2 * len(ref))
        got = np.array([lib.mitos_sample_norm_cr(int(d[2 * i]), int(d[2 * i + 1])) for i in range(len(ref))])
        for i in np.nonzero(got != ref)[0]:
            A, B = int(d[2 * i]), int(d[2 * i + 1])
            assert libm_misrounds(A, B), (key, i)
            assert got[i] == sample_norm_exact(A, B), (key, i)
            differ += 1
        total += len(ref)
    assert differ < 0.01 * total
