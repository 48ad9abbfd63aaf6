"""calc_cross_powerspec_noalloc: the P(k) binning for callers that cannot allocate device memory
(another allocator already owns the GPU's memory, or a cudaMalloc would synchronise their
streaming loop).  Its scratch is a fixed device array; it must bin every mode as the regular
calc_cross_powerspec and the oracle do, call after call.  This file is collected last on purpose."""
import ctypes
import os
import subprocess
import sys

import numpy as np
import pytest

import oracle
import mitos_gb300.lib as ml

pytestmark = pytest.mark.gpu

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _noalloc(N, L, g1, g2, bins, linear=0):
    k = np.zeros(bins)
    p = np.zeros(bins)
    o = np.zeros(bins, np.int64)
    st = ml.load().calc_cross_powerspec_noalloc(
        N, ctypes.c_double(L), ctypes.c_void_p(g1.fbox), ctypes.c_void_p(g2.fbox), g1.precision, bins,
        linear, k.ctypes.data_as(ml._dp), p.ctypes.data_as(ml._dp), o.ctypes.data_as(ml._lp))
    return st, k, p, o


def _fields(N, seed):
    rng = np.random.default_rng(seed)
    shape = (N, N, N // 2 + 1)
    a = rng.standard_normal(shape) + 1j * rng.standard_normal(shape)
    b = rng.standard_normal(shape) + 1j * rng.standard_normal(shape)
    return a, b


@pytest.mark.parametrize("prec", [ml.FP64, ml.FP32])
def test_noalloc_matches_regular_entry_point_twice(prec):
    N, L, bins = 64, 256.0, 24
    a, b = _fields(N, 17)
    g1 = ml.alloc_local_grid(N, L, prec)
    g2 = ml.alloc_local_grid(N, L, prec)
    ml.set_fbox(g1, a)
    ml.set_fbox(g2, b)
    k0, p0, o0 = ml.calc_cross_powerspec(N, L, g1, g2, bins, precision=prec)
    for _ in range(2):  # the shared scratch array must be cleared between calls
        st, k, p, o = _noalloc(N, L, g1, g2, bins)
        assert st == 0, ml.last_error()
        assert np.array_equal(o, o0)
        ok = o0 > 0
        assert np.allclose(p[ok], p0[ok], rtol=1e-12, atol=1e-12 * np.abs(p0[ok]).max())
        assert np.allclose(k[ok], k0[ok], rtol=1e-12)
    ml.free_local_grid(g1)
    ml.free_local_grid(g2)


@pytest.mark.parametrize("N,L,bins,linear", [(64, 256.0, 24, 0), (64, 256.0, 32, 1), (32, 100.0, 7, 0),
                                             (48, 1000.0, 128, 0), (96, 384.0, 48, 1), (128, 500.0, 128, 0),
                                             (16, 10.0, 3, 1), (64, 256.0, 4096, 0)])
def test_noalloc_matches_oracle(N, L, bins, linear):
    """the reference's float-u log bins (src/calc_powerspec.c:61-63) and linear shells, against
    the oracle's restatement, over sizes, boxes and bin counts up to the 4096-bin maximum"""
    a, b = _fields(N, N + bins)
    g1 = ml.alloc_local_grid(N, L, ml.FP64)
    g2 = ml.alloc_local_grid(N, L, ml.FP64)
    ml.set_fbox(g1, a)
    ml.set_fbox(g2, b)
    for _ in range(2):
        st, k, p, o = _noalloc(N, L, g1, g2, bins, linear)
        assert st == 0, ml.last_error()
        rk, rp, ro = oracle.powerspec(N, L, a, b, bins, linear=bool(linear))
        assert np.array_equal(o, ro)
        ok = ro > 0
        assert np.abs(p[ok] - rp[ok]).max() <= 1e-12 * np.abs(rp[ok]).max()
        assert np.abs(k[ok] / rk[ok] - 1).max() < 1e-12
    # the six |n| = 1 modes (multiplicity 1 on the kz = 0 plane, 2 for kz = 1) sit in log bin 0
    # (u = 0 exactly), or in linear shell bins / (N/2) (shells of width (N/2) / bins in |n|)
    one = np.zeros((N, N, N // 2 + 1), complex)
    for x, y, z in ((1, 0, 0), (N - 1, 0, 0), (0, 1, 0), (0, N - 1, 0), (0, 0, 1)):
        one[x, y, z] = 1.0
    ml.set_fbox(g1, one)
    st, k, p, o = _noalloc(N, L, g1, g1, bins, linear)
    assert st == 0
    b1 = bins // (N // 2) if linear else 0
    assert o[b1] >= 6
    others = np.arange(bins) != b1
    assert p[b1] > 0 and np.all(p[others & (o > 0)] == 0)
    ml.free_local_grid(g1)
    ml.free_local_grid(g2)


def test_noalloc_allocates_nothing():
    """free device memory is the same before and after a call (after the set-up call)"""
    torch = pytest.importorskip("torch")
    N, L, bins = 64, 256.0, 512
    a, b = _fields(N, 3)
    g1 = ml.alloc_local_grid(N, L, ml.FP32)
    g2 = ml.alloc_local_grid(N, L, ml.FP32)
    ml.set_fbox(g1, a)
    ml.set_fbox(g2, b)
    assert ml.load().calc_cross_powerspec_noalloc(0, ctypes.c_double(0), None, None, 0, 0, 0, None, None, None) == 0
    torch.cuda.synchronize()
    free0 = torch.cuda.mem_get_info()[0]
    for linear in (0, 1):
        st, *_ = _noalloc(N, L, g1, g2, bins, linear)
        assert st == 0, ml.last_error()
    torch.cuda.synchronize()
    assert torch.cuda.mem_get_info()[0] == free0
    ml.free_local_grid(g1)
    ml.free_local_grid(g2)


def test_noalloc_first_call_in_a_fresh_process():
    """the set-up path: the first call of a new process (set-up-only, then a real call) returns 0"""
    code = (
        "import ctypes, numpy as np, mitos_gb300.lib as ml\n"
        "lib = ml.load()\n"
        "assert lib.calc_cross_powerspec_noalloc(0, ctypes.c_double(0), None, None, 0, 0, 0, None, None, None) == 0\n"
        "N, L, bins = 32, 100.0, 8\n"
        "g = ml.alloc_local_grid(N, L, ml.FP64)\n"
        "r = np.random.default_rng(1)\n"
        "ml.set_fbox(g, r.standard_normal((N, N, N // 2 + 1)) + 0j)\n"
        "k, p, o = np.zeros(bins), np.zeros(bins), np.zeros(bins, np.int64)\n"
        "st = lib.calc_cross_powerspec_noalloc(N, ctypes.c_double(L), ctypes.c_void_p(g.fbox), ctypes.c_void_p(g.fbox),"
        " ml.FP64, bins, 0, k.ctypes.data_as(ml._dp), p.ctypes.data_as(ml._dp), o.ctypes.data_as(ml._lp))\n"
        "assert st == 0, ml.last_error()\n"
        "assert o.sum() == N * N * N - 1, o.sum()\n"
        "print('fresh ok')\n")
    r = subprocess.run([sys.executable, "-c", code], cwd=ROOT, capture_output=True, text=True, timeout=300)
    assert r.returncode == 0 and "fresh ok" in r.stdout, r.stdout + r.stderr


def test_noalloc_rejects_too_many_bins():
    g = ml.alloc_local_grid(16, 10.0, ml.FP64)
    st, *_ = _noalloc(16, 10.0, g, g, 4097)
    assert st == 3 and "at most 4096" in ml.last_error()
    ml.free_local_grid(g)
