"""calc_cross_powerspec_noalloc: the P(k) binning for callers that cannot allocate device memory
(another allocator already owns the GPU's memory, or a cudaMalloc would synchronise their
streaming loop).  Its scratch is a fixed device array; it must give the same bins as the regular
calc_cross_powerspec, call after call.  This file is collected last on purpose."""
import ctypes

import numpy as np
import pytest

import mitos_gb300.lib as ml

pytestmark = pytest.mark.gpu


def _noalloc(N, L, g1, g2, bins, linear=0):
    k = np.zeros(bins)
    p = np.zeros(bins)
    o = np.zeros(bins, np.int64)
    st = ml.load().calc_cross_powerspec_noalloc(
        N, ctypes.c_double(L), ctypes.c_void_p(g1.fbox), ctypes.c_void_p(g2.fbox), g1.precision, bins,
        linear, k.ctypes.data_as(ml._dp), p.ctypes.data_as(ml._dp), o.ctypes.data_as(ml._lp))
    return st, k, p, o


@pytest.mark.parametrize("prec", [ml.FP64, ml.FP32])
def test_noalloc_matches_regular_entry_point_twice(prec):
    N, L, bins = 64, 256.0, 24
    rng = np.random.default_rng(17)
    shape = (N, N, N // 2 + 1)
    a = rng.standard_normal(shape) + 1j * rng.standard_normal(shape)
    b = rng.standard_normal(shape) + 1j * rng.standard_normal(shape)
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


def test_noalloc_rejects_too_many_bins():
    g = ml.alloc_local_grid(16, 10.0, ml.FP64)
    st, *_ = _noalloc(16, 10.0, g, g, 5000)
    assert st == 3 and "at most 4096" in ml.last_error()
    ml.free_local_grid(g)
