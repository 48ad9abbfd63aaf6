"""calc_bispectrum (src/calc_powerspec.c:295-508) on the GPU against the oracle (pinned bit for bit
to the reference's own calc_bispectrum), and its FP32 grid form against FP64."""
import ctypes

import numpy as np
import pytest

import oracle
import mitos_gb300.lib as ml
from conftest import rel_err

pytestmark = pytest.mark.gpu

_dp = ctypes.POINTER(ctypes.c_double)


def _field(N, L, seed):
    f = oracle.grf(N, L, seed)
    return oracle.apply_kernel(N, L, f, "gaussian", np.sqrt(1 / 0.02))


def _gpu_bispectrum_host(N, L, f, bins, bins3, vol, btype, theta, k3):
    """the reference-signature entry point with a host array"""
    buf = None if f is None else np.ascontiguousarray(np.stack([f.real, f.imag], -1), np.float64)
    out = [np.zeros(bins) for _ in range(4)]
    ml.load().calc_bispectrum(N, ctypes.c_double(L), None if buf is None else buf.ctypes.data_as(ctypes.c_void_p),
                              bins, bins3, *[o.ctypes.data_as(_dp) for o in out], int(vol), int(btype),
                              ctypes.c_double(theta), ctypes.c_double(k3))
    return dict(zip(("k1", "k2", "k3", "B"), out))


@pytest.mark.parametrize("N,btype,vol,bins3", [(32, 0, False, 10), (32, 1, False, 10), (32, 0, True, 10),
                                              (48, 0, False, 10), (32, 0, False, 14)])
def test_bispectrum_fp64_vs_oracle(N, btype, vol, bins3):
    """bins3 = bins with type 0 and theta = 4 pi / 3 puts shell 3 on shell 1 (one c2r serves both);
    bins3 != bins and type 1 take two"""
    L = 4.0 * N
    f = _field(N, L, 3)
    args = dict(bins=10, bins3=bins3, vol=vol, btype=btype, theta=4 * np.pi / 3, k3=0.4)
    got = _gpu_bispectrum_host(N, L, None if vol else f, **args)
    ref = oracle.bispectrum(N, L, None if vol else f, bins=10, bins3=bins3, volume_mode=vol, btype=btype,
                            theta=4 * np.pi / 3, k3=0.4)
    full = ref["B"] != 0
    assert full.sum() >= 3
    assert np.all(got["B"][~full] == 0)  # the same empty bins
    # a filled bin may sum to exactly zero in the GPU's summation order only at the cancellation
    # scale (the atomic order varies from run to run)
    assert np.all(np.abs(ref["B"][full & (got["B"] == 0)]) < 1e-9 * np.abs(ref["B"]).max())
    for key in ("k1", "k2", "k3"):
        assert np.allclose(got[key], ref[key], rtol=1e-13, atol=0), key
    # the sums run in another order: cancellation sets the scale of the difference
    assert rel_err(got["B"], ref["B"]) < 1e-9, rel_err(got["B"], ref["B"])


def test_bispectrum_dg_fp32_vs_fp64():
    N, L = 64, 256.0
    f = _field(N, L, 8)
    out = {}
    for prec in (ml.FP64, ml.FP32):
        g = ml.alloc_local_grid(N, L, prec)
        ml.set_fbox(g, f)
        g.momentum_space = b"\x01"
        out[prec] = ml.calc_bispectrum(g, 12, 12, btype=0, theta=4 * np.pi / 3)
        ml.free_local_grid(g)
    b64, b32 = out[ml.FP64]["B"], out[ml.FP32]["B"]
    # the same bins are empty (k1 = 0); the smoothed field's high-k bins fall below 1e-30, where
    # FP32 underflows, so B is compared where it is within 1e-6 of its largest value
    assert np.array_equal(out[ml.FP64]["k1"] == 0, out[ml.FP32]["k1"] == 0)
    big = np.abs(b64) > 1e-6 * np.abs(b64).max()
    assert big.sum() >= 5
    assert rel_err(b32[big], b64[big]) < 1e-4, rel_err(b32[big], b64[big])
    assert np.allclose(out[ml.FP32]["k1"], out[ml.FP64]["k1"], rtol=1e-12)
    g = ml.alloc_local_grid(N, L, ml.FP32)
    with pytest.raises(ml.MitosError):  # not in momentum space
        ml.calc_bispectrum(g, 12, 12)
    ml.free_local_grid(g)


def test_bispectrum_256_fp32_vs_fp64():
    """256^3 (the mask, c2r and triple-sum kernels at a size whose grids together exceed L2): the FP32
    grid form against FP64, equilateral, bins above 1e-6 of the largest"""
    N, L = 256, 500.0
    out = {}
    for prec in (ml.FP32, ml.FP64):
        g = ml.alloc_local_grid(N, L, prec)
        try:
            ml.generate_complex_grf(g, ml.rng_init(9))
            g.momentum_space = b"\x01"
            out[prec] = ml.calc_bispectrum(g, 12, 12, btype=0, theta=4 * np.pi / 3)
        finally:
            ml.free_local_grid(g)
    a, b = out[ml.FP32], out[ml.FP64]
    assert np.array_equal(a["k1"] == 0, b["k1"] == 0)
    assert np.allclose(a["k1"], b["k1"], rtol=1e-12)
    big = np.abs(b["B"]) > 1e-6 * np.abs(b["B"]).max()
    assert big.sum() >= 6
    rel = np.abs(a["B"][big] / b["B"][big] - 1)
    print(f"bispectrum FP32 vs FP64 at 256^3: max rel {rel.max():.2e}")
    assert rel.max() < 1e-3
