"""The one-pass Z + Y step of the FP32 r2c (a thread-block cluster holds each x-plane in distributed
shared memory; FP32 N = 256 and 512): the same transform as the two-pass route and as the oracle's
FFTW-convention r2c (src/fft.c:219-236), through fft_r2c_dg, the IC's density spectrum and the
Monge-Ampere source transform, for each cluster shape."""
import numpy as np
import pytest

import oracle
import mitos_gb300.lib as ml
from conftest import rel_err
from mitos_gb300.perturb import load_table

pytestmark = pytest.mark.gpu


def _names(fn):
    ml.kernel_timing(True)
    try:
        fn()
        return [k for k, _ in ml.kernel_times()]
    finally:
        ml.kernel_timing(False)


def _r2c(g, real, cluster):
    was = ml.set_cluster_fft(cluster)
    try:
        ml.set_box(g, real)
        names = _names(lambda: ml.fft_r2c_dg(g))
        return ml.get_fbox(g), names
    finally:
        ml.set_cluster_fft(was)


@pytest.mark.parametrize("mode", [1, 2, 3])
@pytest.mark.parametrize("N", [256, 512])
def test_cluster_r2c_matches_two_pass(N, mode):
    L = 2.0 * N
    g = ml.alloc_local_grid(N, L, ml.FP32)
    try:
        real = np.random.default_rng(N).standard_normal((N, N, N)).astype(np.float32)
        k1, n1 = _r2c(g, real, mode)
        k0, n0 = _r2c(g, real, 0)
        assert "zy_r2c" in n1 and "z_r2c" not in n1, n1
        assert "zy_r2c" not in n0 and "z_r2c" in n0, n0
        err = rel_err(k1, k0)
        print(f"N={N} mode {mode}: cluster vs two-pass rel err {err:.2e}")
        assert err < 1e-6
        # the packed kz = 0 / N/2 columns: Hermitian in ky like the rest
        for kz in (0, N // 2):
            c = k1[0, :, kz]
            assert rel_err(c[1:], np.conj(c[1:][::-1])) < 1e-6
        # the input stays untouched
        assert np.array_equal(ml.get_box(g)[..., :N], real)
    finally:
        ml.free_local_grid(g)


def test_cluster_r2c_vs_oracle_256():
    N, L = 256, 300.0
    g = ml.alloc_local_grid(N, L, ml.FP32)
    try:
        real = np.random.default_rng(5).standard_normal((N, N, N))
        got, names = _r2c(g, real.astype(np.float32), 1)
        assert "zy_r2c" in names
        ref = oracle.fft_r2c(N, L, real)
        assert rel_err(got, ref) < 3e-6
    finally:
        ml.free_local_grid(g)


def test_cluster_r2c_round_trip_512():
    N, L = 512, 1000.0
    g = ml.alloc_local_grid(N, L, ml.FP32)
    try:
        box = np.random.default_rng(3).standard_normal((N, N, N + 2)).astype(np.float32)
        ml.set_box(g, box)
        was = ml.set_cluster_fft(1)
        try:
            assert "zy_r2c" in _names(lambda: ml.fft_r2c_dg(g))
        finally:
            ml.set_cluster_fft(was)
        ml.fft_c2r_dg(g)
        assert rel_err(ml.get_box(g)[..., :N], box[..., :N]) < 2e-6
    finally:
        ml.free_local_grid(g)


def test_cluster_ic_power_spectrum_256():
    """the IC's density r2c through the cluster pass: P(k) per bin as with the two-pass route"""
    table = load_table()
    spline = ml.Spline(table)
    cfg = ml.ic_config(256, 256, 500.0, 7, table, pk_bins=48, pk_linear=True, precision=ml.FP32)
    was = ml.set_cluster_fft(1)
    try:
        names = _names(lambda: ml.ic_pipeline_run(cfg, spline))
        assert "zy_r2c" in names
        r1 = ml.ic_pipeline_run(cfg, spline)
        ml.set_cluster_fft(0)
        r0 = ml.ic_pipeline_run(cfg, spline)
    finally:
        ml.set_cluster_fft(was)
    p1, p0 = np.asarray(r1["pk_p"]), np.asarray(r0["pk_p"])
    ok = p0 != 0
    assert ok.sum() > 10
    assert np.abs(p1[ok] / p0[ok] - 1).max() < 1e-5
