"""The lattice deposit's tile staging by tensor copies (cp.async.bulk.tensor on an mbarrier, the
bricks off the box's x and y faces) against 16-byte cp.async staging of every brick: the same
tiles, so bit-identical positions and P(k) (src/particle.c:87-129, analyse/src/mitos_read.c:280-334)."""
import numpy as np
import pytest

import mitos_gb300.lib as ml
from mitos_gb300.perturb import load_table

pytestmark = pytest.mark.gpu


def _names(fn):
    ml.kernel_timing(True)
    try:
        fn()
        return [k for k, _ in ml.kernel_times()]
    finally:
        ml.kernel_timing(False)


@pytest.mark.parametrize("N,L,prec", [(64, 128.0, ml.FP32), (256, 500.0, ml.FP32), (128, 256.0, ml.FP64),
                                      (512, 1000.0, ml.FP32)])
def test_tma_staging_bit_identical(N, L, prec):
    table = load_table()
    spline = ml.Spline(table)
    cfg = ml.ic_config(N, N, L, 11, table, pk_bins=32, pk_linear=True, precision=prec)
    was = ml.set_lattice_tma(True)
    try:
        r1 = ml.ic_pipeline_run(cfg, spline, want_pos=True)
        assert "lattice_cic" in _names(lambda: ml.ic_pipeline_run(cfg, spline))
        ml.set_lattice_tma(False)
        r0 = ml.ic_pipeline_run(cfg, spline, want_pos=True)
    finally:
        ml.set_lattice_tma(was)
    assert np.array_equal(r1["pos"], r0["pos"])
    ok = r1["pk_obs"] > 0  # empty shells are 0/0 in both
    assert np.all(np.isfinite(r1["pk_p"][ok])) and r1["pk_p"][ok].max() > 0
    if prec == ml.FP32:
        # 32-bit fixed-point deposit sums: exact and order independent
        assert np.array_equal(r1["pk_p"][ok], r0["pk_p"][ok])
    else:
        # FP64 deposit sums are shared-memory double atomics, whose order varies from run to run
        assert np.abs(r1["pk_p"][ok] / r0["pk_p"][ok] - 1).max() < 1e-12


@pytest.mark.parametrize("N,L", [(256, 500.0), (512, 1000.0)])
def test_region_order_bit_identical(N, L):
    """the deposit's regional brick order against row order: the same particles into the same
    fixed-point sums (FP32), so identical positions and P(k)"""
    table = load_table()
    spline = ml.Spline(table)
    cfg = ml.ic_config(N, N, L, 5, table, pk_bins=32, pk_linear=True, precision=ml.FP32)
    was = ml.set_lattice_order(True)
    try:
        r1 = ml.ic_pipeline_run(cfg, spline, want_pos=True)
        ml.set_lattice_order(False)
        r0 = ml.ic_pipeline_run(cfg, spline, want_pos=True)
    finally:
        ml.set_lattice_order(was)
    assert np.array_equal(r1["pos"], r0["pos"])
    ok = r1["pk_obs"] > 0
    assert np.array_equal(r1["pk_p"][ok], r0["pk_p"][ok])


@pytest.mark.parametrize("N,L,prec", [(128, 256.0, ml.FP32), (128, 256.0, ml.FP64), (256, 500.0, ml.FP32)])
def test_velocity_gather_tma_bit_identical(N, L, prec):
    """the velocity gather's interior bricks staged by tensor copies against cp.async for all:
    the same tiles, identical velocities (src/mitos.c:865-908)"""
    table = load_table()
    spline = ml.Spline(table)
    cfg = ml.ic_config(N, N, L, 8, table, pk_bins=16, pk_linear=True, precision=prec,
                       index_vel=table.index_of("t_cdm"))
    was = ml.set_lattice_tma(True)
    try:
        assert "vel_gather" in _names(lambda: ml.ic_pipeline_run(cfg, spline, want_vel=True))
        r1 = ml.ic_pipeline_run(cfg, spline, want_pos=True, want_vel=True)
        ml.set_lattice_tma(False)
        r0 = ml.ic_pipeline_run(cfg, spline, want_pos=True, want_vel=True)
    finally:
        ml.set_lattice_tma(was)
    assert np.array_equal(r1["pos"], r0["pos"])
    assert np.array_equal(r1["vel"], r0["vel"])
    assert np.abs(r1["vel"]).max() > 0
