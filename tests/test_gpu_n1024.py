"""FP32 ICs against FP64 ICs of the same seed through P(k) per bin, where the box-scale modes are
sensitive: the 1024^3 IC (box 2000 Mpc/h, 256 linear shells), whose FP32 passes are the
compile-time transforms of length 1024 (X, Y; 16 elements a thread in the Hessian and combine X
passes) and 512 (Z rows held by two warps on named barriers), which no smaller case runs; and a
256^3 IC in the same box.  The FP32 deposit maps positions to grid coordinates with N / L split
into two floats: with N / L rounded to one float (2000 / 256 and 2000 / 1024 are not binary
fractions) the stretched particle distribution moved the power of the fundamental modes along the
axes by 3e-4 - 4e-4 against FP64."""
import numpy as np
import pytest

import mitos_gb300.lib as ml

pytestmark = pytest.mark.gpu


def _ic(N, L, table, spline, prec, method=ml.METHOD_2LPT, bins=256):
    cfg = ml.ic_config(N, N, L, 42, table, method=method, pk_bins=bins, pk_linear=True, precision=prec)
    return ml.ic_pipeline_run(cfg, spline)


def _pk_rel(a, b):
    assert np.array_equal(a["pk_obs"], b["pk_obs"])
    ok = b["pk_obs"] > 0
    return np.abs(a["pk_p"][ok] / b["pk_p"][ok] - 1)


@pytest.mark.parametrize("method", [ml.METHOD_ZELDOVICH, ml.METHOD_2LPT])
def test_box_scale_modes_256_fp32(method, table, spline):
    N, L = 256, 2000.0
    a = _ic(N, L, table, spline, ml.FP32, method, 64)
    b = _ic(N, L, table, spline, ml.FP64, method, 64)
    rel = _pk_rel(a, b)
    print(f"256^3 L = 2000 P(k) FP32 vs FP64: bin 0 {rel[0]:.2e}, max {rel.max():.2e}")
    assert rel.max() < 2e-5


def test_ic_1024_fp32_vs_fp64(table, spline):
    N, L = 1024, 2000.0
    # one precision's workspaces at a time (about 65 GB in FP32, 130 GB in FP64)
    ml.load().mitos_release_all()
    try:
        a = _ic(N, L, table, spline, ml.FP32)
        again = _ic(N, L, table, spline, ml.FP32)
        ml.load().mitos_release_all()
        b = _ic(N, L, table, spline, ml.FP64)
    finally:
        ml.load().mitos_release_all()
    assert np.array_equal(a["pk_p"], again["pk_p"]), "FP32 IC not deterministic"
    rel = _pk_rel(a, b)
    assert rel.size > 200
    print(f"1024^3 P(k) FP32 vs FP64: bin 0 {rel[0]:.2e}, max rel {rel.max():.2e} over {rel.size} bins")
    assert rel.max() < 2e-5
