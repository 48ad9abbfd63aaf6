"""Ensembles of realisations captured into one CUDA graph, and the FFT tile autotuner."""
import numpy as np
import pytest

import mitos_gb300.lib as ml

pytestmark = pytest.mark.gpu

# (N, box) pairs of 4 Mpc/h cells
SIZES = [(64, 256.0), (96, 384.0), (128, 512.0)]


def _cfgs(table, per_size, seed0=1000):
    cfgs, s = [], seed0
    for N, L in SIZES:
        for _ in range(per_size):
            cfgs.append(ml.ic_config(N, N, L, s, table, method=ml.METHOD_2LPT, pk_bins=32, pk_linear=True,
                                     precision=ml.FP32))
            s += 1
    return cfgs


def test_graph_replay_matches_single_runs(table, spline):
    """P(k) of every member after a graph replay equals a standalone pipeline run of its config
    (the CIC flush and the P(k) sums are floating-point atomics, so the order of additions may
    differ at the 1e-7 level)"""
    cfgs = _cfgs(table, 2)
    ens = ml.Ensemble(cfgs, spline, streams=4)
    try:
        ens.run()
        ms = ens.run()
        # the members of each size form one batched unit: 14 launches or more per unit
        assert ens.units() == len(SIZES)
        assert ms > 0 and ens.launches() >= 14 * ens.units()
        for i, c in enumerate(cfgs):
            ref = ml.ic_pipeline_run(c, spline)
            got = ens.result(i)
            assert np.array_equal(got["pk_obs"], ref["pk_obs"])
            # an empty shell (the first linear shell holds only the skipped DC mode) is NaN in both
            assert np.allclose(got["pk_k"], ref["pk_k"], rtol=1e-12, equal_nan=True)
            assert np.allclose(got["pk_p"], ref["pk_p"], rtol=1e-5, atol=0, equal_nan=True), i
    finally:
        ens.close()


@pytest.mark.parametrize("max_batch", [1, 3])
def test_batched_units_match_unbatched_runs(table, spline, max_batch):
    """members interleaved across sizes and seeds; batches of 1 (every member its own run) and 3
    (ragged units of 3 + 1 + ...) give the P(k) of the default batching"""
    base = _cfgs(table, 4, seed0=77)
    cfgs = base[::2] + base[1::2]  # interleave: members of one size are not adjacent
    ref = ml.Ensemble(cfgs, spline, streams=3)
    ens = ml.Ensemble(cfgs, spline, streams=5, max_batch=max_batch)
    try:
        ref.run()
        ens.run()
        per = 4
        want_units = len(SIZES) * (per if max_batch == 1 else -(-per // max_batch))
        assert ens.units() == want_units and ref.units() == len(SIZES)
        for i in range(len(cfgs)):
            a, b = ens.result(i), ref.result(i)
            assert np.array_equal(a["pk_obs"], b["pk_obs"])
            assert np.allclose(a["pk_p"], b["pk_p"], rtol=1e-5, atol=0, equal_nan=True), i
        # distinct seeds give distinct spectra (no member reads another's grids)
        p = [ens.result(i)["pk_p"][1:] for i in range(len(cfgs))]
        assert all(not np.allclose(p[i], p[j]) for i in range(len(p)) for j in range(i)
                   if cfgs[i].N == cfgs[j].N)
    finally:
        ens.close()
        ref.close()


def test_autotuner_keeps_results(table, spline):
    N, L = 64, 256.0
    cfg = ml.ic_config(N, N, L, 1000, table, method=ml.METHOD_2LPT, pk_bins=32, precision=ml.FP32)
    default = ml.get_tiles(N, ml.FP32)
    default_radix = ml.get_radix(N, ml.FP32)
    assert default_radix == ([8, 8], [8, 4])
    ref = ml.ic_pipeline_run(cfg, spline)
    try:
        pxy, pz, ms = ml.autotune(cfg, spline)
        assert ml.get_tiles(N, ml.FP32) == (pxy, pz) and ms > 0
        rn, rh = ml.get_radix(N, ml.FP32)
        assert np.prod(rn) == N and np.prod(rh) == N // 2
        got = ml.ic_pipeline_run(cfg, spline)
        assert np.allclose(got["pk_p"], ref["pk_p"], rtol=1e-5, equal_nan=True)
        with pytest.raises(ml.MitosError):
            ml.set_tiles(N, ml.FP32, 4096, 1)
    finally:
        ml.set_tiles(N, ml.FP32, *default)
        ml.set_radix(N, ml.FP32, *default_radix)


@pytest.mark.parametrize("N,prec,rn,rh", [(64, ml.FP32, [2, 4, 8], [4, 2, 4]), (96, ml.FP32, [3, 4, 4, 2], [2, 3, 4, 2]),
                                          (64, ml.FP64, [4, 4, 4], [2, 2, 8]), (256, ml.FP32, [4, 8, 8], [8, 4, 4])])
def test_radix_schedules_keep_results(table, spline, N, prec, rn, rh):
    """every radix order computes the same transforms: the IC's P(k) and positions with a
    non-default schedule (for 256^3 FP32 on the runtime-plan kernels instead of the compile-time
    ones) against the default; a schedule whose product is not N is refused"""
    L = 4.0 * N
    cfg = ml.ic_config(N, N, L, 7, table, method=ml.METHOD_2LPT, pk_bins=16, precision=prec)
    default_radix = ml.get_radix(N, prec)
    ref = ml.ic_pipeline_run(cfg, spline, want_pos=True)
    try:
        ml.set_radix(N, prec, rn, rh)
        assert ml.get_radix(N, prec) == (rn, rh)
        got = ml.ic_pipeline_run(cfg, spline, want_pos=True)
        tol = 1e-5 if prec == ml.FP32 else 1e-12
        assert np.allclose(got["pk_p"], ref["pk_p"], rtol=tol, equal_nan=True)
        d = got["pos"].astype(np.float64) - ref["pos"].astype(np.float64)
        d -= L * np.round(d / L)
        assert np.abs(d).max() < (1e-3 if prec == ml.FP32 else 1e-9) * L / N
        with pytest.raises(ml.MitosError):
            ml.set_radix(N, prec, rn + [2], rh)
    finally:
        ml.set_radix(N, prec, *default_radix)
