"""GPU parity of the fused initial-condition pipeline against the oracle (the reference restated)
and the FP32 precision study against the FP64 GPU path."""
import ctypes

import numpy as np
import pytest

import oracle
import mitos_gb300.lib as ml
from conftest import rel_err

pytestmark = pytest.mark.gpu


def _wrapdiff(a, b, L):
    d = np.asarray(a, np.float64) - np.asarray(b, np.float64)
    return d - L * np.round(d / L)


@pytest.mark.parametrize("N,method,lin", [(32, ml.METHOD_2LPT, True), (32, ml.METHOD_ZELDOVICH, False),
                                          (48, ml.METHOD_2LPT, True), (64, ml.METHOD_2LPT, True)])
def test_pipeline_fp64_vs_oracle(N, method, lin, table, spline):
    """64^3 / L = 256 / seed 42 / z = 31 / 32 linear shells is the reference CPU configuration."""
    L = 256.0 * N / 64
    bins = 32 if N == 64 else 12
    cfg = ml.ic_config(N, N, L, 42, table, method=method, pk_bins=bins, pk_linear=lin, precision=ml.FP64)
    out = ml.ic_pipeline_run(cfg, spline, want_pos=True)
    ref = oracle.ic_pipeline(oracle.ic_params(N, N, L, 42, table, lpt_order=2 if method == ml.METHOD_2LPT else 1,
                                              pk_bins=bins, pk_linear=lin), want=("pos", "pk"))
    assert np.array_equal(out["pk_obs"], ref["pk_obs"])
    ok = ref["pk_obs"] > 0
    assert np.abs(out["pk_p"][ok] / ref["pk_p"][ok] - 1).max() < 1e-9
    assert np.abs(out["pk_k"][ok] / ref["pk_k"][ok] - 1).max() < 1e-12
    assert np.abs(_wrapdiff(out["pos"], ref["pos"], L)).max() < 1e-4


@pytest.mark.parametrize("method", [ml.METHOD_2LPT, ml.METHOD_ZELDOVICH])
def test_large_displacements_take_the_global_gather(method, table, spline):
    """z = 0 in a 64 Mpc/h box of 1 Mpc/h cells: displacements of several cells, so most particles
    leave the lattice deposit's staged tiles and gather from global memory; positions and P(k)
    still equal the oracle's"""
    N, L = 64, 64.0
    cfg = ml.ic_config(N, N, L, 5, table, method=method, pk_bins=16, pk_linear=True, precision=ml.FP64, z_ini=0.0)
    out = ml.ic_pipeline_run(cfg, spline, want_pos=True)
    ref = oracle.ic_pipeline(oracle.ic_params(N, N, L, 5, table, lpt_order=2 if method == ml.METHOD_2LPT else 1,
                                              pk_bins=16, pk_linear=True, z_ini=0.0), want=("pos", "pk"))
    lattice = (np.indices((N, N, N)).reshape(3, -1).T + 0.0) * (L / N)
    disp = np.abs(_wrapdiff(ref["pos"], lattice, L)) / (L / N)
    print(f"displacements: rms {np.sqrt(np.mean(disp ** 2)):.2f} cells, beyond half a cell: {np.mean(disp.max(axis=1) > 0.5):.2f}")
    assert np.mean(disp.max(axis=1) > 0.5) > 0.3
    assert np.abs(_wrapdiff(out["pos"], ref["pos"], L)).max() < 1e-4
    assert np.array_equal(out["pk_obs"], ref["pk_obs"])
    ok = ref["pk_obs"] > 0
    assert np.abs(out["pk_p"][ok] / ref["pk_p"][ok] - 1).max() < 1e-8


def test_pipeline_ma_fp64_vs_oracle(table, spline):
    N, L = 32, 128.0
    cfg = ml.ic_config(N, N, L, 42, table, method=ml.METHOD_MONGE_AMPERE, pk_bins=12, pk_linear=True,
                       precision=ml.FP64, ma_cycles=3)
    out = ml.ic_pipeline_run(cfg, spline, want_pos=True)
    ref = oracle.ic_pipeline(oracle.ic_params(N, N, L, 42, table, ma_cycles=3, pk_bins=12, pk_linear=True),
                             want=("pos", "pk"))
    assert out["ma_iterations"] == 3
    ok = ref["pk_obs"] > 0
    assert np.abs(out["pk_p"][ok] / ref["pk_p"][ok] - 1).max() < 1e-9
    assert np.abs(_wrapdiff(out["pos"], ref["pos"], L)).max() < 1e-4


@pytest.mark.parametrize("N,L,seed,bins", [(128, 250.0, 7, 64), (256, 500.0, 7, 128)])
def test_precision_study_fp32_vs_fp64(N, L, seed, bins, table, spline):
    """FP32 pipeline against the FP64 GPU path: P(k) per bin within 1e-4, displacement rms
    relative error within 1e-5 (256^3, L = 500, seed 7, 128 shells is the precision-study config)."""
    c64 = ml.ic_config(N, N, L, seed, table, pk_bins=bins, pk_linear=True, precision=ml.FP64)
    c32 = ml.ic_config(N, N, L, seed, table, pk_bins=bins, pk_linear=True, precision=ml.FP32)
    o64 = ml.ic_pipeline_run(c64, spline, want_pos=True)
    o32 = ml.ic_pipeline_run(c32, spline, want_pos=True)
    assert np.array_equal(o32["pk_obs"], o64["pk_obs"])
    ok = o64["pk_obs"] > 0
    perbin = np.abs(o32["pk_p"][ok] / o64["pk_p"][ok] - 1)
    assert perbin.max() < 1e-4, perbin.max()
    # displacement = lattice - position (mod L)
    M = N
    q = (np.indices((M, M, M)).reshape(3, -1).T * np.float32(L / M)).astype(np.float64)
    d64 = _wrapdiff(q, o64["pos"], L)
    d32 = _wrapdiff(q, o32["pos"], L)
    rms = np.sqrt(np.mean((d32 - d64) ** 2)) / np.sqrt(np.mean(d64 ** 2))
    assert rms < 1e-5, rms


def test_async_submissions_match_synchronous_runs(table, spline):
    """ic_pipeline_submit: three ICs in flight in a row (positions into pinned and pageable host
    buffers) give the positions of ic_pipeline_run bit for bit and its P(k) to the tolerance of the
    floating-point atomics in the CIC flush and the P(k) sums"""
    torch = pytest.importorskip("torch")
    N, L, bins = 64, 256.0, 32
    seeds = [11, 12, 13]
    refs = [ml.ic_pipeline_run(ml.ic_config(N, N, L, s, table, pk_bins=bins), spline, want_pos=True) for s in seeds]
    keep = []
    for i, s in enumerate(seeds):
        k, p, o = np.zeros(bins), np.zeros(bins), np.zeros(bins, np.int64)
        if i == 1:
            pos_t = torch.zeros((N ** 3, 3), dtype=torch.float32, pin_memory=True)
            pos, ptr = pos_t, ctypes.cast(pos_t.data_ptr(), ctypes.POINTER(ctypes.c_float))
        else:
            pos = np.zeros((N ** 3, 3), np.float32)
            ptr = pos.ctypes.data_as(ctypes.POINTER(ctypes.c_float))
        res = ml.ICResult(k.ctypes.data_as(ctypes.POINTER(ctypes.c_double)),
                          p.ctypes.data_as(ctypes.POINTER(ctypes.c_double)),
                          o.ctypes.data_as(ctypes.POINTER(ctypes.c_long)), ptr, 0, 0.0)
        cfg = ml.ic_config(N, N, L, s, table, pk_bins=bins)
        ml.ic_pipeline_submit(cfg, spline, res)
        keep.append((k, p, o, pos, res, cfg))
    ml.ic_pipeline_wait()
    for (k, p, o, pos, res, cfg), ref in zip(keep, refs):
        got = pos.numpy() if hasattr(pos, "numpy") else pos
        assert np.array_equal(got, ref["pos"])
        assert np.array_equal(o, ref["pk_obs"])
        assert np.allclose(k, ref["pk_k"], rtol=1e-12, equal_nan=True)
        assert np.allclose(p, ref["pk_p"], rtol=1e-5, equal_nan=True)


@pytest.mark.parametrize("N,M,method", [(32, 32, ml.METHOD_2LPT), (32, 32, ml.METHOD_ZELDOVICH),
                                        (48, 48, ml.METHOD_2LPT), (32, 16, ml.METHOD_2LPT)])
def test_velocities_fp64_vs_oracle(N, M, method, table, spline):
    """particle velocities (src/mitos.c:425-490, :865-908): the velocity transfer function t_cdm,
    2LPT with the reference's velocity factors (Zel'dovich otherwise), the TSC gather at the unwrapped
    positions; the lattice-aligned deposit (M = N) and the general one (M != N)"""
    L = 4.0 * N
    iv = table.index_of("t_cdm")
    cfg = ml.ic_config(N, M, L, 42, table, method=method, pk_bins=12, precision=ml.FP64, index_vel=iv)
    out = ml.ic_pipeline_run(cfg, spline, want_pos=True, want_vel=True)
    ref = oracle.ic_pipeline(oracle.ic_params(N, M, L, 42, table, lpt_order=2 if method == ml.METHOD_2LPT else 1,
                                              pk_bins=12, index_vel=iv), want=("pos", "vel", "pk"))
    err = rel_err(out["vel"], ref["vel"])
    print(f"N={N} M={M} method={method}: velocity rel err {err:.3e}, max abs "
          f"{np.abs(out['vel'] - ref['vel']).max():.3e} of rms {np.sqrt(np.mean(ref['vel'] ** 2)):.3e}")
    assert np.abs(_wrapdiff(out["pos"], ref["pos"], L)).max() < 1e-4
    # same arithmetic: bit-identical except where a float position rounded differently (measured
    # 0 at 32^3, 7e-10 at 48^3)
    assert err < 1e-8, err


def test_velocities_large_displacements(table, spline):
    """z = 0 in 1 Mpc/h cells: the velocity gather's particles leave its staged tiles and read global
    memory; still the oracle's velocities"""
    N, L = 64, 64.0
    iv = table.index_of("t_cdm")
    cfg = ml.ic_config(N, N, L, 5, table, pk_bins=12, precision=ml.FP64, index_vel=iv, z_ini=0.0)
    out = ml.ic_pipeline_run(cfg, spline, want_vel=True)
    ref = oracle.ic_pipeline(oracle.ic_params(N, N, L, 5, table, pk_bins=12, index_vel=iv, z_ini=0.0),
                             want=("vel", "pk"))
    assert rel_err(out["vel"], ref["vel"]) < 1e-8


def test_velocities_256_fp32_vs_fp64(table, spline):
    """the 256^3 test configuration (L = 500, seed 7): FP32 velocities (tiled gather) against FP64"""
    N, L = 256, 500.0
    o = {}
    for prec in (ml.FP32, ml.FP64):
        cfg = ml.ic_config(N, N, L, 7, table, pk_bins=16, precision=prec)
        o[prec] = ml.ic_pipeline_run(cfg, spline, want_vel=True)["vel"]
    err = rel_err(o[ml.FP32], o[ml.FP64])
    print(f"velocities FP32 vs FP64 at 256^3: rel err {err:.3e}")
    assert err < 2e-5


def test_velocities_leave_positions_and_pk_unchanged(table, spline):
    N, L = 64, 256.0
    cfg = ml.ic_config(N, N, L, 9, table, pk_bins=16, precision=ml.FP32)
    a = ml.ic_pipeline_run(cfg, spline, want_pos=True)
    b = ml.ic_pipeline_run(cfg, spline, want_pos=True, want_vel=True)
    assert np.array_equal(a["pos"], b["pos"])
    assert np.array_equal(a["pk_obs"], b["pk_obs"])
    assert np.allclose(a["pk_p"], b["pk_p"], rtol=1e-5, equal_nan=True)
    assert np.all(np.isfinite(b["vel"])) and np.abs(b["vel"]).max() > 0
    bad = ml.ic_config(N, N, L, 9, table, pk_bins=16, precision=ml.FP32, index_vel=7)
    with pytest.raises(ml.MitosError):
        ml.ic_pipeline_run(bad, spline, want_vel=True)


def test_velocities_fp32_vs_fp64(table, spline):
    N, L = 128, 250.0
    o = {}
    for prec in (ml.FP32, ml.FP64):
        cfg = ml.ic_config(N, N, L, 7, table, pk_bins=16, precision=prec)
        o[prec] = ml.ic_pipeline_run(cfg, spline, want_vel=True)["vel"]
    err = rel_err(o[ml.FP32], o[ml.FP64])
    print(f"velocities FP32 vs FP64 at 128^3: rel err {err:.3e}")
    assert err < 2e-5, err  # measured 3.6e-6


def test_precision_study_displacement_orders(table, spline):
    """the 256^3 precision study (box 500 Mpc/h, seed 7): the first- and second-order displacement
    grids (gradients of phi_1 = -delta/k^2 and of the 2LPT potential phi_2, each with the TSC
    window undone) from the FP32 entry points against the FP64 ones, rms relative error <= 1e-5
    for each order"""
    from mitos_gb300 import study
    d64 = study.displacement_orders(256, 500.0, 7, table, spline, ml.FP64)
    d32 = study.displacement_orders(256, 500.0, 7, table, spline, ml.FP32)
    e1 = study.rms_rel(d32[1], d64[1])
    e2 = study.rms_rel(d32[2], d64[2])
    print(f"256^3 displacement rms relative error FP32 vs FP64: 1st order {e1:.2e}, 2nd order {e2:.2e}")
    assert np.sqrt(np.mean(d64[2][0] ** 2)) > 0
    assert e1 < 1e-5 and e2 < 1e-5, (e1, e2)
