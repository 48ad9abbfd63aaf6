"""Parity at the benchmark's full size (512^3, box 1000 Mpc/h) through properties that do not need the
oracle to run at that size: the r2c/c2r round trip, noise columns against the reference stream
started from their jumped states, and the FP32 IC against the FP64 IC (P(k) per bin, positions)."""
import ctypes

import numpy as np
import pytest

import oracle
import mitos_gb300.lib as ml
from conftest import rel_err

pytestmark = pytest.mark.gpu

N, L = 512, 1000.0


@pytest.mark.parametrize("prec,tol", [(ml.FP32, 2e-6), (ml.FP64, 1e-14)])
def test_fft_roundtrip_512(prec, tol):
    g = ml.alloc_local_grid(N, L, prec)
    try:
        box = np.random.default_rng(1).standard_normal((N, N, N + 2)).astype(np.float32 if prec == ml.FP32 else np.float64)
        ml.set_box(g, box)
        ml.fft_r2c_dg(g)
        ml.fft_c2r_dg(g)
        back = ml.get_box(g)
        err = rel_err(back[:, :, :N], box[:, :, :N])
        print(f"round trip rel err {err:.2e}")
        assert err < tol
    finally:
        ml.free_local_grid(g)


def test_noise_512_columns_match_stream():
    """FP64 noise at 512^3: sampled columns (the first, the last, Nyquist rows, random ones) equal
    src/grf.c:47-63's sequential stream, started from each column's draw offset"""
    g = ml.alloc_local_grid(N, L, ml.FP64)
    try:
        ml.generate_complex_grf(g, ml.rng_init(42))
        got = ml.get_fbox(g)
    finally:
        ml.free_local_grid(g)
    H = N // 2 + 1
    factor = np.sqrt(L ** 3 / 2)
    s0 = np.array(list(ml.rng_init(42).s), np.uint64)
    cols = sorted({0, 1, N - 1, N * N - 1, (N // 2) * N, (N // 2) * N + N // 2,
                   *np.random.default_rng(2).integers(0, N * N, 12).tolist()})
    lib = oracle.lib()
    for c in cols:
        st = (ctypes.c_uint64 * 4)()
        ml.load().mitos_noise_column_state(N, ctypes.c_long(c), (ctypes.c_uint64 * 4)(*[int(v) for v in s0]), st)
        s = np.array(list(st), np.uint64)
        ref = np.zeros(H, np.complex128)
        for z in range(H):
            if c == 0 and z == 0:
                continue  # the DC mode takes no draws
            a = lib.orc_sample_norm(oracle.P(s, oracle._up)) * factor
            b = lib.orc_sample_norm(oracle.P(s, oracle._up)) * factor
            ref[z] = a + 1j * b
        x, y = divmod(c, N)
        assert rel_err(got[x, y], ref) < 1e-14, c


def test_ic_512_fp32_vs_fp64(table, spline):
    """the benchmark IC in FP32 against FP64: P(k) within 1e-4 per bin (the 256^3 criterion, here at
    512^3) with identical counts; positions within two float ulps at the box size"""
    out = {}
    for prec in (ml.FP32, ml.FP64):
        cfg = ml.ic_config(N, N, L, 42, table, method=ml.METHOD_2LPT, pk_bins=128, pk_linear=True, precision=prec)
        out[prec] = ml.ic_pipeline_run(cfg, spline, want_pos=True)
    a, b = out[ml.FP32], out[ml.FP64]
    assert np.array_equal(a["pk_obs"], b["pk_obs"])
    ok = b["pk_obs"] > 0
    rel = np.abs(a["pk_p"][ok] / b["pk_p"][ok] - 1)
    d = np.asarray(a["pos"], np.float64) - np.asarray(b["pos"], np.float64)
    d -= L * np.round(d / L)
    print(f"P(k) FP32 vs FP64 max rel {rel.max():.2e}; positions max {np.abs(d).max():.2e}, rms {np.sqrt(np.mean(d ** 2)):.2e}")
    assert rel.max() < 1e-4
    assert np.abs(d).max() < 2 * np.spacing(np.float32(L))
