"""CPU tests of the oracle: pinned against the reference build (when present) and the committed
golden vectors, plus the assertions of the reference's own test-suite restated."""
import os

import numpy as np
import pytest

import oracle
from conftest import rel_err

GOLDEN = os.path.join(os.path.dirname(__file__), "golden")


def test_golden_draws():
    g = np.load(os.path.join(GOLDEN, "xoshiro_draws.npz"))
    for key in g.files:
        seed = int(key.split("_")[1])
        assert np.array_equal(oracle.draws(seed, len(g[key])), g[key]), key


def test_golden_norms():
    g = np.load(os.path.join(GOLDEN, "sample_norm.npz"))
    for key in g.files:
        seed = int(key.split("_")[1])
        assert np.array_equal(oracle.norms(seed, len(g[key])), g[key]), key


def test_golden_grf():
    g = np.load(os.path.join(GOLDEN, "grf.npz"))
    for key in g.files:
        _, N, seed = key.split("_")
        N, seed = int(N), int(seed)
        got = oracle.grf(N, 256.0 * N / 64, seed)
        assert np.array_equal(got, g[key]), key


def test_golden_pipeline(table):
    g = np.load(os.path.join(GOLDEN, "pipeline.npz"))
    for name in sorted({k.rsplit("_", 1)[0] for k in g.files}):
        N, seed, lpt, ma, lin = [int(v) for v in name.split("_")[1:]]
        prm = oracle.ic_params(N, N, 256.0 * N / 64, seed, table, lpt_order=lpt, ma_cycles=ma,
                               pk_bins=8, pk_linear=bool(lin))
        out = oracle.ic_pipeline(prm, want=("pos", "pk"))
        assert np.array_equal(out["pos"], g[name + "_pos"]), name
        assert np.array_equal(out["pk_obs"], g[name + "_obs"]), name
        assert np.array_equal(out["pk_p"], g[name + "_pk"], equal_nan=True), name


def test_golden_bispectrum():
    """the oracle's calc_bispectrum against the reference build's outputs (carried to machines
    without the reference tree)"""
    g = np.load(os.path.join(GOLDEN, "bispectrum.npz"))
    for name in sorted({k.rsplit("_", 1)[0] for k in g.files}):
        N, btype, vol = [int(v) for v in name.split("_")[1:]]
        L = 4.0 * N
        f = oracle.apply_kernel(N, L, oracle.grf(N, L, 3), "gaussian", np.sqrt(1 / 0.02))
        r = oracle.bispectrum(N, L, None if vol else f, 8, 8, volume_mode=bool(vol), btype=btype,
                              theta=4 * np.pi / 3, k3=0.4)
        for key in ("k1", "k2", "k3", "B"):
            assert np.array_equal(r[key], g[f"{name}_{key}"]), (name, key)


def test_golden_stages(table):
    """every stage grid of the oracle's 2LPT and Monge-Ampere ICs at 16^3 against the reference
    build's (noise, delta(k), phi(k), displacement grids, CIC overdensity)"""
    g = np.load(os.path.join(GOLDEN, "stages.npz"))
    for lpt, ma in ((2, 0), (2, 3)):
        prm = oracle.ic_params(16, 16, 64.0, 42, table, lpt_order=lpt, ma_cycles=ma, pk_bins=8)
        out = oracle.ic_pipeline(prm, want=("grf", "delta_k", "phi_k", "disp", "rho", "pk"))
        for key in ("grf", "delta_k", "phi_k", "disp0", "disp1", "disp2", "rho"):
            assert np.array_equal(out[key], g[f"s_{lpt}_{ma}_{key}"]), (lpt, ma, key)


def test_golden_velocities(table):
    """the oracle's particle velocities against the reference build's (16^3, 2LPT and Zel'dovich)"""
    g = np.load(os.path.join(GOLDEN, "velocity.npz"))
    for lpt in (2, 1):
        prm = oracle.ic_params(16, 16, 64.0, 42, table, lpt_order=lpt, pk_bins=8, index_vel=table.index_of("t_cdm"))
        assert np.array_equal(oracle.ic_pipeline(prm, want=("vel", "pk"))["vel"], g[f"v_16_{lpt}"]), lpt


@pytest.mark.skipif(oracle.ref_lib() is None, reason="reference build not present here")
@pytest.mark.parametrize("N,lin,lpt,ma", [(16, True, 2, 0), (32, False, 2, 0), (16, True, 1, 0),
                                          (16, False, 2, 2)])
def test_pin_against_reference_build(table, N, lin, lpt, ma):
    """every intermediate and the velocities (the velocity transfer function t_cdm) of the oracle
    equal the reference's own functions bit for bit"""
    prm = oracle.ic_params(N, N, 256.0 * N / 64, 42, table, lpt_order=lpt, ma_cycles=ma,
                           pk_bins=8, pk_linear=lin, index_vel=table.index_of("t_cdm"))
    want = ("grf", "delta_k", "phi_k", "disp", "pos", "rho", "pk", "vel")
    a = oracle.ic_pipeline(prm, want)
    b = oracle.ref_ic_pipeline(prm, want)
    assert np.abs(a["vel"]).max() > 0
    for key in ["grf", "delta_k", "phi_k", "disp0", "disp1", "disp2", "pos", "rho", "pk_k",
                "pk_p", "pk_obs", "vel"]:
        assert np.array_equal(a[key], b[key], equal_nan=True), key


@pytest.mark.skipif(oracle.ref_lib() is None, reason="reference build not present here")
def test_pin_rng_against_reference_build():
    for seed in (42, 7, 1000):
        assert np.array_equal(oracle.draws(seed, 5000), oracle.ref_draws(seed, 5000))
        assert np.array_equal(oracle.norms(seed, 5000), oracle.ref_norms(seed, 5000))
    for N in (16, 32):
        assert np.array_equal(oracle.grf(N, 64.0, 3), oracle.ref_grf(N, 64.0, 3))


def test_sample_norm_moments():
    """tests/test_random.c:64-65: 1e6 draws, |mean| < 1e-2 and |sd - 1| < 1e-2."""
    x = oracle.norms(100, 1_000_000)
    assert abs(x.mean()) < 1e-2
    assert abs(x.std(ddof=1) - 1.0) < 1e-2


def _smooth_grf(N, L, seed):
    f = oracle.grf(N, L, seed)
    return oracle.apply_kernel(N, L, f, "gaussian", np.sqrt(1 / 0.02))


def test_fft_roundtrip():
    """tests/test_fft.c:69: c2r then r2c returns the input within 1e-10."""
    N, L = 64, 128.0
    f = _smooth_grf(N, L, 100)
    box = oracle.fft_c2r(N, L, f.copy())
    back = oracle.fft_r2c(N, L, box)
    assert np.abs(back - f).max() < 1e-10


def test_fft_matches_numpy():
    N = 24
    x = np.random.default_rng(0).standard_normal((N, N, N))
    got = oracle.fft_r2c(N, float(N), x)  # boxlen = N: normalisation V / N^3 = 1
    assert rel_err(got, np.fft.rfftn(x)) < 1e-13


def _fd(f, h, axis, order):
    r = lambda s: np.roll(f, -s, axis=axis)
    if order == 1:
        return (r(-2) / 12 - 8 * r(-1) / 12 + 8 * r(1) / 12 - r(2) / 12) / h
    return (-r(-2) + 16 * r(-1) - 30 * f + 16 * r(1) - r(2)) / 12 / h / h


def test_poisson_derivatives():
    """tests/test_poisson.c:119-121,157-159,187: spectral derivatives of the potential agree
    with 5-point finite differences, and the sum of second derivatives returns the field."""
    N, L = 64, 256.0
    f = _smooth_grf(N, L, 100)
    rho = oracle.fft_c2r(N, L, f.copy())[..., :N]
    fk = oracle.fft_r2c(N, L, rho)
    phik = oracle.apply_kernel(N, L, fk, "inv_poisson")
    phi = oracle.fft_c2r(N, L, phik.copy())[..., :N]
    h = L / N
    lap = 0
    for ax, name in enumerate(("dx", "dy", "dz")):
        d1k = oracle.apply_kernel(N, L, phik, name)
        d1 = oracle.fft_c2r(N, L, d1k.copy())[..., :N]
        assert np.abs(d1 - _fd(phi, h, ax, 1)).max() < 1e-3
        d2 = oracle.fft_c2r(N, L, oracle.apply_kernel(N, L, d1k, name))[..., :N]
        assert np.abs(d2 - _fd(phi, h, ax, 2)).max() < 1e-4
        lap = lap + d2
    assert np.abs(lap - rho).max() < 1e-10


def test_powerspec_recovers_input():
    """tests/test_calc_powerspec.c:86-98: binned power of a filtered GRF follows the filter."""
    N, L, bins = 64, 256.0, 50
    sig = lambda k: np.exp(-k * k / 0.02)
    f = oracle.grf(N, L, 100)
    f = oracle.apply_kernel(N, L, f, "gaussian", np.sqrt(1 / 0.02))
    k, p, o = oracle.powerspec(N, L, f, f, bins, linear=False)
    for i in range(bins):
        if o[i] == 0:
            continue
        exp = sig(k[i]) ** 2
        if exp < 1e-50:
            continue
        if exp < 1e-3:
            err, tol = abs(np.log(p[i]) - np.log(exp)) / abs(np.log(exp)), 0.1
        else:
            err, tol = abs(p[i] - exp) / exp, 0.7
        assert err <= tol, (i, k[i], p[i], exp)


def test_linear_bins_integer_exact():
    for N, bins in ((64, 32), (256, 128), (96, 32)):
        for n2 in range(1, 3 * (N // 2) ** 2 + 1, 97):
            b = oracle.lib().orc_lin_bin(N, bins, n2)
            # shell b holds modes with b * (N/2)/bins <= |n| < (b+1) * (N/2)/bins
            w = (N / 2) / bins
            assert b * w <= np.sqrt(n2) + 1e-12 and np.sqrt(n2) < (b + 1) * w + 1e-12


@pytest.mark.skipif(oracle.ref_lib() is None, reason="reference build not present here")
@pytest.mark.parametrize("btype,vol", [(0, False), (1, False), (0, True)])
def test_pin_bispectrum_against_reference_build(btype, vol):
    """orc_bispectrum equals the reference's calc_bispectrum (src/calc_powerspec.c:295-508) bit for
    bit: equilateral (type 0, theta = 4 pi / 3), fixed k3 (type 1) and the bin volumes"""
    N, L = 16, 64.0
    f = _smooth_grf(N, L, 5)
    args = dict(bins=8, bins3=8, volume_mode=vol, btype=btype, theta=4 * np.pi / 3, k3=0.3)
    a = oracle.bispectrum(N, L, None if vol else f, **args)
    b = oracle.ref_bispectrum(N, L, None if vol else f, **args)
    assert np.any(a["B"] != 0)
    for key in ("k1", "k2", "k3", "B"):
        assert np.array_equal(a[key], b[key]), key


@pytest.mark.skipif(oracle.ref_lib() is None, reason="reference build not present here")
@pytest.mark.parametrize("X0,NX", [(0, 32), (0, 8), (5, 11), (24, 8)])
def test_pin_float_slab_spectrum_against_reference_build(X0, NX):
    """orc_powerspec_float_slab equals the reference's calc_cross_powerspec_float_mpi
    (src/calc_powerspec.c:152-217, one rank) bit for bit on x-slabs of a 32^3 grid"""
    N, L, bins = 32, 100.0, 12
    r = np.random.default_rng(X0 + 100 * NX)
    sh = (N, N, N // 2 + 1)
    a = (r.standard_normal(sh) + 1j * r.standard_normal(sh)).astype(np.complex64)[X0:X0 + NX]
    b = (r.standard_normal(sh) + 1j * r.standard_normal(sh)).astype(np.complex64)[X0:X0 + NX]
    got = oracle.powerspec_float_slab(N, X0, NX, L, a, b, bins)
    ref = oracle.ref_powerspec_float_slab(N, X0, NX, L, a, b, bins)
    assert got[2].sum() > 0
    for x, y in zip(got, ref):
        assert np.array_equal(x, y, equal_nan=True)
