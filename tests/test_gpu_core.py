"""GPU parity of the reference entry points against the oracle (FP64 tight, FP32 loose)."""
import ctypes
import math

import numpy as np
import pytest

import oracle
import mitos_gb300.lib as ml
from oracle import crcheck
from conftest import rel_err

pytestmark = pytest.mark.gpu

SIZES = [16, 32, 48, 64, 96, 128]


def _rand_c(N, seed):
    r = np.random.default_rng(seed)
    return r.standard_normal((N, N, N // 2 + 1)) + 1j * r.standard_normal((N, N, N // 2 + 1))


def _gaussian_draws(N, seed):
    """the draw pairs (A, B) of every Gaussian of an N^3 noise grid, in the reference's order
    (src/grf.c:47-63: modes x -> y -> z, DC skipped, real part first)"""
    n = N * N * (N // 2 + 1) - 1
    d = oracle.draws(seed, 4 * n)
    return d[0::2], d[1::2]


def _check_noise_fp64(N, seed, L):
    """the GPU's FP64 Gaussians equal the reference's (oracle, host libm) bit for bit, except where
    the host libm misrounded log or cos; there they are the exactly rounded values"""
    g = ml.alloc_local_grid(N, L, ml.FP64)
    st = ml.rng_init(seed)
    ml.generate_complex_grf(g, st)
    got = ml.get_fbox(g).view(np.float64).ravel()[2:]  # Gaussian i is float i after the DC mode
    ref = oracle.grf(N, L, seed, hermitian=False).view(np.float64).ravel()[2:]
    ml.free_local_grid(g)
    factor = math.sqrt(L ** 3 / 2)  # src/grf.c:33
    A, B = _gaussian_draws(N, seed)
    differ = np.nonzero(got != ref)[0]
    for i in differ:
        u, y = crcheck.sample_norm_parts(int(A[i]), int(B[i]))
        lu, cy = crcheck.exact_log(u), crcheck.exact_cos(y)
        assert math.log(u) != lu or math.cos(y) != cy, (N, seed, i)  # the host libm misrounded
        assert got[i] == math.sqrt(-2.0 * lu) * cy * factor, (N, seed, i)
    assert len(differ) < 0.005 * len(ref)
    return st, len(ref), len(differ)


@pytest.mark.parametrize("N,seed", [(16, 42), (32, 42), (48, 42), (64, 42)])
def test_noise_fp64_bit_exact(N, seed):
    """C1's noise (64^3, seed 42) and smaller grids"""
    st, n, nd = _check_noise_fp64(N, seed, 256.0 * N / 64)
    print(f"N={N} seed={seed}: {n} Gaussians, {n - nd} equal to the reference's, {nd} at libm misroundings")
    # the state advanced past every draw, as the sequential reference leaves it
    d = oracle.draws(seed, 4 * (N * N * (N // 2 + 1) - 1) + 1)
    from test_abi import _next
    assert _next(list(st.s)) == int(d[-1])


def test_noise_fp64_bit_exact_c2():
    """C2's noise: 256^3, seed 7, box 500 Mpc/h (16.9 million Gaussians)"""
    _, n, nd = _check_noise_fp64(256, 7, 500.0)
    print(f"N=256 seed=7: {n} Gaussians, {n - nd} equal to the reference's, {nd} at libm misroundings")


def test_noise_fp32_against_fp64_reference():
    """FP32 noise against float(reference): the fraction of equal floats and the largest error in
    float ulps (reported; the FP32 Box-Muller is a fast approximation, see rng.cuh)"""
    N, seed = 64, 42
    L = 256.0 * N / 64
    g = ml.alloc_local_grid(N, L, ml.FP32)
    ml.generate_complex_grf(g, ml.rng_init(seed))
    got = ml.get_fbox(g).view(np.float32).ravel()[2:]
    ml.free_local_grid(g)
    ref = oracle.grf(N, L, seed, hermitian=False).view(np.float64).ravel()[2:].astype(np.float32)
    u = crcheck.ulps(got, ref)
    frac = float(np.mean(got == ref))
    print(f"FP32 noise 64^3 seed 42: {frac:.4f} equal to float(reference), max {u.max():.0f} ulp, "
          f"99.9th percentile {np.percentile(u, 99.9):.1f} ulp")
    # __cosf's error is absolute (about 2^-21), so the ulp count grows without bound near the cosine's
    # zeros, where the Gaussian itself is near zero; the error against the largest value stays small
    assert frac > 0.1
    assert np.median(u) <= 8
    assert rel_err(got.astype(np.float64), ref.astype(np.float64)) < 2e-6


def test_noise_384_matches_stream():
    """a production-sized grid: 147456 column jumps from the block tables, every column checked
    (the odd ones separately, as a column-pairing mistake would show there)"""
    N, L = 384, 1536.0
    ref = oracle.grf(N, L, 11, hermitian=False)
    for prec, tol in ((ml.FP64, 1e-14), (ml.FP32, 2e-6)):
        g = ml.alloc_local_grid(N, L, prec)
        ml.generate_complex_grf(g, ml.rng_init(11))
        got = ml.get_fbox(g).astype(np.complex128)
        assert rel_err(got, ref) < tol, prec
        assert rel_err(got.reshape(N * N, -1)[1::2], ref.reshape(N * N, -1)[1::2]) < tol, prec
        ml.free_local_grid(g)


@pytest.mark.parametrize("N", [16, 64, 96])
def test_noise_fp32(N):
    L = 256.0 * N / 64
    g = ml.alloc_local_grid(N, L, ml.FP32)
    ml.generate_complex_grf(g, ml.rng_init(7))
    got = ml.get_fbox(g).astype(np.complex128)
    ref = oracle.grf(N, L, 7, hermitian=False)
    assert rel_err(got, ref) < 2e-6
    ml.free_local_grid(g)


@pytest.mark.parametrize("prec", [ml.FP64, ml.FP32])
def test_hermiticity(prec):
    N, L = 32, 64.0
    src = _rand_c(N, 1)
    g = ml.alloc_local_grid(N, L, prec)
    ml.set_fbox(g, src)
    ml.enforce_hermiticity(g)
    got = ml.get_fbox(g)
    buf = np.ascontiguousarray(np.stack([src.real, src.imag], -1))
    oracle.lib().orc_enforce_hermiticity(N, oracle.P(buf))
    ref = oracle.to_complex(buf)
    if prec == ml.FP64:
        assert np.array_equal(got, ref)
    else:
        assert np.array_equal(got, ref.astype(np.complex64))


@pytest.mark.parametrize("N", SIZES)
@pytest.mark.parametrize("prec", [ml.FP64, ml.FP32])
def test_fft_c2r_r2c(N, prec):
    L = 100.0 + N
    tol = 1e-13 if prec == ml.FP64 else 3e-6
    src = _rand_c(N, N)
    g = ml.alloc_local_grid(N, L, prec)
    ml.set_fbox(g, src)
    ml.fft_c2r_dg(g)
    got = ml.get_box(g)
    ref = oracle.fft_c2r(N, L, src.copy())
    assert rel_err(got[..., :N], ref[..., :N]) < tol
    assert np.all(got[..., N:] == 0)
    # r2c of a real field, input preserved
    real = np.random.default_rng(N + 1).standard_normal((N, N, N))
    ml.set_box(g, real)
    ml.fft_r2c_dg(g)
    gotk = ml.get_fbox(g)
    refk = oracle.fft_r2c(N, L, real)
    assert rel_err(gotk, refk) < tol
    assert rel_err(ml.get_box(g)[..., :N], real) == 0 or prec == ml.FP32
    ml.free_local_grid(g)


def _kernel_params(name, N, L, table, spline):
    if name in ("constant", "lowpass", "hipass", "gaussian"):
        return 0.5, 0.5
    if name == "tophat":
        return [0.1, 0.5], [0.1, 0.5]
    if name == "undo_Hermite_window":
        return ml.HermiteParams(3, N, L), oracle.HermiteParams(3, N, L)
    if name == "power_no_transfer":
        c = ml.Cosmology(0.67, table.n_s, table.A_s, table.k_pivot, 31, 0, 0, 31, 0)
        return c, oracle.OrcCosmo(table.A_s, table.n_s, table.k_pivot)
    if name == "transfer_function":
        osp = oracle.Spline(table)
        tp = oracle.transfer_params(osp, 31.0)
        mp = ml.SplineParams(ctypes.pointer(spline.sp), 0, tp.tau_index, tp.u_tau)
        _kernel_params.keep = osp
        return mp, tp
    return None, None


@pytest.mark.parametrize("name", ["constant", "lowpass", "hipass", "tophat", "gaussian", "inv_poisson",
                                  "dx", "dy", "dz", "power_no_transfer", "transfer_function",
                                  "undo_Hermite_window"])
def test_kernels_fp64(name, table, spline):
    N, L = 32, 128.0
    src = _rand_c(N, 3)
    g = ml.alloc_local_grid(N, L, ml.FP64)
    w = ml.alloc_local_grid(N, L, ml.FP64)
    ml.set_fbox(g, src)
    mp, op = _kernel_params(name, N, L, table, spline)
    assert ml.fft_apply_kernel_dg(w, g, name, mp) == 0
    got = ml.get_fbox(w)
    oname = {"transfer_function": "transfer", "undo_Hermite_window": "undo_hermite"}.get(name, name)
    ref = oracle.apply_kernel(N, L, src, oname, op)
    if name in ("constant", "inv_poisson", "dx", "dy", "dz", "lowpass", "hipass", "tophat", "transfer_function"):
        assert np.array_equal(got, ref), rel_err(got, ref)
    else:
        assert rel_err(got, ref) < 1e-14
    ml.free_local_grid(g)
    ml.free_local_grid(w)


@pytest.mark.parametrize("name", ["constant", "lowpass", "hipass", "tophat", "gaussian", "inv_poisson",
                                  "dx", "power_no_transfer", "transfer_function", "undo_Hermite_window"])
@pytest.mark.parametrize("N", [32, 96])
def test_kernels_fp32(name, N, table, spline):
    """FP32 grids: the k-only kernels from a table per |n|^2, the window undo from per-axis tables
    (a k-only factor evaluated at k = sqrt(n^2) dk): within FP32 rounding of the FP64 oracle"""
    L = 4.0 * N
    src = _rand_c(N, 3)
    g = ml.alloc_local_grid(N, L, ml.FP32)
    w = ml.alloc_local_grid(N, L, ml.FP32)
    ml.set_fbox(g, src)
    mp, op = _kernel_params(name, N, L, table, spline)
    assert ml.fft_apply_kernel_dg(w, g, name, mp) == 0
    got = ml.get_fbox(w)
    oname = {"transfer_function": "transfer", "undo_Hermite_window": "undo_hermite"}.get(name, name)
    ref = oracle.apply_kernel(N, L, src.astype(np.complex64).astype(complex), oname, op)
    assert np.abs(ref).max() > 0
    tol = 2e-7 if name in ("constant", "lowpass", "hipass", "tophat", "dx") else 1e-6
    assert rel_err(got, ref) < tol
    ml.free_local_grid(g)
    ml.free_local_grid(w)


def test_kernel_error_paths():
    g = ml.alloc_local_grid(16, 10.0, ml.FP64)
    w = ml.alloc_local_grid(32, 10.0, ml.FP64)
    assert ml.fft_apply_kernel_dg(g, g, "inv_poisson") == 2  # not in momentum space
    g.momentum_space = b"\x01"
    assert ml.fft_apply_kernel_dg(w, g, "inv_poisson") == 1  # shape mismatch
    bogus = ctypes.cast(ml.load().fft_r2c_dg, ctypes.c_void_p)
    assert ml.fft_apply_kernel_dg(g, g, bogus) == 3  # not a known kernel callback
    with pytest.raises(ml.MitosError) as e:
        ml.alloc_local_grid(20, 10.0)
    assert e.value.code == 3
    ml.free_local_grid(g)
    ml.free_local_grid(w)


def _solver_grids(N, L, prec, table):
    f = oracle.grf(N, L, 11)
    f = oracle.apply_kernel(N, L, f, "gaussian", 4.0 * L / N) * 1e-3
    dens = ml.alloc_local_grid(N, L, prec)
    ml.set_fbox(dens, f)
    ml.fft_c2r_dg(dens)
    ml.fft_r2c_dg(dens)
    return f, dens


@pytest.mark.parametrize("N", [32, 48])
def test_solve_2lpt_fp64(N, table):
    L = 4.0 * N
    f, dens = _solver_grids(N, L, ml.FP64, table)
    pot = ml.alloc_local_grid(N, L, ml.FP64)
    work = ml.alloc_local_grid(N, L, ml.FP64)
    ml.solve2LPT(pot, dens, work, 1.0, -3.0 / 7.0)
    got = ml.get_fbox(pot)
    a, b, c = [oracle.lib() and None] * 3
    og = [oracle.OrcGrid() for _ in range(3)] if hasattr(oracle, "OrcGrid") else None
    ref = oracle_2lpt(N, L, f)
    assert rel_err(got, ref) < 1e-11
    for g in (pot, work, dens):
        ml.free_local_grid(g)


def oracle_2lpt(N, L, fk, ma_cycles=0):
    """run orc_solve_2lpt / orc_solve_ma on the same density (momentum space after c2r, r2c)."""
    class OrcGrid(ctypes.Structure):
        _fields_ = [("N", ctypes.c_int), ("boxlen", ctypes.c_double), ("momentum_space", ctypes.c_int),
                    ("fbox", ctypes.POINTER(ctypes.c_double)), ("box", ctypes.POINTER(ctypes.c_double))]
    lib = oracle.lib()
    gs = [OrcGrid() for _ in range(3)]
    for g in gs:
        lib.orc_grid_alloc(ctypes.byref(g), N, ctypes.c_double(L))
    pot, dens, work = gs
    H = N // 2 + 1
    buf = np.ctypeslib.as_array(dens.fbox, shape=(N * N * H * 2,))
    buf[:] = np.stack([fk.real, fk.imag], -1).ravel()
    dens.momentum_space = 1
    lib.orc_grid_c2r(ctypes.byref(dens))
    lib.orc_grid_r2c(ctypes.byref(dens))
    if ma_cycles:
        eps = np.zeros(ma_cycles)
        rel = np.zeros(ma_cycles)
        lib.orc_solve_ma(ctypes.byref(pot), ctypes.byref(dens), ctypes.byref(work), ma_cycles,
                         oracle.P(eps), oracle.P(rel))
    else:
        lib.orc_solve_2lpt(ctypes.byref(pot), ctypes.byref(dens), ctypes.byref(work),
                           ctypes.c_double(1.0), ctypes.c_double(-3.0 / 7.0))
    out = np.ctypeslib.as_array(pot.fbox, shape=(N, N, H, 2)).copy()
    for g in gs:
        lib.orc_grid_free(ctypes.byref(g))
    res = out[..., 0] + 1j * out[..., 1]
    return (res, eps, rel) if ma_cycles else res


def test_solve_monge_ampere_fp64(table):
    N, L = 32, 128.0
    f, dens = _solver_grids(N, L, ml.FP64, table)
    pot = ml.alloc_local_grid(N, L, ml.FP64)
    work = ml.alloc_local_grid(N, L, ml.FP64)
    ml.solveMongeAmpere(pot, dens, work, 3)
    got = ml.get_fbox(pot)
    ref, eps, rel = oracle_2lpt(N, L, f, ma_cycles=3)
    assert rel_err(got, ref) < 1e-10
    geps, grel = ml.ma_history()
    assert np.allclose(geps, eps, rtol=1e-6)
    for g in (pot, work, dens):
        ml.free_local_grid(g)


def test_poisson_fp64():
    N, L = 32, 128.0
    real = np.random.default_rng(5).standard_normal((N, N, N))
    g = ml.alloc_local_grid(N, L, ml.FP64)
    ml.set_box(g, real)
    ml.solvePoisson_dg(g)
    got = ml.get_box(g)[..., :N]
    fk = oracle.fft_r2c(N, L, real)
    ref = oracle.fft_c2r(N, L, oracle.apply_kernel(N, L, fk, "inv_poisson"))[..., :N]
    assert rel_err(got, ref) < 1e-12
    ml.free_local_grid(g)


@pytest.mark.parametrize("prec", [ml.FP64, ml.FP32])
def test_calc_cross_powerspec(prec):
    N, L, bins = 64, 256.0, 20
    f1 = oracle.grf(N, L, 3)
    f2 = oracle.grf(N, L, 4)
    k, p, o = ml.calc_cross_powerspec(N, L, f1, f2, bins, precision=prec)
    rk, rp, ro = oracle.powerspec(N, L, f1, f2, bins, linear=False)
    assert np.array_equal(o, ro)
    ok = ro > 0
    tol = 1e-12 if prec == ml.FP64 else 1e-5
    assert np.abs(p[ok] - rp[ok]).max() <= tol * np.abs(rp[ok]).max()
    assert rel_err(k[ok], rk[ok]) < 1e-12


def test_cic_deposit_fp64():
    N, L, n = 32, 64.0, 5000
    pos = np.random.default_rng(9).uniform(-1, L + 1, (n, 3)).astype(np.float32)
    g = ml.alloc_local_grid(N, L, ml.FP64)
    tot = ml.cic_deposit_dg(g, pos, 2.5)
    got = ml.get_box(g)[..., :N]
    ref = np.zeros(N ** 3)
    wrapped = np.ascontiguousarray(pos)
    t2 = oracle.lib().orc_cic_deposit(ctypes.c_long(n), oracle.P(wrapped, oracle._fp), ctypes.c_double(2.5), N,
                                      ctypes.c_double(L), oracle.P(ref))
    assert abs(tot - t2) < 1e-9 * t2
    assert rel_err(got.ravel(), ref) < 1e-12
    ml.free_local_grid(g)
