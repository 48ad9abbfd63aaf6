"""GPU parity of two reference entry points that the pipeline does not reach:
generatePerturbationGrid (src/generate_grids.c:28-67) and calc_cross_powerspec_float_mpi on x-slabs
(src/calc_powerspec.c:152-217), both through the C ABI against the oracle."""
import ctypes

import numpy as np
import pytest

import oracle
import mitos_gb300.lib as ml
from conftest import rel_err

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("prec,tol", [(ml.FP64, 1e-13), (ml.FP32, 3e-6)])
@pytest.mark.parametrize("rescale", [1.0, 0.37])
def test_generate_perturbation_grid(table, spline, prec, tol, rescale):
    """delta(x) = c2r(grf(k) T(k, tau_src) rescale): the transfer function at the source time, the
    growth-factor rescaling when it is not 1, the c2r; the white-noise grid is left unchanged"""
    N, L, z = 32, 128.0, 31.0
    osp = oracle.Spline(table)
    tp = oracle.transfer_params(osp, z)
    lt = oracle.lib().orc_log_tau_at_redshift(ctypes.byref(osp.s), ctypes.c_double(z))
    cosmo = ml.Cosmology(0.67, table.n_s, table.A_s, table.k_pivot, z, lt, 0.0, z, lt)
    src = oracle.grf(N, L, 5)
    grf = ml.alloc_local_grid(N, L, prec)
    grid = ml.alloc_local_grid(N, L, prec)
    ml.set_fbox(grf, src)
    ml.generatePerturbationGrid(cosmo, spline, grf, grid, "d_cdm", rescale)
    assert grid.momentum_space == b"\x00"
    got = ml.get_box(grid)[..., :N]
    refk = oracle.apply_kernel(N, L, src, "transfer", tp)
    if rescale != 1.0:
        refk = oracle.apply_kernel(N, L, refk, "constant", rescale)
    ref = oracle.fft_c2r(N, L, refk)[..., :N]
    assert np.abs(ref).max() > 0
    assert rel_err(got, ref) < tol
    kept = ml.get_fbox(grf)
    if prec == ml.FP64:
        assert np.array_equal(kept, src)
    else:
        assert np.array_equal(kept, src.astype(np.complex64))
    # an unknown transfer-function title is the reference's error 1 (src/generate_grids.c:43-46)
    with pytest.raises(ml.MitosError) as e:
        ml.generatePerturbationGrid(cosmo, spline, grf, grid, "no_such_function", rescale)
    assert e.value.code == 1
    ml.free_local_grid(grf)
    ml.free_local_grid(grid)


def _float_mpi(N, X0, NX, L, a, b, bins, on_device):
    lib = ml.load()
    k, p, o = np.zeros(bins), np.zeros(bins), np.zeros(bins, np.int64)
    keep = []
    ptrs = []
    for arr in (a, b):
        arr = np.ascontiguousarray(arr, np.complex64)
        keep.append(arr)
        if on_device:
            import torch
            t = torch.from_numpy(arr.view(np.float32).copy()).cuda()
            keep.append(t)
            ptrs.append(ctypes.c_void_p(t.data_ptr()))
        else:
            ptrs.append(arr.ctypes.data_as(ctypes.c_void_p))
    lib.calc_cross_powerspec_float_mpi(ctypes.c_long(N), ctypes.c_long(X0), ctypes.c_long(NX), ctypes.c_double(L),
                                       ptrs[0], ptrs[1], bins, k.ctypes.data_as(ml._dp), p.ctypes.data_as(ml._dp),
                                       o.ctypes.data_as(ml._lp))
    return k, p, o


@pytest.mark.parametrize("N,X0,NX", [(32, 0, 32), (32, 0, 8), (32, 5, 11), (32, 24, 8), (48, 17, 1), (64, 31, 2)])
@pytest.mark.parametrize("on_device", [False, True])
def test_cross_powerspec_float_mpi_slabs(N, X0, NX, on_device):
    """each rank's slab of the reference's float spectrum: the slab's modes only, binned as the
    reference bins them; host and device slabs"""
    if on_device:
        pytest.importorskip("torch")
    L, bins = 3.0 * N, 12
    r = np.random.default_rng(N * 1000 + X0 * 10 + NX)
    sh = (NX, N, N // 2 + 1)
    a = (r.standard_normal(sh) + 1j * r.standard_normal(sh)).astype(np.complex64)
    b = (r.standard_normal(sh) + 1j * r.standard_normal(sh)).astype(np.complex64)
    k, p, o = _float_mpi(N, X0, NX, L, a, b, bins, on_device)
    rk, rp, ro = oracle.powerspec_float_slab(N, X0, NX, L, a, b, bins)
    assert np.array_equal(o, ro)
    ok = ro > 0
    assert ok.any()
    assert np.abs(p[ok] - rp[ok]).max() <= 1e-12 * np.abs(rp[ok]).max()
    assert rel_err(k[ok], rk[ok]) < 1e-14
    # the slabs of all ranks together give the whole grid's counts
    if (N, X0, NX) == (32, 0, 8):
        tot = np.zeros(bins, np.int64)
        for x0 in range(0, N, NX):
            tot += _float_mpi(N, x0, NX, L, a, b, bins, on_device)[2]
        full = oracle.powerspec_float_slab(N, 0, N, L, np.zeros((N, N, N // 2 + 1), np.complex64),
                                           np.zeros((N, N, N // 2 + 1), np.complex64), bins)[2]
        assert np.array_equal(tot, full)
