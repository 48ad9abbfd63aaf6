"""generate_ngeniclike_grf (src/grf_ngeniclike.c): the oracle's structure, the library's host
RANLUX stream against the oracle's, and the GPU field against the oracle.  Parity with libgsl's
ranlxd1 is unpinned (GSL is absent); these tests pin the GPU to the oracle restatement."""
import ctypes

import numpy as np
import pytest

import oracle
import mitos_gb300.lib as ml


def test_ranlxd1_stream_statistics_and_seeds():
    u = oracle.ranlxd1_uniforms(12345, 120000)
    assert np.all((u >= 0) & (u < 1))
    assert abs(u.mean() - 0.5) < 4e-3 and abs(u.var() - 1 / 12) < 2e-3
    # 48-bit values: every uniform is a multiple of 2^-48
    assert np.all(np.floor(u * 2.0 ** 48) == u * 2.0 ** 48)
    # lag-1 correlation small; seed 0 is seed 1 (the default seed)
    assert abs(np.corrcoef(u[:-1], u[1:])[0, 1]) < 1e-2
    assert np.array_equal(oracle.ranlxd1_uniforms(0, 50), oracle.ranlxd1_uniforms(1, 50))
    assert not np.array_equal(oracle.ranlxd1_uniforms(2, 50), oracle.ranlxd1_uniforms(1, 50))


def test_library_host_generator_matches_oracle():
    for seed in (1, 7, 2147483647, 123456789):
        assert np.array_equal(ml.ranlxd1_uniforms(seed, 1000), oracle.ranlxd1_uniforms(seed, 1000))


def test_seed_table_fill_covers_every_column():
    for N in (8, 16, 32):
        t = oracle.ngenic_seedtable(N, 42)
        assert np.count_nonzero(t) == N * N  # each entry written once by the mirrored fill (:71-88)


def test_oracle_field_structure():
    N, L = 16, 100.0
    f = oracle.ngeniclike_grf(N, L, 7)
    assert not f[N // 2].any() and not f[:, N // 2].any() and not f[..., N // 2].any() and f[0, 0, 0] == 0
    fac = L ** 1.5
    # kz = 0 plane: f(-x, -y) = conj f(x, y) where the reference fills pairs
    for i in range(1, N // 2):
        for j in range(N):
            if j == N // 2:
                continue
            assert f[N - i, (N - j) % N, 0] == np.conj(f[i, j, 0])
    for j in range(1, N // 2):
        assert f[0, N - j, 0] == np.conj(f[0, j, 0])
    a2 = np.abs(f[:, :, 1:N // 2]) ** 2 / fac ** 2
    a2 = a2[a2 > 0]
    assert abs(a2.mean() - 1.0) < 0.1  # -ln U is exponential with mean 1


@pytest.mark.gpu
@pytest.mark.parametrize("N", [16, 32, 48])
def test_gpu_field_matches_oracle(N):
    L = 2.0 * N
    ref = oracle.ngeniclike_grf(N, L, 99)
    g = ml.alloc_local_grid(N, L, ml.FP64)
    ml.generate_ngeniclike_grf_dg(g, 99)
    got = ml.get_fbox(g)
    # identical uniforms; the GPU's log / sincos against the host libm: a few ulp
    assert np.array_equal(got == 0, ref == 0)
    assert np.abs(got - ref).max() <= 1e-13 * np.abs(ref).max()
    g32 = ml.alloc_local_grid(N, L, ml.FP32)
    ml.generate_ngeniclike_grf_dg(g32, 99)
    assert np.abs(ml.get_fbox(g32) - ref).max() <= 2e-6 * np.abs(ref).max()
    for x in (g, g32):
        ml.free_local_grid(x)


@pytest.mark.gpu
def test_gpu_field_slab_rows_match_full_field():
    """NX / X0 slabs (the reference's per-rank loop :101-105) give the rows of the full field"""
    N, L = 32, 64.0
    ref = oracle.ngeniclike_grf(N, L, 5)
    H = N // 2 + 1
    for X0, NX in ((0, 8), (8, 8), (20, 12)):
        g = ml.alloc_local_grid(N, L, ml.FP64)
        g.NX, g.X0 = NX, X0
        ml.generate_ngeniclike_grf_dg(g, 5)
        buf = np.zeros(N * N * H * 2)  # dg_copy_to_host copies the allocation (local_size)
        ml.load().dg_copy_to_host(ctypes.byref(g), 0, buf.ctypes.data_as(ctypes.c_void_p))
        b = buf.reshape(N, N, H, 2)[:NX]
        got = b[..., 0] + 1j * b[..., 1]
        assert np.abs(got - ref[X0:X0 + NX]).max() <= 1e-13 * np.abs(ref).max()
        g.NX, g.X0 = N, 0
        ml.free_local_grid(g)
