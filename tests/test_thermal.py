"""Thermal motion of a particle species (src/random.c:52-289, src/mitos.c:910-1064 without Firebolt).

CPU: the oracle's sampler and thermal loop against the reference build and the golden vectors, and the
library's host-side sampler (thermal_sampler_init) against the oracle.  GPU (marked): the kernel through
the C ABI against the oracle, the FP32 build against FP64, the stream position it leaves, the struct
particle stride, device buffers, and the pipeline's thermal stage against the oracle pipeline."""
import os

import numpy as np
import pytest

import oracle
import mitos_gb300.lib as ml

GOLDEN = os.path.join(os.path.dirname(__file__), "golden")
T_NU = 1.9517578 * 8.617333262e-5  # relic neutrino temperature today, eV
CASES = ((ml.FERMION, T_NU), (ml.BOSON, T_NU), (ml.FERMION, 0.25))
C_KMS = 299792.458


def _needs_ref():
    if oracle.ref_lib() is None:
        pytest.skip("reference build absent (no reference tree on this machine)")


# ---- CPU ------------------------------------------------------------------------------------------
@pytest.mark.parametrize("kind,T", CASES)
def test_oracle_sampler_pinned_to_reference(kind, T):
    _needs_ref()
    a, b = oracle.sampler_table(kind, T), oracle.ref_sampler_table(kind, T)
    assert np.array_equal(a["pieces"], b["pieces"])
    assert np.array_equal(a["table"], b["table"])
    assert a["norm"] == b["norm"]
    for seed, skip in ((42, 0), (7, 1000), (1001, 12345)):
        st = oracle.rng_state(seed, skip)
        assert np.array_equal(oracle.sampler_draws(kind, T, st, 20000), oracle.ref_sampler_draws(kind, T, st, 20000))
    vel = np.random.default_rng(kind).standard_normal((3000, 3)).astype(np.float32)
    st = oracle.rng_state(3, 77)
    assert np.array_equal(oracle.thermal(kind, T, 0.06, 1 / 32.0, C_KMS, st, vel),
                          oracle.ref_thermal(kind, T, 0.06, 1 / 32.0, C_KMS, st, vel))


def test_oracle_thermal_golden():
    g = np.load(os.path.join(GOLDEN, "thermal.npz"))
    for kind, T in CASES:
        name = f"k{kind}_T{T:.6e}"
        tab = oracle.sampler_table(kind, T)
        assert np.array_equal(tab["pieces"], g[name + "_pieces"])
        assert np.array_equal(tab["table"], g[name + "_table"])
        st = g[name + "_state"]
        assert np.array_equal(oracle.sampler_draws(kind, T, st, 2048), g[name + "_draws"])
        assert np.array_equal(oracle.thermal(kind, T, 0.06, 1 / 32.0, C_KMS, st, g[name + "_vel_in"]),
                              g[name + "_vel_out"])


def test_sampler_moments():
    """Fermi-Dirac <p> = 3.1514 kT, Bose-Einstein 2.7012 kT; the reference draw (which evaluates the
    cubic of the piece left of u, beyond its end) stays within 1% of them"""
    st = oracle.rng_state(11, 0)
    for kind, mean in ((ml.FERMION, 3.15137), (ml.BOSON, 2.70118)):
        d = oracle.sampler_draws(kind, 1.0, st, 400000)
        assert d.min() > 0 and d.max() <= 15.0 * 1.01
        assert abs(d.mean() / mean - 1) < 0.01, d.mean()


def _reference_pick(Fr, r, table, w):
    """samplerCustom's piece choice (src/random.c:264-281), restated literally in Python doubles"""
    u = float(np.uint64(w).astype(np.float64)) / 18446744073709551616.0  # (double)UINT64_MAX = 2^64
    t = int(np.floor(u * 1000))
    idx = int(table[t if t < 1000 else 999])
    rmax, pick = 0.0, idx
    for i in range(idx, len(Fr)):
        if Fr[i] < u and r[i] > rmax:
            rmax, pick = r[i], i
        else:
            break
    return pick


@pytest.mark.parametrize("kind", [ml.FERMION, ml.BOSON])
def test_kernel_piece_choice_is_the_reference_scan(kind):
    """the kernel's integer piece choice (thresholds on w and a bucket table; evaluated on the host
    from the same table image) equals the reference scan on u = w / 2^64 for random draws and for
    the draws around every threshold, search-table step and bucket edge, and the extremes"""
    import ctypes
    from fractions import Fraction
    s = ml.thermal_sampler(kind, T_NU)
    try:
        rows, table = ml.sampler_rows(s), ml.sampler_index(s)
        Fr, r = rows[:, 3], rows[:, 1]
        ws = set(int(x) for x in np.random.default_rng(kind).integers(0, 2 ** 63, 40000, dtype=np.uint64))
        ws |= set(int(x) * 2 + 1 for x in np.random.default_rng(kind + 5).integers(0, 2 ** 63, 20000, dtype=np.uint64))
        edges = [int(Fraction(f) * 2 ** 64) for f in Fr] + [int(Fraction(i, 1000) * 2 ** 64) for i in range(1, 1001)]
        for e in edges:
            ws.update(w for w in range(e - 2100, e + 2100, 37) if 0 <= w < 2 ** 64)
            ws.update(w for w in (e - 1, e, e + 1) if 0 <= w < 2 ** 64)
        # the exact threshold of each piece: the largest w with (double)w / 2^64 <= Fr, and the next w
        for f in Fr:
            lo, hi = 0, 2 ** 64 - 1
            if float(np.uint64(hi).astype(np.float64)) / 2.0 ** 64 <= f:
                continue
            while hi - lo > 1:
                mid = (lo + hi) // 2
                if float(np.uint64(mid).astype(np.float64)) / 2.0 ** 64 <= f:
                    lo = mid
                else:
                    hi = mid
            ws.update((lo, lo + 1))
        for b in range(1024):
            ws.update(w for w in ((b << 54) - 1, b << 54, (b << 54) + 1) if 0 <= w < 2 ** 64)
        ws.update((0, 1, 2 ** 64 - 1, 2 ** 64 - 1024, 2 ** 64 - 1025, 2 ** 64 - 2048))
        w = np.array(sorted(ws), np.uint64)
        got = np.zeros(w.size, np.int32)
        assert ml.load().mitos_thermal_pieces(ctypes.byref(s), w.ctypes.data_as(ctypes.POINTER(ctypes.c_uint64)),
                                             ctypes.c_long(w.size),
                                             got.ctypes.data_as(ctypes.POINTER(ctypes.c_int))) == 0
        want = np.array([_reference_pick(Fr, r, table, int(x)) for x in w])
        bad = np.nonzero(got != want)[0]
        assert bad.size == 0, (w[bad[:5]], got[bad[:5]], want[bad[:5]])
    finally:
        ml.thermal_sampler_free(s)


@pytest.mark.parametrize("kind,T", CASES)
def test_library_sampler_matches_oracle(kind, T):
    """thermal_sampler_init is host code (no GPU): its pieces, search table and norm equal the oracle's"""
    s = ml.thermal_sampler(kind, T)
    try:
        o = oracle.sampler_table(kind, T)
        assert np.array_equal(ml.sampler_rows(s), o["pieces"])
        assert np.array_equal(ml.sampler_index(s), o["table"])
        assert s.norm == o["norm"] and s.I_max == 1000
    finally:
        ml.thermal_sampler_free(s)
    with pytest.raises(ml.MitosError):
        ml.thermal_sampler(3, T)


def test_oracle_pipeline_thermal_pinned_to_reference(table):
    """the thermal stage of the oracle pipeline, from the stream the white noise leaves (src/mitos.c:148,
    :220, :935), equals the reference functions driven in the reference order"""
    _needs_ref()
    iv = table.index_of("t_cdm")
    for kind, off in ((ml.FERMION, 0), (ml.BOSON, 5000)):
        prm = oracle.ic_params(16, 16, 64.0, 42, table, pk_bins=8, index_vel=iv, thermal=kind,
                               thermal_T_eV=T_NU, thermal_M_eV=0.06, speed_of_light=C_KMS,
                               thermal_draw_offset=off)
        a = oracle.ic_pipeline(prm, want=("vel", "pk"))
        b = oracle.ref_ic_pipeline(prm, want=("vel", "pk"))
        assert np.array_equal(a["vel"], b["vel"])
        plain = oracle.ic_pipeline(dict(prm, thermal=0), want=("vel", "pk"))
        assert not np.array_equal(a["vel"], plain["vel"])


# ---- GPU ------------------------------------------------------------------------------------------
def _ulps(a, b):
    a = np.asarray(a, np.float32).view(np.int32).astype(np.int64)
    b = np.asarray(b, np.float32).view(np.int32).astype(np.int64)
    return np.abs(a - b)


def _gpu_thermal(kind, T, st, vel, prec, M_eV=0.06, a_ini=1 / 32.0, stride=3, n=None, offset=0):
    s = ml.thermal_sampler(kind, T)
    ml.set_precision(prec)
    try:
        return ml.thermal_velocities(s, st, vel, M_eV, a_ini, C_KMS, stride=stride, n=n, offset=offset)
    finally:
        ml.set_precision(ml.FP64)
        ml.thermal_sampler_free(s)


@pytest.mark.gpu
@pytest.mark.parametrize("kind,T", CASES)
def test_thermal_fp64_vs_oracle(kind, T):
    """FP64: the reference's draws, pieces and operations; only GPU log/cos/hypot may move a float
    result by one unit in the last place"""
    n = 200003
    vel = np.random.default_rng(1).standard_normal((n, 3)).astype(np.float32) * 100
    st = oracle.rng_state(42, 999)
    ref = oracle.thermal(kind, T, 0.06, 1 / 32.0, C_KMS, st, vel)
    out = vel.copy()
    st2 = _gpu_thermal(kind, T, st, out, ml.FP64)
    u = _ulps(out, ref)
    print(f"kind {kind} T {T:.3e}: {np.count_nonzero(u)} of {u.size} floats differ, max {u.max()} ulp")
    assert u.max() <= 1 and np.count_nonzero(u) <= u.size * 1e-4
    # the stream continues after 7 n draws, as the reference loop leaves it
    assert np.array_equal(st2, oracle.rng_state(42, 999 + 7 * n))


@pytest.mark.gpu
def test_thermal_fp32_vs_fp64():
    n = 1 << 20
    vel = np.zeros((n, 3), np.float32)
    st = oracle.rng_state(8, 0)
    a, b = vel.copy(), vel.copy()
    _gpu_thermal(ml.FERMION, T_NU, st, a, ml.FP32)
    _gpu_thermal(ml.FERMION, T_NU, st, b, ml.FP64)
    speed = np.linalg.norm(b, axis=1)
    err = np.abs(a - b).max(axis=1) / speed
    print(f"FP32 vs FP64 thermal velocities: max rel {err.max():.3e}, mean {err.mean():.3e}")
    # measured 6.6e-6 (mean 7.5e-8) on 2^20 particles
    assert err.max() < 1e-5


@pytest.mark.gpu
def test_thermal_struct_particle_stride_and_device_buffer():
    """stride 10 floats (struct particle: X Y Z v_X v_Y v_Z mass pad id) leaves the other fields alone;
    a device buffer gives the same result as a host one"""
    import torch
    n = 50000
    parts = np.random.default_rng(2).standard_normal((n, 10)).astype(np.float32)
    packed = np.ascontiguousarray(parts[:, 3:6])
    st = oracle.rng_state(5, 17)
    want = parts.copy()
    want[:, 3:6] = oracle.thermal(ml.FERMION, T_NU, 0.06, 1 / 32.0, C_KMS, st, packed)
    got = parts.copy()
    _gpu_thermal(ml.FERMION, T_NU, st, got, ml.FP64, stride=10, n=n, offset=3)
    assert np.array_equal(np.delete(got, [3, 4, 5], axis=1), np.delete(parts, [3, 4, 5], axis=1))
    assert _ulps(got[:, 3:6], want[:, 3:6]).max() <= 1
    dev = torch.from_numpy(packed.copy()).cuda()
    _gpu_thermal(ml.FERMION, T_NU, st, dev, ml.FP64)
    host = packed.copy()
    _gpu_thermal(ml.FERMION, T_NU, st, host, ml.FP64)
    assert np.array_equal(dev.cpu().numpy(), host)


@pytest.mark.gpu
def test_thermal_full_size_thread_boundaries():
    """512^3 particles (R = 432 a thread): particles at and around thread-run boundaries, and a spread
    of others, equal the oracle started from the jumped stream; isotropy of the increments"""
    n = 1 << 27
    vel = np.zeros((n, 3), np.float32)
    st = oracle.rng_state(1000, 0)
    _gpu_thermal(ml.FERMION, T_NU, st, vel, ml.FP64)
    R = -(-n // (152 * 2048))
    picks = sorted({0, 1, R - 1, R, R + 1, 2 * R, 5000 * R - 1, 5000 * R, n - R, n - 2, n - 1,
                    *np.random.default_rng(0).integers(0, n, 40).tolist()})
    for i in picks:
        s = st.copy()
        ml.load().mitos_rng_jump(s.ctypes.data_as(ml.ctypes.POINTER(ml.ctypes.c_uint64)),
                                 ml.ctypes.c_ulonglong(7 * i))
        ref = oracle.thermal(ml.FERMION, T_NU, 0.06, 1 / 32.0, C_KMS, s, np.zeros((1, 3), np.float32))
        assert _ulps(vel[i], ref[0]).max() <= 1, i
    v64 = vel.astype(np.float64)
    mean = v64.mean(axis=0)
    speed = np.sqrt((v64 ** 2).sum(axis=1))
    sigma = np.sqrt((speed ** 2).mean() / 3)  # per component
    assert np.abs(mean).max() < 6 * sigma / np.sqrt(n)
    # <p> = 3.1514 kT for the Fermi-Dirac momentum, speed = p / (a M) c
    assert abs(speed.mean() / (3.15137 * T_NU * 32 / 0.06 * C_KMS) - 1) < 0.01


@pytest.mark.gpu
def test_thermal_fp32_large_ragged():
    """FP32 on 2^25 + 12345 particles (400 MB of velocities, above L2; the last thread's run is
    short): sampled particles against the oracle started from the jumped stream"""
    import torch
    n = (1 << 25) + 12345
    dev = torch.zeros((n, 3), dtype=torch.float32, device="cuda")
    st = oracle.rng_state(77, 0)
    _gpu_thermal(ml.FERMION, T_NU, st, dev, ml.FP32)
    vel = dev.cpu().numpy()
    R = -(-n // (152 * 2048))
    picks = sorted({0, R - 1, R, n - 1, n - R, *np.random.default_rng(3).integers(0, n, 30).tolist()})
    for i in picks:
        s = st.copy()
        ml.load().mitos_rng_jump(s.ctypes.data_as(ml.ctypes.POINTER(ml.ctypes.c_uint64)),
                                 ml.ctypes.c_ulonglong(7 * i))
        ref = oracle.thermal(ml.FERMION, T_NU, 0.06, 1 / 32.0, C_KMS, s, np.zeros((1, 3), np.float32))[0]
        assert np.abs(vel[i] - ref).max() <= 1e-5 * np.linalg.norm(ref), i


@pytest.mark.gpu
@pytest.mark.parametrize("prec,M", [(ml.FP64, 32), (ml.FP32, 32), (ml.FP64, 16)])
def test_pipeline_thermal_vs_oracle(prec, M, table, spline):
    """the pipeline's thermal stage: the species' draws start after the white noise's (and after
    thermal_draw_offset more), on top of the gathered velocities; M = N (lattice-aligned deposit and
    gather) and M < N (the general ones)"""
    N, L = 32, 128.0
    iv = table.index_of("t_cdm")
    for kind, off in ((ml.FERMION, 0), (ml.BOSON, 4242)):
        cfg = ml.ic_config(N, M, L, 42, table, pk_bins=12, precision=prec, index_vel=iv, thermal=kind,
                           thermal_M_eV=0.06, thermal_T_eV=T_NU, speed_of_light=C_KMS, thermal_draw_offset=off)
        out = ml.ic_pipeline_run(cfg, spline, want_vel=True)
        ref = oracle.ic_pipeline(oracle.ic_params(N, M, L, 42, table, pk_bins=12, index_vel=iv, thermal=kind,
                                                  thermal_T_eV=T_NU, thermal_M_eV=0.06, speed_of_light=C_KMS,
                                                  thermal_draw_offset=off), want=("vel", "pk"))
        if prec == ml.FP64:
            u = _ulps(out["vel"], ref["vel"])
            assert u.max() <= 1 and np.count_nonzero(u) <= u.size * 1e-3, (u.max(), np.count_nonzero(u))
        else:
            err = np.abs(out["vel"] - ref["vel"]).max() / np.abs(ref["vel"]).max()
            assert err < 2e-5, err
    bad = ml.ic_config(N, N, L, 42, table, pk_bins=12, precision=prec, index_vel=iv, thermal=ml.FERMION,
                       thermal_M_eV=0.0, thermal_T_eV=T_NU, speed_of_light=C_KMS)
    with pytest.raises(ml.MitosError):
        ml.ic_pipeline_run(bad, spline, want_vel=True)


@pytest.mark.gpu
def test_async_submissions_with_thermal(table, spline):
    """ic_pipeline_submit with velocities and thermal motion (three ICs in flight, one without thermal
    motion): the velocities of ic_pipeline_run bit for bit"""
    import ctypes
    N, L, bins = 32, 128.0, 12
    iv = table.index_of("t_cdm")
    kinds = [ml.FERMION, 0, ml.BOSON]

    def cfg(kind, seed):
        return ml.ic_config(N, N, L, seed, table, pk_bins=bins, index_vel=iv, thermal=kind, thermal_M_eV=0.06,
                            thermal_T_eV=T_NU, speed_of_light=C_KMS)

    refs = [ml.ic_pipeline_run(cfg(k, 20 + i), spline, want_vel=True) for i, k in enumerate(kinds)]
    keep = []
    for i, k in enumerate(kinds):
        kk, p, o = np.zeros(bins), np.zeros(bins), np.zeros(bins, np.int64)
        vel = np.zeros((N ** 3, 3), np.float32)
        res = ml.ICResult(kk.ctypes.data_as(ml._dp), p.ctypes.data_as(ml._dp), o.ctypes.data_as(ml._lp), None, 0, 0.0,
                          vel.ctypes.data_as(ml._fp))
        c = cfg(k, 20 + i)
        ml.ic_pipeline_submit(c, spline, res)
        keep.append((vel, p, res, c))
    ml.ic_pipeline_wait()
    for (vel, p, res, c), ref in zip(keep, refs):
        assert np.array_equal(vel, ref["vel"])
        assert np.allclose(p, ref["pk_p"], rtol=1e-5, equal_nan=True)
    assert not np.array_equal(refs[0]["vel"], refs[1]["vel"])


@pytest.mark.gpu
@pytest.mark.parametrize("prec", [ml.FP64, ml.FP32])
def test_thermal_invalid_momentum_reports_status_8(prec):
    """a sampler whose cubic is negative everywhere: the reference exits (src/mitos.c:939-942), the
    library returns status 8 and leaves the context usable"""
    import ctypes
    iv = (ml.Interval * 1)()
    iv[0].l, iv[0].r, iv[0].Fl, iv[0].Fr, iv[0].a0 = 1.0, 2.0, 0.0, 1.0, -1.0
    index = (ctypes.c_double * 1)(0.0)
    s = ml.Sampler(1.0, 1.0, 2.0, None, None, iv, 1, 1, index)
    vel = np.zeros((1000, 3), np.float32)
    ml.set_precision(prec)
    try:
        with pytest.raises(ml.MitosError) as e:
            ml.thermal_velocities(s, oracle.rng_state(1, 0), vel, 0.06, 1 / 32.0, C_KMS)
        assert e.value.code == 8
    finally:
        ml.set_precision(ml.FP64)
    # a sampler whose search table is not initSampler's is refused before any launch (status 3)
    index[0] = 5.0
    with pytest.raises(ml.MitosError) as e:
        ml.thermal_velocities(s, oracle.rng_state(1, 0), vel, 0.06, 1 / 32.0, C_KMS)
    assert e.value.code == 3
    out = vel.copy()
    st = ml.thermal_sampler(ml.FERMION, T_NU)
    try:
        ml.thermal_velocities(st, oracle.rng_state(1, 0), out, 0.06, 1 / 32.0, C_KMS)
    finally:
        ml.thermal_sampler_free(st)
    assert np.all(np.isfinite(out)) and np.abs(out).max() > 0


@pytest.mark.gpu
@pytest.mark.parametrize("n", [1, 7, 129])
def test_thermal_few_particles(n):
    """fewer particles than one block's threads (one particle a thread)"""
    vel = np.random.default_rng(n).standard_normal((n, 3)).astype(np.float32)
    st = oracle.rng_state(99, 5)
    ref = oracle.thermal(ml.BOSON, T_NU, 0.06, 1 / 32.0, C_KMS, st, vel)
    out = vel.copy()
    st2 = _gpu_thermal(ml.BOSON, T_NU, st, out, ml.FP64)
    assert _ulps(out, ref).max() <= 1
    assert np.array_equal(st2, oracle.rng_state(99, 5 + 7 * n))


@pytest.mark.gpu
def test_release_all_then_rerun(table, spline):
    """mitos_release_all frees the cached jump and sampler tables with the workspaces; the next calls
    rebuild them and give the same results"""
    N, L = 32, 128.0
    iv = table.index_of("t_cdm")
    cfg = ml.ic_config(N, N, L, 42, table, pk_bins=12, precision=ml.FP32, index_vel=iv, thermal=ml.FERMION,
                       thermal_M_eV=0.06, thermal_T_eV=T_NU, speed_of_light=C_KMS)
    a = ml.ic_pipeline_run(cfg, spline, want_vel=True)
    v = np.zeros((5000, 3), np.float32)
    st = oracle.rng_state(3, 0)
    va = v.copy()
    _gpu_thermal(ml.FERMION, T_NU, st, va, ml.FP32)
    assert ml.load().mitos_release_all() == 0
    b = ml.ic_pipeline_run(cfg, spline, want_vel=True)
    vb = v.copy()
    _gpu_thermal(ml.FERMION, T_NU, st, vb, ml.FP32)
    assert np.array_equal(a["vel"], b["vel"]) and np.array_equal(va, vb)


def test_reference_built_sampler_is_accepted():
    """the drop-in case: a struct sampler filled from the reference's own initSampler (its pieces in
    its order, its search table) is taken by the library, with the same piece choice as the literal
    samplerCustom scan (CPU: the kernel's table, evaluated on the host)"""
    import ctypes
    _needs_ref()
    for kind, T in CASES:
        ref = oracle.ref_sampler_table(kind, T)
        rows, table = ref["pieces"], ref["table"]
        n = rows.shape[0]
        iv = (ml.Interval * n)()
        for j in range(n):
            iv[j].id = j
            iv[j].l, iv[j].r, iv[j].Fl, iv[j].Fr, iv[j].a0, iv[j].a1, iv[j].a2, iv[j].a3 = rows[j]
            iv[j].nid = j + 1
        index = (ctypes.c_double * 1000)(*[float(t) for t in table])
        s = ml.Sampler(ref["norm"], 1e-10 * T, 15.0 * T, None, None, iv, n, 1000, index)
        w = np.random.default_rng(kind).integers(0, 2 ** 63, 20000, dtype=np.uint64) * np.uint64(2)
        got = np.zeros(w.size, np.int32)
        assert ml.load().mitos_thermal_pieces(ctypes.byref(s), w.ctypes.data_as(ctypes.POINTER(ctypes.c_uint64)),
                                             ctypes.c_long(w.size),
                                             got.ctypes.data_as(ctypes.POINTER(ctypes.c_int))) == 0
        want = np.array([_reference_pick(rows[:, 3], rows[:, 1], table, int(x)) for x in w])
        assert np.array_equal(got, want), (kind, T)


def test_thermal_arguments_checked_before_any_launch():
    """empty and invalid inputs are settled on the host (no GPU): n = 0 leaves the stream where it is;
    a bad stride, mass or scale factor is status 1; pieces out of order are status 3"""
    import ctypes
    s = ml.thermal_sampler(ml.FERMION, T_NU)
    try:
        st = oracle.rng_state(1, 0)
        v = np.zeros((10, 3), np.float32)
        assert np.array_equal(ml.thermal_velocities(s, st, v, 0.06, 1 / 32.0, C_KMS, n=0), st)
        for args, kw in (((0.06, 1 / 32.0), dict(stride=2)), ((0.0, 1 / 32.0), {}), ((0.06, -1.0), {})):
            with pytest.raises(ml.MitosError) as e:
                ml.thermal_velocities(s, st, v, *args, C_KMS, **kw)
            assert e.value.code == 1
        n = s.intervalNum
        rev = (ml.Interval * n)(*[s.intervals[n - 1 - j] for j in range(n)])
        bad = ml.Sampler(s.norm, s.xl, s.xr, None, None, rev, n, s.I_max, s.index)
        with pytest.raises(ml.MitosError) as e:
            ml.thermal_velocities(bad, st, v, 0.06, 1 / 32.0, C_KMS)
        assert e.value.code == 3
        out = np.zeros(4, np.int32)
        assert ml.load().mitos_thermal_pieces(ctypes.byref(bad), np.zeros(4, np.uint64).ctypes.data_as(
            ctypes.POINTER(ctypes.c_uint64)), ctypes.c_long(4), out.ctypes.data_as(ctypes.POINTER(ctypes.c_int))) == 3
    finally:
        ml.thermal_sampler_free(s)
