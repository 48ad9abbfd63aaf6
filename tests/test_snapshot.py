"""The snapshot and field-file datasets made on the device: the particle arrays src/mitos.c:1106-1117
hands to H5Dwrite (Coordinates, Velocities, Masses, ParticleIDs) and the /Field/Field dataset of
writeFieldFile_dg (src/output_mpi.c:52-141).  The HDF5 calls themselves stay with the caller."""
import numpy as np
import pytest

import oracle
import mitos_gb300.lib as ml

pytestmark = pytest.mark.gpu


def _wrapdiff(a, b, L):
    d = np.asarray(a, np.float64) - np.asarray(b, np.float64)
    return d - L * np.round(d / L)


@pytest.mark.parametrize("prec,M", [(ml.FP64, 32), (ml.FP32, 32), (ml.FP32, 16)])
def test_snapshot_datasets(prec, M, table, spline):
    """Coordinates / Velocities are the float particle fields as double (wrapped positions, velocities
    with thermal motion), Masses the float mass as double, ParticleIDs the row-major lattice index plus
    FirstID (src/particle.c:114-121); the positions also match the oracle's"""
    N, L = 32, 128.0
    iv = table.index_of("t_cdm")
    cfg = ml.ic_config(N, M, L, 42, table, pk_bins=12, precision=prec, index_vel=iv, thermal=ml.FERMION,
                       thermal_M_eV=0.06, thermal_T_eV=1.68e-4, speed_of_light=299792.458,
                       particle_mass=3.3e-3, id_first_particle=1000)
    out = ml.ic_pipeline_run(cfg, spline, want_pos=True, want_vel=True, want_snapshot=True)
    n = M ** 3
    assert np.array_equal(out["coords"], out["pos"].astype(np.float64))
    assert np.array_equal(out["vels"], out["vel"].astype(np.float64))
    assert np.array_equal(out["masses"], np.full(n, np.float32(3.3e-3), np.float64))
    assert np.array_equal(out["ids"], np.arange(n, dtype=np.int64) + 1000)
    assert out["coords"].min() >= 0 and out["coords"].max() < L
    ref = oracle.ic_pipeline(oracle.ic_params(N, M, L, 42, table, pk_bins=12), want=("pos",))
    assert np.abs(_wrapdiff(out["coords"], ref["pos"], L)).max() < 1e-4
    # without velocities requested the snapshot has no Velocities array; the rest is the same
    cfg0 = ml.ic_config(N, M, L, 42, table, pk_bins=12, precision=prec, index_vel=-1, particle_mass=3.3e-3,
                        id_first_particle=1000)
    o0 = ml.ic_pipeline_run(cfg0, spline, want_snapshot=True)
    assert "vels" not in o0
    assert np.array_equal(o0["coords"], out["coords"]) and np.array_equal(o0["ids"], out["ids"])


@pytest.mark.parametrize("prec", [ml.FP64, ml.FP32])
def test_field_dataset(prec):
    """/Field/Field: N x N x (N + 2) doubles, padding included; refused in momentum space"""
    N, L = 32, 64.0
    dg = ml.alloc_local_grid(N, L, prec)
    try:
        box = np.random.default_rng(4).standard_normal((N, N, N + 2))
        ml.set_box(dg, box)
        got = ml.field_to_host(dg)
        want = box.astype(np.float32).astype(np.float64) if prec == ml.FP32 else box
        assert got.shape == (N, N, N + 2) and np.array_equal(got, want)
        ml.fft_r2c_dg(dg)
        with pytest.raises(ml.MitosError) as e:
            ml.field_to_host(dg)
        assert e.value.code == 2
    finally:
        ml.free_local_grid(dg)

