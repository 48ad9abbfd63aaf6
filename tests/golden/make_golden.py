"""Generate the golden vectors in tests/golden/ from the reference's own code.

Runs the reference hot-path sources compiled by oracle/Makefile (`make -C oracle ref`,
needs the reference tree) through oracle.ref_* and stores small fixtures:
  xoshiro_draws.npz  rand_uint64 streams (include/random.h:27-33) for seeds 42, 7, 1000..1002
  sample_norm.npz    sampleNorm streams (src/random.c:34-49)
  grf.npz            generate_complex_grf + enforce_hermiticity at 16^3 and 32^3
  pipeline.npz       positions and P(k) of src/mitos.c + analyse/src/mitos_read.c at 16^3 / 32^3
  thermal.npz        initSampler pieces and search tables (src/random.c:87-209), samplerCustom
                     draws (:261-289) and the thermal-motion loop of src/mitos.c:928-1062
  bispectrum.npz     calc_bispectrum (src/calc_powerspec.c:295-508) of a 16^3 / 32^3 field, types 0
                     and 1, field and volume mode
  velocity.npz       particle velocities of src/mitos.c:425-490,865-908 (t_cdm) at 16^3, 2LPT and
                     Zel'dovich
  stages.npz         every stage grid of the 2LPT and Monge-Ampere (3 cycles) ICs at 16^3: noise,
                     delta(k), phi(k), the displacement grids and the CIC overdensity
Usage: python tests/golden/make_golden.py
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

import oracle  # noqa: E402
from mitos_gb300.perturb import load_table  # noqa: E402


def main():
    oracle.build(ref=True)
    assert oracle.ref_lib() is not None, "the reference build is required"
    np.savez_compressed(os.path.join(HERE, "xoshiro_draws.npz"),
                        **{f"seed_{s}": oracle.ref_draws(s, 4096) for s in (42, 7, 1000, 1001, 1002)})
    np.savez_compressed(os.path.join(HERE, "sample_norm.npz"),
                        **{f"seed_{s}": oracle.ref_norms(s, 4096) for s in (42, 7, 100)})
    np.savez_compressed(os.path.join(HERE, "grf.npz"),
                        **{f"grf_{N}_{s}": oracle.ref_grf(N, 256.0 * N / 64, s)
                           for N, s in ((16, 42), (32, 7))})
    table = load_table()
    fx = {}
    for N, seed, lpt, ma, lin in ((16, 42, 2, 0, 1), (32, 7, 2, 0, 0), (16, 42, 1, 0, 1),
                                  (16, 42, 2, 3, 1)):
        prm = oracle.ic_params(N, N, 256.0 * N / 64, seed, table, lpt_order=lpt, ma_cycles=ma,
                               pk_bins=8, pk_linear=bool(lin))
        out = oracle.ref_ic_pipeline(prm, want=("pos", "pk"))
        name = f"p_{N}_{seed}_{lpt}_{ma}_{lin}"
        fx[name + "_pos"] = out["pos"]
        fx[name + "_obs"] = out["pk_obs"]
        fx[name + "_pk"] = out["pk_p"]
    np.savez_compressed(os.path.join(HERE, "pipeline.npz"), **fx)
    thermal_fixture()
    bispectrum_fixture()
    velocity_fixture()
    stages_fixture()
    print("golden vectors written to", HERE)


# neutrino temperature today (1.9517578 K) in eV, and a heavier relic
THERMAL_CASES = ((1, 1.9517578 * 8.617333262e-5), (2, 1.9517578 * 8.617333262e-5), (1, 0.25))


def thermal_fixture():
    oracle.build(ref=True)
    fx = {}
    rng = np.random.default_rng(5)
    for kind, T in THERMAL_CASES:
        name = f"k{kind}_T{T:.6e}"
        tab = oracle.ref_sampler_table(kind, T)
        fx[name + "_pieces"] = tab["pieces"]
        fx[name + "_table"] = tab["table"]
        st = oracle.rng_state(42, 123)
        fx[name + "_state"] = st
        fx[name + "_draws"] = oracle.ref_sampler_draws(kind, T, st, 2048)
        vel = rng.standard_normal((512, 3)).astype(np.float32)
        fx[name + "_vel_in"] = vel
        fx[name + "_vel_out"] = oracle.ref_thermal(kind, T, 0.06, 1 / 32.0, 299792.458, st, vel)
    np.savez_compressed(os.path.join(HERE, "thermal.npz"), **fx)



BISPEC_CASES = ((16, 0, False), (16, 1, False), (32, 0, False), (16, 0, True))


def bispectrum_fixture():
    oracle.build(ref=True)
    fx = {}
    for N, btype, vol in BISPEC_CASES:
        L = 4.0 * N
        f = oracle.apply_kernel(N, L, oracle.grf(N, L, 3), "gaussian", np.sqrt(1 / 0.02))
        name = f"b_{N}_{btype}_{int(vol)}"
        r = oracle.ref_bispectrum(N, L, None if vol else f, 8, 8, volume_mode=vol, btype=btype,
                                  theta=4 * np.pi / 3, k3=0.4)
        for key in ("k1", "k2", "k3", "B"):
            fx[f"{name}_{key}"] = r[key]
    np.savez_compressed(os.path.join(HERE, "bispectrum.npz"), **fx)


def velocity_fixture():
    oracle.build(ref=True)
    table = load_table()
    fx = {}
    for lpt in (2, 1):
        prm = oracle.ic_params(16, 16, 64.0, 42, table, lpt_order=lpt, pk_bins=8,
                               index_vel=table.index_of("t_cdm"))
        fx[f"v_16_{lpt}"] = oracle.ref_ic_pipeline(prm, want=("vel", "pk"))["vel"]
    np.savez_compressed(os.path.join(HERE, "velocity.npz"), **fx)



def stages_fixture():
    oracle.build(ref=True)
    table = load_table()
    fx = {}
    want = ("grf", "delta_k", "phi_k", "disp", "rho", "pk")
    for lpt, ma in ((2, 0), (2, 3)):
        prm = oracle.ic_params(16, 16, 64.0, 42, table, lpt_order=lpt, ma_cycles=ma, pk_bins=8)
        out = oracle.ref_ic_pipeline(prm, want=want)
        for key in ("grf", "delta_k", "phi_k", "disp0", "disp1", "disp2", "rho"):
            fx[f"s_{lpt}_{ma}_{key}"] = out[key]
    np.savez_compressed(os.path.join(HERE, "stages.npz"), **fx)


if __name__ == "__main__":
    main()
