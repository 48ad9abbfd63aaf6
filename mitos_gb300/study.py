"""The precision study of the 256^3 configuration (box 500 Mpc/h, seed 7): the first- and
second-order displacement grids computed through the reference entry points in FP32 and FP64.

The reference combines both orders into one potential phi = f1 phi_1 + f2 phi_2 (src/2lpt.c:38-143,
f1 = 1, f2 = -3/7) before taking its gradient (src/mitos.c:395-416).  To report the error of each
order on its own, the two potentials are formed separately with the same entry points:

  delta(k)   generate_complex_grf + enforce_hermiticity (src/grf.c), the primordial power
             (kernel_power_no_transfer), generatePerturbationGrid with the density transfer
             function at z_ini (src/generate_grids.c:28-67), r2c
  phi_1(k)   kernel_inv_poisson of delta(k)         (the Zel'dovich potential)
  phi_2(k)   solve2LPT with f1 = 0, f2 = 1           (the second-order potential alone)
  d_i        kernel_undo_Hermite_window (TSC), kernel_d{x,y,z}, c2r   (src/mitos.c:395-416)
"""
from __future__ import annotations

import numpy as np

from . import lib as ml


def _to_real(dg, N):
    return ml.get_box(dg)[..., :N].astype(np.float64)


def displacement_orders(N: int, L: float, seed: int, table, spline, precision: int, z: float = 31.0):
    """{1: [d_x, d_y, d_z], 2: [d_x, d_y, d_z]} of the first- and second-order potentials (host
    FP64 copies of the device grids)"""
    lt = float(spline.tau_params(z))
    cosmo = ml.Cosmology(getattr(table, "h", 0.67), table.n_s, table.A_s, table.k_pivot, z, lt, 0.0, z, lt)
    grf = ml.alloc_local_grid(N, L, precision)
    grid = ml.alloc_local_grid(N, L, precision)
    pot = ml.alloc_local_grid(N, L, precision)
    work = ml.alloc_local_grid(N, L, precision)
    der = ml.alloc_local_grid(N, L, precision)
    try:
        ml.generate_complex_grf(grf, ml.rng_init(seed))
        ml.enforce_hermiticity(grf)
        ml._check(ml.fft_apply_kernel_dg(grf, grf, "power_no_transfer", cosmo))
        ml.generatePerturbationGrid(cosmo, spline, grf, grid, "d_cdm", 1.0)
        ml.fft_r2c_dg(grid)
        hp = ml.HermiteParams(3, N, L)
        out = {}
        for order in (1, 2):
            if order == 1:
                ml._check(ml.fft_apply_kernel_dg(pot, grid, "inv_poisson"))
            else:
                ml.solve2LPT(pot, grid, work, 0.0, 1.0)
            ml._check(ml.fft_apply_kernel_dg(pot, pot, "undo_Hermite_window", hp))
            comps = []
            for name in ("dx", "dy", "dz"):
                ml._check(ml.fft_apply_kernel_dg(der, pot, name))
                ml.fft_c2r_dg(der)
                comps.append(_to_real(der, N))
            out[order] = comps
        return out
    finally:
        for g in (grf, grid, pot, work, der):
            ml.free_local_grid(g)


def rms_rel(a, b) -> float:
    """rms(a - b) / rms(b) over all components"""
    num = sum(float(np.sum((x - y) ** 2)) for x, y in zip(a, b))
    den = sum(float(np.sum(y ** 2)) for y in b)
    return float(np.sqrt(num / den))
