"""Host driver of the learned Monge-Ampere warm start.

Training pairs come from the plain (cold) Monge-Ampere iteration on the device
(manet_training_pair); the network trains on the GPU through the library's own BF16 forward /
backward / Adam kernels (manet_train_step); the comparison runs solveMongeAmpereTol cold and warm
on held-out realisations and reports cycles and device time to the tolerance.
"""
from __future__ import annotations

import ctypes

import numpy as np

from . import lib as ml

Z_INI = 31.0


def cosmology(table, spline, z: float = Z_INI) -> ml.Cosmology:
    lt = spline.tau_params(z)
    return ml.Cosmology(0.67, table.n_s, table.A_s, table.k_pivot, z, lt, 0.0, z, lt)


def density(N: int, L: float, seed: int, table, spline, prec: int = ml.FP32, z: float = Z_INI):
    """delta at z in momentum space with delta(x) kept in the box: generate_complex_grf,
    enforce_hermiticity, primordial power, generatePerturbationGrid, r2c (src/mitos.c:216-362)."""
    cosmo = cosmology(table, spline, z)
    grf = ml.alloc_local_grid(N, L, prec)
    dens = ml.alloc_local_grid(N, L, prec)
    ml.generate_complex_grf(grf, ml.rng_init(seed))
    ml.enforce_hermiticity(grf)
    ml.fft_apply_kernel_dg(grf, grf, "power_no_transfer", cosmo)
    ml.generatePerturbationGrid(cosmo, spline, grf, dens, "d_cdm", 1.0)
    ml.fft_r2c_dg(dens)
    ml.free_local_grid(grf)
    return dens


def _real_grid(N: int, L: float):
    """an FP32 device real grid of N*N*(N+2) floats (the complex buffer released)"""
    g = ml.alloc_local_grid(N, L, ml.FP32)
    ml.load().free_local_complex_grid(ctypes.byref(g))
    return g


class PairSet:
    """device-resident training pairs (delta, phi_1, phi_2, sigma) at one grid size"""

    def __init__(self, N: int, L: float, seeds, table, spline, cycles: int = 10):
        self.N, self.L = N, L
        self.pairs = []
        self.stats = []
        pot, work = ml.alloc_local_grid(N, L, ml.FP32), ml.alloc_local_grid(N, L, ml.FP32)
        try:
            for s in seeds:
                dens = density(N, L, int(s), table, spline)
                grids = [_real_grid(N, L) for _ in range(4)]
                self.stats.append(ml.manet_training_pair(pot, dens, work, cycles, *grids))
                self.pairs.append(grids)
                ml.free_local_grid(dens)
        finally:
            ml.free_local_grid(pot)
            ml.free_local_grid(work)

    def rms(self, n: int = 8) -> np.ndarray:
        """rms of delta, phi_1, phi_2, sigma over the first n pairs"""
        acc = np.zeros(4)
        k = min(n, len(self.pairs))
        for grids in self.pairs[:k]:
            for c, g in enumerate(grids):
                a = ml.get_box(g)[..., :self.N]
                acc[c] += np.mean(a.astype(np.float64) ** 2)
        return np.sqrt(acc / k)

    def free(self) -> None:
        for grids in self.pairs:
            for g in grids:
                ml.free_local_grid(g)
        self.pairs = []


def set_scales(net: ml.Manet, rms: np.ndarray) -> None:
    for c in range(3):
        net.scale_in[c] = float(rms[c])
    net.scale_out = float(rms[3])


def train(net: ml.Manet, pairs: PairSet, steps: int, lr: float = 2e-3, seed: int = 0) -> np.ndarray:
    """Adam steps on randomly drawn pairs with a cosine learning-rate decay to lr / 20."""
    rng = np.random.default_rng(seed)
    losses = np.zeros(steps)
    N = pairs.N
    for i in range(steps):
        d, p1, p2, sg = pairs.pairs[rng.integers(len(pairs.pairs))]
        lr_i = lr * (0.05 + 0.95 * 0.5 * (1 + np.cos(np.pi * i / steps)))
        losses[i] = ml.manet_train_step(net, N, N + 2, d, p1, p2, sg, lr_i)
    return losses


def evaluate(net: ml.Manet, pairs: PairSet) -> float:
    """mean loss (relative to the target variance, i.e. 1 - explained fraction) without updates"""
    N = pairs.N
    out = []
    for d, p1, p2, sg in pairs.pairs:
        out.append(ml.manet_loss_grad(net, N, N + 2, d, p1, p2, sg))
    return float(np.mean(out))


def compare(net: ml.Manet | None, N: int, L: float, seeds, table, spline, tol: float = 1e-6,
            max_cycles: int = 40) -> dict:
    """cold and (if net) warm solveMongeAmpereTol on each seed; per-seed statistics"""
    out = {"cold": [], "warm": []}
    pot, work = ml.alloc_local_grid(N, L, ml.FP32), ml.alloc_local_grid(N, L, ml.FP32)
    try:
        for s in seeds:
            dens = density(N, L, int(s), table, spline)
            out["cold"].append(ml.solveMongeAmpereTol(pot, dens, work, tol, max_cycles))
            if net is not None:
                out["warm"].append(ml.solveMongeAmpereTol(pot, dens, work, tol, max_cycles, net))
            ml.free_local_grid(dens)
    finally:
        ml.free_local_grid(pot)
        ml.free_local_grid(work)
    return out


def save(net: ml.Manet, path: str) -> None:
    np.savez(path, params=ml.manet_params(net), scale_in=np.array(net.scale_in[:], np.float32),
             scale_out=np.float32(net.scale_out), steps=np.int64(net.steps))


def load(path: str, seed: int = 1) -> ml.Manet:
    z = np.load(path)
    net = ml.manet_init(seed)
    ml.manet_set_params(net, z["params"])
    for c in range(3):
        net.scale_in[c] = float(z["scale_in"][c])
    net.scale_out = float(z["scale_out"])
    net.steps = int(z["steps"])
    return net
