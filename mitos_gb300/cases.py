"""Small workloads that run one part of the library a few times, for profiling one kernel at a size
whose grids still exceed L2 but whose device footprint stays at a few GB:

    python -m mitos_gb300.cases conv 256     # network inference (k_conv), 4 layers
    python -m mitos_gb300.cases ngenic 512   # the N-GenIC-like field (k_ngenic)
    python -m mitos_gb300.cases ma 256       # Monge-Ampere cycles (z_hess_ma, x_add_poisson)
    python -m mitos_gb300.cases noise 512    # white noise (k_noise), FP32 (noise64: FP64)
    python -m mitos_gb300.cases ic 256       # one FP32 initial condition (every pass; ic64: FP64)
    python -m mitos_gb300.cases ensemble 0 3 # the 48 realisations (16 each of 64^3, 96^3, 128^3) as
                                             # one graph; the size argument is unused
    python -m mitos_gb300.cases r2c 512 3 2  # fft_r2c_dg, FP32; fourth argument: the cluster mode
                                             # of the Z + Y step (mitos_set_cluster_fft; 0 = off)

Each runs its workload `reps` times (third argument, default 3) after one warm-up and prints the
device time per repetition (CUDA events on the library stream).
"""
from __future__ import annotations

import sys

import numpy as np

from . import lib as ml
from . import manet
from .perturb import load_table


def conv(N: int, reps: int) -> float:
    net = ml.manet_init(1)
    g = [ml.alloc_local_grid(N, 2.0 * N, ml.FP32) for _ in range(4)]
    rng = np.random.default_rng(0)
    for x in g[:3]:
        ml.set_box(x, rng.standard_normal((N, N, N)).astype(np.float32))
    args = [ml._vp(x.box) for x in g]
    ml.manet_infer(net, N, N + 2, *args)
    ml.timer_start()
    for _ in range(reps):
        ml.manet_infer(net, N, N + 2, *args)
    ms = ml.timer_stop() / reps
    for x in g:
        ml.free_local_grid(x)
    ml.manet_free(net)
    return ms


def ngenic(N: int, reps: int) -> float:
    g = ml.alloc_local_grid(N, 2.0 * N, ml.FP32)
    ml.generate_ngeniclike_grf_dg(g, 1)
    ml.timer_start()
    for r in range(reps):
        ml.generate_ngeniclike_grf_dg(g, 2 + r)
    ms = ml.timer_stop() / reps
    ml.free_local_grid(g)
    return ms


def ma(N: int, reps: int) -> float:
    table = load_table()
    spline = ml.Spline(table)
    L = 500.0 * N / 256
    dens = manet.density(N, L, 3000, table, spline)
    pot, work = ml.alloc_local_grid(N, L, ml.FP32), ml.alloc_local_grid(N, L, ml.FP32)
    ml.solveMongeAmpereTol(pot, dens, work, 0.0, 2)
    ms = 0.0
    for _ in range(reps):
        st = ml.solveMongeAmpereTol(pot, dens, work, 0.0, 3)
        ms += st["ms"]
    for x in (pot, work, dens):
        ml.free_local_grid(x)
    return ms / reps


def noise(N: int, reps: int, prec: int = ml.FP32) -> float:
    g = ml.alloc_local_grid(N, 2.0 * N, prec)
    ml.generate_complex_grf(g, ml.rng_init(1))
    ml.timer_start()
    for r in range(reps):
        ml.generate_complex_grf(g, ml.rng_init(2 + r))
    ms = ml.timer_stop() / reps
    ml.free_local_grid(g)
    return ms


def ic(N: int, reps: int, prec: int = ml.FP32) -> float:
    table = load_table()
    spline = ml.Spline(table)
    cfg = lambda s: ml.ic_config(N, N, 1000.0 * N / 512, s, table, pk_bins=64, pk_linear=True, precision=prec)
    ml.ic_pipeline_run(cfg(1), spline)
    ml.timer_start()
    for r in range(reps):
        ml.ic_pipeline_run(cfg(2 + r), spline)
    return ml.timer_stop() / reps


def r2c(N: int, reps: int) -> float:
    g = ml.alloc_local_grid(N, 2.0 * N, ml.FP32)
    ml.set_box(g, np.random.default_rng(1).standard_normal((N, N, N + 2)).astype(np.float32))
    ml.fft_r2c_dg(g)
    ml.timer_start()
    for _ in range(reps):
        ml.fft_r2c_dg(g)
    ms = ml.timer_stop() / reps
    ml.free_local_grid(g)
    return ms


def ensemble(N: int, reps: int) -> float:
    """ms per replay of the 48-member graph (2LPT, 32 linear shells, FP32, 4 Mpc/h cells), the
    library's default tiles and batching"""
    table = load_table()
    spline = ml.Spline(table)
    cfgs = [ml.ic_config(n, n, box, 1000 + 16 * k + i, table, pk_bins=32, pk_linear=True, precision=ml.FP32)
            for k, (n, box) in enumerate([(64, 256.0), (96, 384.0), (128, 512.0)]) for i in range(16)]
    ens = ml.Ensemble(cfgs, spline, streams=8)
    ens.run()
    ms = sum(ens.run() for _ in range(reps)) / reps
    ens.close()
    return ms


def noise64(N: int, reps: int) -> float:
    return noise(N, reps, ml.FP64)


def ic64(N: int, reps: int) -> float:
    return ic(N, reps, ml.FP64)


CASES = {"conv": conv, "ngenic": ngenic, "ma": ma, "noise": noise, "noise64": noise64, "ic": ic, "ic64": ic64, "r2c": r2c, "ensemble": ensemble}

if __name__ == "__main__":
    name = sys.argv[1]
    N = int(sys.argv[2]) if len(sys.argv) > 2 else 256
    reps = int(sys.argv[3]) if len(sys.argv) > 3 else 3
    if len(sys.argv) > 4:
        ml.set_cluster_fft(int(sys.argv[4]))
    print(f"{name} N={N}: {CASES[name](N, reps):.4f} ms per repetition")
    # the same workload once more with per-launch timing: device time per kernel name (not for the
    # ensemble: its launches are captured into a graph)
    if name == "ensemble":
        sys.exit(0)
    ml.kernel_timing(True)
    CASES[name](N, 1)
    per = {}
    for k, t in ml.kernel_times():
        per.setdefault(k, []).append(t)
    ml.kernel_timing(False)
    for k, v in sorted(per.items(), key=lambda kv: -sum(kv[1])):
        print(f"  {k:24s} {len(v):4d} launches  {sum(v):9.4f} ms")
