#!/usr/bin/env python3
"""Initial-condition throughput on GB300: 512^3 grid, 512^3 particles, box 1000 Mpc/h, FP32.

One step = one full initial condition through the C ABI (ic_pipeline_run): xoshiro256** white
noise -> primordial power x BBKS transfer -> 2LPT potential (six Hessians, second-order
source, Poisson) -> TSC window undo -> three displacement grids -> lattice displacement (TSC
gather) + wrap -> CIC -> overdensity r2c -> CIC window undo -> P(k) in 128 linear shells.

  value  ICs/s with the transfer table on the host and all grids in HBM (device-timed,
         CUDA events on the library stream); every grid is 0.54 GB, larger than L2.
  e2e    the same call with the particle positions (512^3 x 3 floats) copied to pinned host
         memory every step, plus the table upload and the P(k) read.
  --impl reference   the reference algorithm restated in C (oracle/, OpenMP, FP64) on the
         host cores: one full 512^3 IC per step.
  noise_exact   (CPU leg) the GPU's white noise of the 64^3 and 256^3 precision configurations
         against the reference's, value by value.

N > 1 GPUs run independent replicas (different seeds): the IC does not shard.
"""
from __future__ import annotations

import argparse
import ctypes
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, HERE)

METRIC = "512^3 2LPT initial-condition throughput (noise->2LPT->displacements->CIC->P(k))"
UNIT = "IC/s"


def algorithmic_bytes(name: str, G: float) -> float:
    """minimum bytes a launch of each kernel must move, in units of one complex grid G (in the 2LPT
    IC the 2LPT-source Z pass also clears the deposit's density grid: 7 + 1 G; the noise launch
    writes the noise, 1 G)"""
    table = {"noise": 1, "x_hess": 4, "y_hess": 9, "y_hess_a": 4, "y_hess_b": 3, "y_disp_a": 3, "y_stn": 2, "z_hess_2lpt": 7,
             "z_hess_2lpt_r2c": 8, "z_hess_ma": 8, "z_hess_ma_r2c": 8, "z_r2c": 2,
             "y_plain": 2, "x_plain": 2, "x_combine": 3, "x_add_poisson": 3, "x_disp": 3,
             "y_disp": 5, "z_disp": 6, "displace_cic": 4, "x_pk": 1, "z_c2r": 2,
             "lattice_cic": 4, "x_combine_disp": 4, "filter": 0}
    return table.get(name, 0) * G


def replica_seed(base: int, rank: int) -> int:
    """first seed of a rank's replicas: ranks 1000 seeds apart, so up to 1000 steps never share one"""
    return base + 1000 * rank


def max_over_ranks(x: float, dist) -> float:
    """the largest value of x over the ranks (the slowest replica sets the job's time)"""
    if dist is None:
        return x
    import torch
    dev = "cuda" if dist.get_backend() == "nccl" else "cpu"
    t = torch.tensor([x], dtype=torch.float64, device=dev)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def job_throughput(ws: int, steps: int, seconds: float) -> float:
    """units all ranks processed (steps each) per second of the slowest rank"""
    return ws * steps / seconds


def dist_setup():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


class Clocks:
    """nvidia-smi samples (every 20 ms, timestamped) kept for the timed region only: start() returns
    once the sampler has written its first line, mark() brackets the region"""

    def __init__(self, gpu: int):
        self.gpu = gpu
        self.proc = None
        self.path = None
        self.t0 = self.t1 = None

    def start(self):
        fd, self.path = tempfile.mkstemp(suffix=".csv")
        os.close(fd)
        q = ("timestamp,index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")
        try:
            self.proc = subprocess.Popen(["nvidia-smi", f"--id={self.gpu}", f"--query-gpu={q}",
                                          "--format=csv,noheader,nounits", "-lms", "20"],
                                         stdout=open(self.path, "w"), stderr=subprocess.DEVNULL)
        except (FileNotFoundError, OSError):
            self.proc = None
            return
        deadline = time.time() + 5.0
        while time.time() < deadline and os.path.getsize(self.path) == 0 and self.proc.poll() is None:
            time.sleep(0.01)

    def mark(self, begin: bool):
        if begin:
            self.t0 = time.time()
        else:
            self.t1 = time.time()

    def stop(self):
        if not self.proc:
            return None
        time.sleep(0.05)
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        import datetime
        rows = []
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in open(self.path):
            f = [x.strip() for x in line.split(",")]
            if len(f) < 10:
                continue
            try:
                ts = datetime.datetime.strptime(f[0], "%Y/%m/%d %H:%M:%S.%f").timestamp()
                rows.append((ts, float(f[2]), float(f[3]), [n for n, v in zip(names, f[6:10]) if v.lower() == "active"]))
            except ValueError:
                continue
        os.unlink(self.path)
        if not rows:
            return None
        t0 = self.t0 if self.t0 is not None else rows[0][0]
        t1 = self.t1 if self.t1 is not None else rows[-1][0]
        inside = [r for r in rows if t0 <= r[0] <= t1]
        if not inside:  # a region shorter than the sampling interval: the samples on either side
            before = [r for r in rows if r[0] < t0][-1:]
            after = [r for r in rows if r[0] > t1][:1]
            inside = before + after
        sm = [r[1] for r in inside]
        load = [x for x in sm if x > 0.5 * max(sm)] or sm
        return {"sm_mhz": statistics.median(load), "sm_max_mhz": max(r[2] for r in inside),
                "reasons": sorted({n for r in inside for n in r[3]}), "samples": len(inside),
                "region_s": round(t1 - t0, 3)}


def peak_hbm():
    p = os.path.join(HERE, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        return float(json.load(open(p))["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


def ncu_traffic(kernel: str, N: int):
    """DRAM bytes per launch of a kernel from the committed ncu summary (scaled to N)"""
    p = os.path.join(HERE, "profiles", "ncu_traffic.json")
    if not os.path.exists(p):
        return None
    d = json.load(open(p))
    e = d.get(kernel)
    if not e:
        return None
    return e["dram_bytes"] * (N / e["N"]) ** 3


def cpu_baseline(args, table, steps=1):
    """the oracle (the reference's algorithm restated in C, FP64, all host threads) on one full IC of
    the benchmark configuration per step"""
    import oracle
    times = []
    for i in range(steps):
        prm = oracle.ic_params(args.N, args.N, args.boxlen, args.seed + i, table, pk_bins=args.bins, pk_linear=True)
        t0 = time.perf_counter()
        oracle.ic_pipeline(prm)
        times.append(time.perf_counter() - t0)
    sec_per_ic = sum(times) / len(times)
    return {"value": 1.0 / sec_per_ic, "unit": UNIT, "cores": oracle.lib().orc_num_threads(),
            "kind": "port",
            "sample": f"{steps} full {args.N}^3 IC(s) (L = {args.boxlen:g}, {args.bins} linear shells), "
                      f"{sec_per_ic:.1f} s each: the reference's algorithm (src/mitos.c:205-422,794-863, "
                      "analyse/src/mitos_read.c:278-419) restated in C, FP64, OpenMP over the host cores "
                      "where the reference loops are parallel, its CIC serial as in mitos_read; the FFTs are "
                      "the project's CPU FFT with FFTW's conventions, not FFTW (absent on this host)"}, times


def run_reference(args):
    ws, rank, _ = dist_setup()
    if rank != 0:
        return 0
    from mitos_gb300.perturb import load_table
    table = load_table()
    # no warm-up runs: the C port keeps no state between ICs (its FFT twiddles are built on first
    # use, a few milliseconds), so a warm-up would only repeat a full IC
    base, times = cpu_baseline(args, table, steps=args.steps)
    cfg = config(args)
    cfg["precision"] = "fp64"
    line = {"impl": "reference", "metric": METRIC, "value": base["value"], "unit": UNIT,
            "n_gpus": ws, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": 1e3 / base["value"], "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f64", "data": "synthetic (xoshiro noise, BBKS table)",
            "config": cfg, "cpu_baseline": base,
            "e2e": {"value": base["value"], "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)
    return 0


NOISE_CASES = (("64^3 seed 42 L 256 (C1)", 64, 42, 256.0), ("256^3 seed 7 L 500 (C2)", 256, 7, 500.0))


def gpu_noise(ml) -> dict:
    """FP64 and FP32 white noise of the two precision configurations from the GPU (host copies)"""
    out = {}
    for name, N, seed, L in NOISE_CASES:
        for prec in (ml.FP64, ml.FP32):
            g = ml.alloc_local_grid(N, L, prec)
            ml.generate_complex_grf(g, ml.rng_init(seed))
            out[(name, prec)] = ml.get_fbox(g)
            ml.free_local_grid(g)
    return out


def noise_exactness(ml, noise: dict) -> dict:
    """(CPU leg: the oracle as the checker) the GPU's Gaussians against the reference's (the oracle,
    host libm): FP64 equal bit for bit except where the host libm misrounded log or cos (each such
    value checked to be the exactly rounded one); FP32 against the reference rounded to float"""
    import math
    import oracle
    from oracle import crcheck
    out = {}
    for name, N, seed, L in NOISE_CASES:
        ref = oracle.grf(N, L, seed, hermitian=False).view(np.float64).ravel()[2:]
        g64 = noise[(name, ml.FP64)].view(np.float64).ravel()[2:]
        g32 = noise[(name, ml.FP32)].view(np.float32).ravel()[2:]
        d = oracle.draws(seed, 2 * len(ref))
        factor = math.sqrt(L ** 3 / 2)
        differ = np.nonzero(g64 != ref)[0]
        explained = 0
        for i in differ:
            u, y = crcheck.sample_norm_parts(int(d[2 * i]), int(d[2 * i + 1]))
            lu, cy = crcheck.exact_log(u), crcheck.exact_cos(y)
            misround = math.log(u) != lu or math.cos(y) != cy
            explained += int(misround and g64[i] == math.sqrt(-2.0 * lu) * cy * factor)
        u32 = crcheck.ulps(g32, ref.astype(np.float32))
        out[name] = {"gaussians": int(len(ref)),
                     "fp64": {"equal": int(len(ref) - len(differ)), "differ": int(len(differ)),
                              "differ_at_libm_misroundings_exact": explained,
                              "max_ulp": float(crcheck.ulps(g64, ref).max())},
                     "fp32": {"equal_to_float_of_reference": float(np.mean(g32 == ref.astype(np.float32))),
                              "max_ulp": float(u32.max()), "p999_ulp": float(np.percentile(u32, 99.9))}}
    return out


def config(args):
    return {"workload": f"{args.N}^3 grid, {args.N}^3 particles, box {args.boxlen:g} Mpc/h, z=31, 2LPT, "
                        f"CIC, P(k) {args.bins} linear shells",
            "N": args.N, "M": args.N, "boxlen": args.boxlen, "precision": args.precision,
            "pk_bins": args.bins, "parallelism": "replicas (independent seeds per GPU)",
            "l2": f"inputs larger than L2 (each grid {args.N ** 3 * 4 / 1e9:.2f} GB)" if args.N ** 3 * 4 > 129e6
                  else "grids smaller than L2 (no flush)", "cuda_graph": False}


def extras(ml, table, spline, args) -> dict:
    """the other parts of the benchmark configuration, measured after the main line's timing"""
    out = {}
    N, L = args.N, args.boxlen

    def cfg(prec, seed, n=N, box=L, bins=args.bins):
        return ml.ic_config(n, n, box, seed, table, method=ml.METHOD_2LPT, pk_bins=bins, pk_linear=True,
                            precision=prec)

    # FP64 512^3 IC (the FP64 GPU path) and the FP32 P(k) against it on the same seed
    r32 = ml.ic_pipeline_run(cfg(ml.FP32, args.seed), spline)
    r64 = ml.ic_pipeline_run(cfg(ml.FP64, args.seed), spline)
    ml.timer_start()
    for i in range(3):
        ml.ic_pipeline_run(cfg(ml.FP64, args.seed + 1 + i), spline)
    ms64 = ml.timer_stop() / 3
    ok = np.isfinite(r64["pk_p"]) & (r64["pk_p"] != 0)
    rel = np.abs(r32["pk_p"][ok] / r64["pk_p"][ok] - 1)
    out["fp64"] = {"ms_per_ic": ms64, "ic_per_s": 1e3 / ms64,
                   "pk_fp32_vs_fp64": {"max_rel": float(rel.max()), "bins": int(ok.sum()), "target": 1e-4}}

    # the precision study at 256^3 (box 500 Mpc/h, seed 7, 128 linear shells): FP32 against the FP64
    # GPU path for the first- and second-order displacement grids separately and P(k) per bin
    from mitos_gb300 import study
    d64 = study.displacement_orders(256, 500.0, 7, table, spline, ml.FP64)
    d32 = study.displacement_orders(256, 500.0, 7, table, spline, ml.FP32)
    c64 = ml.ic_pipeline_run(cfg(ml.FP64, 7, 256, 500.0, 128), spline)
    c32 = ml.ic_pipeline_run(cfg(ml.FP32, 7, 256, 500.0, 128), spline)
    okc = c64["pk_obs"] > 0
    out["precision_256"] = {"disp1_rms_rel": study.rms_rel(d32[1], d64[1]),
                            "disp2_rms_rel": study.rms_rel(d32[2], d64[2]),
                            "disp_target": 1e-5,
                            "pk_max_rel_per_bin": float(np.abs(c32["pk_p"][okc] / c64["pk_p"][okc] - 1).max()),
                            "pk_bins": int(okc.sum()), "pk_target": 1e-4,
                            "pk_obs_equal": bool(np.array_equal(c32["pk_obs"], c64["pk_obs"]))}
    del d64, d32

    # the library's 3D FFTs against cuFFT (torch.fft) at 512^3 FP32: a comparison line only (cuFFT is
    # never on the path); both CUDA-event timed on their own streams, median of 5 after a warm-up
    import torch
    g = ml.alloc_local_grid(N, L, ml.FP32)
    ml.set_box(g, np.random.default_rng(1).standard_normal((N, N, N)).astype(np.float32))
    ours = {"r2c": [], "c2r": []}
    for i in range(6):
        ml.timer_start()
        ml.fft_r2c_dg(g)
        t_r2c = ml.timer_stop()
        ml.timer_start()
        ml.fft_c2r_dg(g)
        t_c2r = ml.timer_stop()
        if i:
            ours["r2c"].append(t_r2c)
            ours["c2r"].append(t_c2r)
    ml.free_local_grid(g)
    x = torch.randn((N, N, N), dtype=torch.float32, device="cuda")
    cu = {"r2c": [], "c2r": []}
    for i in range(6):
        e = [torch.cuda.Event(enable_timing=True) for _ in range(3)]
        e[0].record()
        k = torch.fft.rfftn(x)
        e[1].record()
        y = torch.fft.irfftn(k, s=(N, N, N))
        e[2].record()
        torch.cuda.synchronize()
        if i:
            cu["r2c"].append(e[0].elapsed_time(e[1]))
            cu["c2r"].append(e[1].elapsed_time(e[2]))
    del x, k, y
    torch.cuda.empty_cache()
    Gc = N * N * (N // 2 + 1) * 8
    med = statistics.median
    out["fft_vs_cufft"] = {
        "N": N, "precision": "fp32", "note": "read real + write complex (or the reverse) once = 2 G per transform",
        "ours_ms": {k: med(v) for k, v in ours.items()}, "cufft_ms": {k: med(v) for k, v in cu.items()},
        "ours_GBps_at_2G": {k: 2 * Gc / (med(v) / 1e3) / 1e9 for k, v in ours.items()},
        "cufft_GBps_at_2G": {k: 2 * Gc / (med(v) / 1e3) / 1e9 for k, v in cu.items()}}

    # particle velocities (the velocity transfer function t_cdm, 2LPT with the reference's velocity
    # factors, TSC gather at the displaced positions): the 512^3 FP32 IC with positions and velocities
    # into pinned host buffers, CUDA events on the library stream (the copies run on the copy stream)
    import torch
    pv = [torch.empty((N ** 3, 3), dtype=torch.float32, pin_memory=True) for _ in range(2)]
    kv, pk_, ov = np.zeros(args.bins), np.zeros(args.bins), np.zeros(args.bins, np.int64)
    rv = ml.ICResult(kv.ctypes.data_as(ml._dp), pk_.ctypes.data_as(ml._dp), ov.ctypes.data_as(ml._lp),
                     ctypes.cast(pv[0].data_ptr(), ml._fp), 0, 0.0, ctypes.cast(pv[1].data_ptr(), ml._fp))
    cv = cfg(ml.FP32, args.seed)
    ml._check(ml.load().ic_pipeline_run(ctypes.byref(cv), ctypes.byref(spline.sp), ctypes.byref(rv)))
    ml.kernel_timing(True)
    ml.timer_start()
    for i in range(3):
        ml._check(ml.load().ic_pipeline_run(ctypes.byref(cv), ctypes.byref(spline.sp), ctypes.byref(rv)))
    msv = ml.timer_stop() / 3
    kt = ml.kernel_times()
    ml.kernel_timing(False)
    vg = [t for n, t in kt if n == "vel_gather"]
    out["velocities"] = {"ms_per_ic": msv, "ic_per_s": 1e3 / msv,
                         "vel_gather_ms": sum(vg) / max(len(vg), 1),
                         "vel_rms": float(np.sqrt(np.mean(pv[1].numpy()[::4096] ** 2)))}

    # thermal motion (src/mitos.c:910-1064 without Firebolt) of a 512^3 species: Fermi-Dirac at the
    # relic neutrino temperature, 0.06 eV, km/s.  The kernel alone on device velocities (7 draws, one
    # sampler lookup and three Box-Muller normals a particle; 24 bytes read and written), FP32 and FP64,
    # then the IC with positions, velocities and thermal motion
    t_nu = 1.9517578 * 8.617333262e-5
    smp = ml.thermal_sampler(ml.FERMION, t_nu)
    dv = torch.zeros((N ** 3, 3), dtype=torch.float32, device="cuda")
    st0 = np.array(list(ml.rng_init(args.seed).s), np.uint64)
    th = {}
    for name, prec in (("fp32", ml.FP32), ("fp64", ml.FP64)):
        ml.set_precision(prec)
        ml.thermal_velocities(smp, st0, dv, 0.06, 1 / 32.0, 299792.458)
        ml.kernel_timing(True)
        for i in range(3):
            ml.thermal_velocities(smp, st0, dv, 0.06, 1 / 32.0, 299792.458)
        kt = ml.kernel_times()
        ml.kernel_timing(False)
        tk = [t for n_, t in kt if n_ == "thermal"]
        ms = sum(tk) / max(len(tk), 1)
        th[name] = {"kernel_ms": ms, "particles_per_s": N ** 3 / (ms * 1e-3),
                    "GB_per_s": 24.0 * N ** 3 / (ms * 1e-3) / 1e9}
    ml.set_precision(ml.FP64)
    ml.thermal_sampler_free(smp)
    del dv
    ct = ml.ic_config(N, N, L, args.seed, table, method=ml.METHOD_2LPT, pk_bins=args.bins, pk_linear=True,
                      precision=ml.FP32, thermal=ml.FERMION, thermal_M_eV=0.06, thermal_T_eV=t_nu,
                      speed_of_light=299792.458)
    ml._check(ml.load().ic_pipeline_run(ctypes.byref(ct), ctypes.byref(spline.sp), ctypes.byref(rv)))
    ml.timer_start()
    for i in range(3):
        ml._check(ml.load().ic_pipeline_run(ctypes.byref(ct), ctypes.byref(spline.sp), ctypes.byref(rv)))
    th["ic_ms_with_thermal"] = ml.timer_stop() / 3
    out["thermal"] = th
    del pv

    # bispectrum (src/calc_powerspec.c:295-508) of a 512^3 FP32 field in 16 equilateral log bins, as
    # analyse/src/mitos_box_bispec.c calls it (the field, then the bin volumes)
    gb_ = ml.alloc_local_grid(N, L, ml.FP32)
    ml.generate_complex_grf(gb_, ml.rng_init(args.seed))
    gb_.momentum_space = b"\x01"
    ml.calc_bispectrum(gb_, 16, 16, btype=0, theta=4 * np.pi / 3)
    t0 = time.perf_counter()
    bsp = ml.calc_bispectrum(gb_, 16, 16, btype=0, theta=4 * np.pi / 3)
    ml.calc_bispectrum(gb_, 16, 16, volume_mode=True, btype=0, theta=4 * np.pi / 3)
    ms_eq = (time.perf_counter() - t0) * 1e3
    # squeezed (type 1, k3 = 0.02 h/Mpc): two c2r a bin; kernel times of the field call
    ml.kernel_timing(True)
    ml.calc_bispectrum(gb_, 16, 16, btype=1, k3=0.02)
    kt = ml.kernel_times()
    ml.kernel_timing(False)
    Gb = N * N * (N // 2 + 1) * 8
    mk = [t for n_, t in kt if n_ == "bispec_mask"]
    sk = [t for n_, t in kt if n_ == "bispec_sum"]
    out["bispectrum"] = {"N": N, "bins": 16, "ms_field_and_volumes": ms_eq,
                         "nonempty_bins": int(np.count_nonzero(bsp["k1"])),
                         "squeezed_field_ms": sum(t for _, t in kt),
                         # mask: two masks written (2 G; the field is read in the shells only);
                         # sum: two real grids read (2 G)
                         "mask_ms": sum(mk) / max(len(mk), 1), "mask_GBps": 2 * Gb / (sum(mk) / max(len(mk), 1) / 1e3) / 1e9,
                         "sum_ms": sum(sk) / max(len(sk), 1), "sum_GBps": 2 * Gb / (sum(sk) / max(len(sk), 1) / 1e3) / 1e9}
    ml.free_local_grid(gb_)

    # 48 realisations (16 x 64^3 / 256, 16 x 96^3 / 384, 16 x 128^3 / 512 Mpc/h; 4 Mpc/h cells),
    # seeds 1000-1047, one captured CUDA graph over 8 streams, tiles from the autotuner
    sizes = [(64, 256.0), (96, 384.0), (128, 512.0)]
    tiles, radix = {}, {}
    for n, box in sizes:
        pxy, pz, _ = ml.autotune(cfg(ml.FP32, 1000, n, box, 32), spline)
        tiles[n] = [pxy, pz]
        radix[n] = ml.get_radix(n, ml.FP32)
    cfgs = [cfg(ml.FP32, 1000 + 16 * k + i, n, box, 32) for k, (n, box) in enumerate(sizes) for i in range(16)]
    # batched units of the members of each size (one launch per pass per unit): the library's
    # default (16 per unit), 8 per unit, and unbatched (48 pipeline runs over 8 streams)
    by_batch = {}
    for mb in (0, 8, 1):
        ens = ml.Ensemble(cfgs, spline, streams=8, max_batch=mb)
        ens.run()
        by_batch[mb] = (min(ens.run() for _ in range(5)), ens.launches(), ens.units())
        ens.close()
    best = min(by_batch, key=lambda mb: by_batch[mb][0])
    t, launches, units = by_batch[best]
    lat = {}
    for n, box in sizes:
        e1 = ml.Ensemble([cfg(ml.FP32, 1000, n, box, 32)], spline, streams=1)
        e1.run()
        lat[str(n)] = min(e1.run() for _ in range(10))
        e1.close()
    G = lambda n: n * n * (n // 2 + 1) * 8
    model = 16 * 15 * G(64) + 16 * 37 * G(96) + 16 * 37 * G(128)  # byte model (N <= 64: one-pass FFT)
    peak, _ = peak_hbm()
    out["ensemble"] = {"realizations": 48, "ms_per_replay": t, "realizations_per_s": 48e3 / t,
                       "max_batch": best, "units": units,
                       "ms_by_max_batch": {str(mb): v[0] for mb, v in by_batch.items()},
                       "latency_ms": lat, "gpu_launches_per_replay": launches, "tiles": tiles,
                       "radix_schedules": {str(n): {"N": r[0], "N/2": r[1]} for n, r in radix.items()},
                       "roofline": {"model_bytes": model, "GBps": model / (t / 1e3) / 1e9,
                                    "frac": model / (t / 1e3) / 1e9 / peak}}

    # Monge-Ampere to a relative rms residual of 1e-6 at 256^3 / 500 Mpc/h, cold against the
    # learned warm start (trained here: 256 seeds at 128^3 / 250 Mpc/h, 3000 Adam steps)
    from mitos_gb300 import manet
    t0 = time.perf_counter()
    pairs = manet.PairSet(128, 250.0, range(2000, 2256), table, spline, cycles=10)
    held = manet.PairSet(128, 250.0, range(3000, 3016), table, spline, cycles=10)
    t_pairs = time.perf_counter() - t0
    net = ml.manet_init(1)
    manet.set_scales(net, pairs.rms())
    t0 = time.perf_counter()
    losses = manet.train(net, pairs, 3000, lr=2e-3)
    ml.load().mitos_sync()
    t_train = time.perf_counter() - t0
    held_loss = manet.evaluate(net, held)
    pairs.free()
    held.free()
    cmp = manet.compare(net, 256, 500.0, range(3000, 3016), table, spline, tol=1e-6, max_cycles=30)
    ml.manet_free(net)
    mean = lambda k, f: float(np.mean([x[f] for x in cmp[k]]))
    out["monge_ampere"] = {
        "config": "256^3, L = 500 Mpc/h, z = 31, FP32 grids, FP64 residual sums, tol = 1e-6 on "
                  "sqrt(sum res^2 / sum rho^2) (reference eps = that / N^1.5), 16 held-out seeds 3000-3015",
        "cold": {"cycles": mean("cold", "cycles"), "ms": mean("cold", "ms"),
                 "converged": sum(x["converged"] for x in cmp["cold"])},
        "warm": {"cycles": mean("warm", "cycles"), "ms": mean("warm", "ms"), "ms_warm_start": mean("warm", "ms_warm"),
                 "converged": sum(x["converged"] for x in cmp["warm"])},
        "rel_after_first_update": {"cold": mean("cold", "rel_second"), "warm": mean("warm", "rel_second")},
        "net": {"train_pairs_s": t_pairs, "train_s": t_train, "steps": 3000,
                "loss_first": float(losses[:10].mean()), "loss_last": float(losses[-100:].mean()),
                "held_out_loss": held_loss}}

    # 1024^3 FP32 IC, L = 2000 Mpc/h (the large configuration; about 80 GB of workspace)
    c1k = lambda seed: ml.ic_config(1024, 1024, 2000.0, seed, table, method=ml.METHOD_2LPT, pk_bins=256,
                                    pk_linear=True, precision=ml.FP32)
    r1k = ml.ic_pipeline_run(c1k(args.seed), spline)
    ml.timer_start()
    for i in range(3):
        ml.ic_pipeline_run(c1k(args.seed + 1 + i), spline)
    ms1k = ml.timer_stop() / 3
    G1k = 1024 * 1024 * 513 * 8
    peak, _ = peak_hbm()
    out["ic1024"] = {"ms_per_ic": ms1k, "ic_per_s": 1e3 / ms1k, "pk_bins": 256,
                     "pk_finite_bins": int(np.isfinite(r1k["pk_p"]).sum()),
                     "roofline": {"model_bytes": 37 * G1k, "GBps": 37 * G1k / (ms1k / 1e3) / 1e9,
                                  "frac": 37 * G1k / (ms1k / 1e3) / 1e9 / peak}}
    ml.load().mitos_release_all()

    # N-GenIC-like field (src/grf_ngeniclike.c) at 512^3
    g = ml.alloc_local_grid(N, L, ml.FP32)
    ml.generate_ngeniclike_grf_dg(g, 1)
    ml.timer_start()
    ml.generate_ngeniclike_grf_dg(g, 2)
    out["ngeniclike_ms"] = ml.timer_stop()
    ml.free_local_grid(g)
    return out


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--N", type=int, default=512)
    ap.add_argument("--boxlen", type=float, default=1000.0)
    ap.add_argument("--bins", type=int, default=128)
    ap.add_argument("--seed", type=int, default=42)
    ap.add_argument("--precision", default="fp32", choices=["fp32", "fp64"])
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-extras", action="store_true",
                    help="skip the FP64, ensemble, Monge-Ampere and N-GenIC measurements")
    ap.add_argument("--quick", action="store_true",
                    help="timed steps only (no e2e, per-kernel timing or CPU baseline): the profiling run")
    args = ap.parse_args()
    args.warmup = max(args.warmup, 3)
    if args.impl == "reference":
        return run_reference(args)

    ws, rank, local = dist_setup()
    dist = None
    if ws > 1:
        import torch
        import torch.distributed as td
        torch.cuda.set_device(local)
        td.init_process_group("nccl" if torch.cuda.is_available() else "gloo")
        dist = td

    import mitos_gb300.lib as ml
    from mitos_gb300.perturb import load_table
    table = load_table()
    spline = ml.Spline(table)
    prec = ml.FP32 if args.precision == "fp32" else ml.FP64
    N = args.N
    seed0 = replica_seed(args.seed, rank)

    def cfg(step):
        return ml.ic_config(N, N, args.boxlen, seed0 + step, table, method=ml.METHOD_2LPT,
                            pk_bins=args.bins, pk_linear=True, precision=prec)

    L = ml.load()
    bins = args.bins
    kb, pb, ob = np.zeros(bins), np.zeros(bins), np.zeros(bins, np.int64)
    res = ml.ICResult(kb.ctypes.data_as(ml._dp), pb.ctypes.data_as(ml._dp), ob.ctypes.data_as(ml._lp),
                      None, 0, 0.0)

    def step(i, with_pos=None):
        c = cfg(i)
        res.pos = with_pos
        ml._check(L.ic_pipeline_run(ctypes.byref(c), ctypes.byref(spline.sp), ctypes.byref(res)))

    def barrier():
        L.mitos_sync()
        if dist:
            dist.barrier()

    for i in range(args.warmup):
        step(i)
    launches0 = ml.launch_count()
    clocks = Clocks(local)
    clocks.start()
    barrier()
    clocks.mark(True)
    ml.timer_start()
    for i in range(args.steps):
        step(args.warmup + i)
    ms = ml.timer_stop()
    barrier()
    clocks.mark(False)
    clk = clocks.stop()
    launches = (ml.launch_count() - launches0) // args.steps
    ms = max_over_ranks(ms, dist)
    ms_per_step = ms / args.steps
    value = job_throughput(ws, args.steps, ms / 1e3)
    if args.quick:
        if rank == 0:
            print(json.dumps({"metric": METRIC, "value": value, "unit": UNIT, "ms_per_step": ms_per_step,
                              "config": config(args), "clocks": clk, "quick": True}), flush=True)
        return 0

    # e2e: every step's positions (the IC product, 1.6 GB) to pinned host memory, the table up and
    # P(k) down, through ic_pipeline_submit: two pinned position buffers alternate, so one IC's
    # positions cross the link while the next computes; the clock stops after ic_pipeline_wait
    import torch
    npart = N ** 3
    pinned = [torch.empty((npart, 3), dtype=torch.float32, pin_memory=True) for _ in range(2)]
    pos_ptrs = [ctypes.cast(p.data_ptr(), ml._fp) for p in pinned]
    outs = []
    for i in range(args.steps):
        k_, p_, o_ = np.zeros(bins), np.zeros(bins), np.zeros(bins, np.int64)
        outs.append((k_, p_, o_, ml.ICResult(k_.ctypes.data_as(ml._dp), p_.ctypes.data_as(ml._dp),
                                             o_.ctypes.data_as(ml._lp), pos_ptrs[i % 2], 0, 0.0)))
    # the host link's device-to-host rate into the same pinned buffer (one 1.6 GB copy, best of 3;
    # e2e is bound by it once the kernels take less than a copy)
    link = []
    dsrc = torch.empty((npart, 3), dtype=torch.float32, device="cuda")
    cs = torch.cuda.Stream()
    for _ in range(3):
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(cs)
        with torch.cuda.stream(cs):
            pinned[0].copy_(dsrc, non_blocking=True)
        e1.record(cs)
        cs.synchronize()
        link.append(npart * 12 / (e0.elapsed_time(e1) / 1e3) / 1e9)
    del dsrc
    link_gbps = max(link)
    # warm-up: one submission into each pinned buffer (their first transfers are slow)
    warm = [(np.zeros(bins), np.zeros(bins), np.zeros(bins, np.int64)) for _ in range(2)]
    for j, (k_, p_, o_) in enumerate(warm):
        r_ = ml.ICResult(k_.ctypes.data_as(ml._dp), p_.ctypes.data_as(ml._dp), o_.ctypes.data_as(ml._lp),
                         pos_ptrs[j], 0, 0.0)
        warm[j] = (k_, p_, o_, r_)
        ml.ic_pipeline_submit(cfg(j), spline, r_)
    ml.ic_pipeline_wait()
    barrier()
    t0 = time.perf_counter()
    for i in range(args.steps):
        ml.ic_pipeline_submit(cfg(args.warmup + i), spline, outs[i][3])
    ml.ic_pipeline_wait()
    barrier()
    e2e_s = max_over_ranks(time.perf_counter() - t0, dist)
    e2e_val = job_throughput(ws, args.steps, e2e_s)
    assert all(np.isfinite(o[1][1:]).all() for o in outs[:args.steps])

    # per-kernel durations of one IC (roofline of the dominant kernel)
    # per-kernel durations: the mean over three ICs
    KT_ICS = 3
    ml.kernel_timing(True)
    for i in range(KT_ICS):
        step(i)
    kt = ml.kernel_times()
    ml.kernel_timing(False)
    G = N * N * (N // 2 + 1) * (8 if prec == ml.FP32 else 16)
    agg = {}
    for name, t in kt:
        a = agg.setdefault(name, [0.0, 0])
        a[0] += t
        a[1] += 1
    dom = max(agg, key=lambda k: agg[k][0])
    dom_ms = agg[dom][0] / agg[dom][1]
    peak, peak_kind = peak_hbm()
    achieved = algorithmic_bytes(dom, G) / (dom_ms / 1e3) / 1e9
    traffic = ncu_traffic(dom, N)
    kernels = {k: {"ms": round(v[0] / v[1], 4), "launches": v[1] // KT_ICS,
                   "GBps": round(algorithmic_bytes(k, G) / (v[0] / v[1] / 1e3) / 1e9, 1) if algorithmic_bytes(k, G) else None}
               for k, v in sorted(agg.items(), key=lambda kv: -kv[1][0])}
    alg_ic = 37 * G  # byte model per IC with two-pass FFTs, (15 + 22 (P - 1)) G
    if rank != 0:
        return 0
    line = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": ws, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": ms_per_step, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32" if prec == ml.FP32 else "f64",
            "data": "synthetic (xoshiro256** white noise, BBKS transfer table)", "config": config(args),
            "gpu_launches": int(launches),
            "e2e": {"value": e2e_val, "unit": UNIT, "h2d_bytes_per_step": 3 * table.k_size * 8,
                    "d2h_bytes_per_step": npart * 12 + 3 * bins * 8, "link_d2h_GBps": link_gbps,
                    "link_bound_IC_per_s": link_gbps * 1e9 / (npart * 12)},
            "roofline": {"bound": "hbm", "kernel": dom, "achieved": achieved, "peak": peak,
                         "unit": "GB/s", "frac": achieved / peak, "peak_source": peak_kind,
                         "traffic": traffic, "algorithmic_bytes": algorithmic_bytes(dom, G),
                         "ms": dom_ms},
            "ic_hbm": {"model_bytes": alg_ic, "GBps": alg_ic / (ms_per_step / 1e3) / 1e9,
                       "frac": alg_ic / (ms_per_step / 1e3) / 1e9 / peak},
            "kernels": kernels, "clocks": clk}
    if not args.no_extras and N == 512 and prec == ml.FP32:
        line["extras"] = extras(ml, table, spline, args)
    noise = gpu_noise(ml) if not args.no_cpu_baseline else None
    if not args.no_cpu_baseline:
        base, _ = cpu_baseline(args, table, steps=1)
        line["cpu_baseline"] = base
        if noise is not None:
            line["noise_exact"] = noise_exactness(ml, noise)
    print(json.dumps(line), flush=True)
    if dist:
        dist.destroy_process_group()
    return 0


if __name__ == "__main__":
    sys.exit(main())
