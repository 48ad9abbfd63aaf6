"""ctypes mirror of the C ABI in include/mitos_gb300.h.

The names and argument meanings follow the reference entry points (alloc_local_grid,
fft_r2c_dg, fft_c2r_dg, fft_apply_kernel_dg, generate_complex_grf, enforce_hermiticity,
solvePoisson_dg, solve2LPT, solveMongeAmpere, calc_cross_powerspec, ...).  A non-zero status
raises MitosError with the library's description.  The CUDA library is required: importing
this module on a machine without it, or calling into it without a GPU, fails loudly.
"""
from __future__ import annotations

import ctypes
import os

import numpy as np

from . import build as _build

FP64 = 0
FP32 = 1
METHOD_ZELDOVICH = 1
METHOD_2LPT = 2
METHOD_MONGE_AMPERE = 3

_dp = ctypes.POINTER(ctypes.c_double)
_fp = ctypes.POINTER(ctypes.c_float)
_lp = ctypes.POINTER(ctypes.c_long)
_ip = ctypes.POINTER(ctypes.c_int)


class MitosError(RuntimeError):
    def __init__(self, code: int, msg: str):
        super().__init__(f"mitos_gb300 status {code}: {msg}")
        self.code = code


class DistributedGrid(ctypes.Structure):
    _fields_ = [("N", ctypes.c_int), ("boxlen", ctypes.c_double), ("comm", ctypes.c_void_p),
                ("momentum_space", ctypes.c_char), ("NX", ctypes.c_long), ("X0", ctypes.c_long),
                ("local_size", ctypes.c_long), ("fbox", ctypes.c_void_p), ("box", ctypes.c_void_p),
                ("precision", ctypes.c_int), ("flags", ctypes.c_int), ("priv", ctypes.c_void_p)]


class RngState(ctypes.Structure):
    _fields_ = [("s", ctypes.c_uint64 * 4)]


class Kernel(ctypes.Structure):
    _fields_ = [("kx", ctypes.c_double), ("ky", ctypes.c_double), ("kz", ctypes.c_double),
                ("k", ctypes.c_double), ("kern", ctypes.c_double * 2), ("params", ctypes.c_void_p)]


class Cosmology(ctypes.Structure):
    _fields_ = [(n, ctypes.c_double) for n in
                ("h", "n_s", "A_s", "k_pivot", "z_ini", "log_tau_ini", "rho_crit", "z_source",
                 "log_tau_source")]


class PerturbData(ctypes.Structure):
    _fields_ = [("k_size", ctypes.c_int), ("tau_size", ctypes.c_int), ("n_functions", ctypes.c_int),
                ("delta", _dp), ("k", _dp), ("log_tau", _dp), ("redshift", _dp), ("D_growth", _dp),
                ("f_growth", _dp), ("H_Hubble", _dp), ("titles", ctypes.POINTER(ctypes.c_char_p)),
                ("Omega", _dp)]


class PerturbSpline(ctypes.Structure):
    _fields_ = [("ptdat", ctypes.POINTER(PerturbData)), ("k_acc_table", _dp),
                ("k_acc_table_size", ctypes.c_int)]


class SplineParams(ctypes.Structure):
    _fields_ = [("spline", ctypes.POINTER(PerturbSpline)), ("index_src", ctypes.c_int),
                ("tau_index", ctypes.c_int), ("u_tau", ctypes.c_double)]


class HermiteParams(ctypes.Structure):
    _fields_ = [("order", ctypes.c_int), ("N", ctypes.c_int), ("boxlen", ctypes.c_double)]


class ICConfig(ctypes.Structure):
    _fields_ = [("N", ctypes.c_int), ("M", ctypes.c_int), ("boxlen", ctypes.c_double),
                ("seed", ctypes.c_uint64), ("A_s", ctypes.c_double), ("n_s", ctypes.c_double),
                ("k_pivot", ctypes.c_double), ("z_ini", ctypes.c_double), ("index_src", ctypes.c_int),
                ("method", ctypes.c_int), ("ma_cycles", ctypes.c_int), ("ma_tol", ctypes.c_double),
                ("pk_bins", ctypes.c_int), ("pk_linear", ctypes.c_int), ("precision", ctypes.c_int),
                ("keep_outputs", ctypes.c_int), ("index_vel", ctypes.c_int),
                ("thermal", ctypes.c_int), ("thermal_M_eV", ctypes.c_double),
                ("thermal_T_eV", ctypes.c_double), ("speed_of_light", ctypes.c_double),
                ("thermal_draw_offset", ctypes.c_uint64),
                ("particle_mass", ctypes.c_double), ("id_first_particle", ctypes.c_longlong)]


class Interval(ctypes.Structure):
    """struct interval (include/random.h:43-51)"""
    _fields_ = [("id", ctypes.c_int), ("l", ctypes.c_double), ("r", ctypes.c_double),
                ("Fl", ctypes.c_double), ("Fr", ctypes.c_double), ("a0", ctypes.c_double),
                ("a1", ctypes.c_double), ("a2", ctypes.c_double), ("a3", ctypes.c_double),
                ("error", ctypes.c_double), ("nid", ctypes.c_int)]


class Sampler(ctypes.Structure):
    """struct sampler (include/random.h:54-81)"""
    _fields_ = [("norm", ctypes.c_double), ("xl", ctypes.c_double), ("xr", ctypes.c_double),
                ("f", ctypes.c_void_p), ("params", ctypes.c_void_p),
                ("intervals", ctypes.POINTER(Interval)), ("intervalNum", ctypes.c_int),
                ("I_max", ctypes.c_int), ("index", _dp)]


FERMION, BOSON = 1, 2


class ICResult(ctypes.Structure):
    _fields_ = [("pk_k", _dp), ("pk_p", _dp), ("pk_obs", _lp), ("pos", _fp),
                ("ma_iterations", ctypes.c_int), ("ma_residual", ctypes.c_double), ("vel", _fp),
                ("coords", _dp), ("vels", _dp), ("masses", _dp), ("ids", ctypes.POINTER(ctypes.c_longlong))]


_lib = None

KERNEL_NAMES = ["constant", "lowpass", "hipass", "tophat", "elliptic_tophat", "translate",
                "gaussian", "gaussian_inv", "inv_poisson", "dx", "dy", "dz", "power_no_transfer",
                "transfer_function", "inv_transfer_function", "undo_Hermite_window"]

# every symbol include/mitos_gb300.h declares
EXPORTS = ["alloc_local_grid", "free_local_grid", "free_local_real_grid", "free_local_complex_grid",
           "fft_wavevector", "fft_r2c_dg", "fft_c2r_dg", "fft_apply_kernel_dg",
           "generate_complex_grf", "enforce_hermiticity", "generatePerturbationGrid",
           "solvePoisson_dg", "solve2LPT", "solveMongeAmpere", "calc_cross_powerspec",
           "calc_cross_powerspec_float", "calc_cross_powerspec_float_mpi", "mitos_set_precision",
           "mitos_get_precision", "alloc_local_grid_prec", "dg_copy_to_host", "dg_copy_from_host",
           "mitos_last_error", "mitos_launch_count", "mitos_release_all", "cic_deposit_dg",
           "ic_pipeline_run", "ic_pipeline_run_table", "mitos_timer_start", "mitos_timer_stop",
           "mitos_sync", "mitos_kernel_timing", "mitos_kernel_times", "mitos_stage_times",
           "mitos_ma_history", "mitos_rng_jump", "mitos_noise_column_state", "mitos_cr_log", "mitos_cr_cos",
           "mitos_sample_norm_cr", "mitos_cr_steps", "snapshot_header_attributes", "manet_set_warm_grid", "mitos_set_radix", "mitos_get_radix", "mitos_set_cluster_fft", "mitos_set_lattice_tma", "mitos_set_lattice_order", "mitos_set_stream"] + \
          ["kernel_" + k for k in KERNEL_NAMES]


def lib_path() -> str:
    return _build.LIB


def load(build_if_missing: bool = True):
    """Load the CUDA library (building it first when missing)."""
    global _lib
    if _lib is not None:
        return _lib
    path = _build.LIB
    if not os.path.exists(path):
        if not build_if_missing:
            raise MitosError(4, f"{path} is missing; run mitos_gb300.build.build()")
        _build.build()
    L = ctypes.CDLL(path)
    L.mitos_last_error.restype = ctypes.c_char_p
    L.mitos_timer_stop.restype = ctypes.c_double
    L.mitos_launch_count.restype = ctypes.c_long
    _lib = L
    return L


def _check(status: int) -> None:
    if status != 0:
        raise MitosError(status, load().mitos_last_error().decode())


def last_error() -> str:
    return load().mitos_last_error().decode()


def launch_count() -> int:
    return int(load().mitos_launch_count())


def set_precision(p: int) -> None:
    _check(load().mitos_set_precision(p))


# ---- grids ---------------------------------------------------------------------------------
def alloc_local_grid(N: int, boxlen: float, precision: int = FP64) -> DistributedGrid:
    dg = DistributedGrid()
    _check(load().alloc_local_grid_prec(ctypes.byref(dg), N, ctypes.c_double(boxlen), None, precision))
    return dg


def free_local_grid(dg: DistributedGrid) -> None:
    _check(load().free_local_grid(ctypes.byref(dg)))


def _ctype(dg):
    return (np.complex64, np.float32) if dg.precision == FP32 else (np.complex128, np.float64)


def get_fbox(dg: DistributedGrid) -> np.ndarray:
    c, _ = _ctype(dg)
    out = np.empty((dg.N, dg.N, dg.N // 2 + 1), c)
    _check(load().dg_copy_to_host(ctypes.byref(dg), 0, out.ctypes.data_as(ctypes.c_void_p)))
    return out


def get_box(dg: DistributedGrid) -> np.ndarray:
    _, r = _ctype(dg)
    out = np.empty((dg.N, dg.N, dg.N + 2), r)
    _check(load().dg_copy_to_host(ctypes.byref(dg), 1, out.ctypes.data_as(ctypes.c_void_p)))
    return out


def set_fbox(dg: DistributedGrid, a: np.ndarray, momentum_space: bool = True) -> None:
    c, _ = _ctype(dg)
    a = np.ascontiguousarray(a, dtype=c).reshape(dg.N, dg.N, dg.N // 2 + 1)
    _check(load().dg_copy_from_host(ctypes.byref(dg), 0, a.ctypes.data_as(ctypes.c_void_p)))
    dg.momentum_space = b"\x01" if momentum_space else b"\x00"


def set_box(dg: DistributedGrid, a: np.ndarray) -> None:
    _, r = _ctype(dg)
    a = np.ascontiguousarray(a, dtype=r)
    if a.shape[-1] == dg.N:
        a = np.concatenate([a, np.zeros(a.shape[:-1] + (2,), r)], axis=-1)
    a = np.ascontiguousarray(a).reshape(dg.N, dg.N, dg.N + 2)
    _check(load().dg_copy_from_host(ctypes.byref(dg), 1, a.ctypes.data_as(ctypes.c_void_p)))
    dg.momentum_space = b"\x00"


# ---- FFT and kernels -----------------------------------------------------------------------
def fft_r2c_dg(dg):
    _check(load().fft_r2c_dg(ctypes.byref(dg)))


def fft_c2r_dg(dg):
    _check(load().fft_c2r_dg(ctypes.byref(dg)))


def kernel_fn(name: str):
    return ctypes.cast(getattr(load(), "kernel_" + name), ctypes.c_void_p)


def fft_apply_kernel_dg(w, r, kernel: str, params=None) -> int:
    """Returns the status (does not raise) so that the error paths can be tested."""
    L = load()
    if params is None:
        pp = None
    elif isinstance(params, ctypes.Structure):
        pp = ctypes.cast(ctypes.byref(params), ctypes.c_void_p)
    else:
        arr = (ctypes.c_double * len(np.atleast_1d(params)))(*np.atleast_1d(params).tolist())
        pp = ctypes.cast(arr, ctypes.c_void_p)
        fft_apply_kernel_dg._keep = arr
    fn = kernel_fn(kernel) if isinstance(kernel, str) else kernel
    return L.fft_apply_kernel_dg(ctypes.byref(w), ctypes.byref(r), fn, pp)


def rng_init(seed: int) -> RngState:
    """splitmix64 seeding of xoshiro256** (include/random_xorshift.h:49-59), host side."""
    s = RngState()
    st = seed & 0xFFFFFFFFFFFFFFFF
    for i in range(4):
        r = st
        st = (r + 0x9E3779B97F4A7C15) & 0xFFFFFFFFFFFFFFFF
        r = ((r ^ (r >> 30)) * 0xBF58476D1CE4E5B9) & 0xFFFFFFFFFFFFFFFF
        r = ((r ^ (r >> 27)) * 0x94D049BB133111EB) & 0xFFFFFFFFFFFFFFFF
        s.s[i] = r ^ (r >> 31)
    return s


def generate_complex_grf(dg, state: RngState):
    _check(load().generate_complex_grf(ctypes.byref(dg), ctypes.byref(state)))


def enforce_hermiticity(dg):
    _check(load().enforce_hermiticity(ctypes.byref(dg)))


def solvePoisson_dg(dg):
    _check(load().solvePoisson_dg(ctypes.byref(dg)))


def solve2LPT(pot, dens, work, f1=1.0, f2=-3.0 / 7.0):
    _check(load().solve2LPT(ctypes.byref(pot), ctypes.byref(dens), ctypes.byref(work),
                            ctypes.c_double(f1), ctypes.c_double(f2)))


def solveMongeAmpere(pot, dens, work, cycles: int):
    _check(load().solveMongeAmpere(ctypes.byref(pot), ctypes.byref(dens), ctypes.byref(work), cycles))


def ma_history(max_cycles: int = 256):
    eps = np.zeros(max_cycles)
    rel = np.zeros(max_cycles)
    n = load().mitos_ma_history(eps.ctypes.data_as(_dp), rel.ctypes.data_as(_dp), max_cycles)
    return eps[:n], rel[:n]


def calc_cross_powerspec(N, boxlen, f1, f2, bins, precision=FP64):
    """f1, f2: host numpy complex arrays or DistributedGrid (device fbox)."""
    L = load()
    k = np.zeros(bins)
    p = np.zeros(bins)
    o = np.zeros(bins, np.int32)

    def ptr(x, c):
        if isinstance(x, DistributedGrid):
            return ctypes.c_void_p(x.fbox)
        x = np.ascontiguousarray(x, dtype=c)
        ptr._keep.append(x)
        return x.ctypes.data_as(ctypes.c_void_p)
    ptr._keep = []
    c = np.complex64 if precision == FP32 else np.complex128
    fn = L.calc_cross_powerspec_float if precision == FP32 else L.calc_cross_powerspec
    fn(N, ctypes.c_double(boxlen), ptr(f1, c), ptr(f2, c), bins, k.ctypes.data_as(_dp),
       p.ctypes.data_as(_dp), o.ctypes.data_as(_ip))
    return k, p, o


# ---- perturbation table ----------------------------------------------------------------------
class Spline:
    """struct perturb_data + struct perturb_spline over a PerturbTable (arrays kept alive)."""

    def __init__(self, table):
        self.arrays = [np.ascontiguousarray(a, np.float64) for a in
                       (table.delta, table.k, table.log_tau, table.redshift, table.D_growth,
                        table.f_growth, table.H_Hubble)]
        self.titles = (ctypes.c_char_p * table.n_functions)(*[t.encode() for t in table.titles])
        d, k, lt, z, D, f, H = [a.ctypes.data_as(_dp) for a in self.arrays]
        self.pd = PerturbData(table.k_size, table.tau_size, table.n_functions, d, k, lt, z, D, f, H,
                              self.titles, None)
        self.sp = PerturbSpline(ctypes.pointer(self.pd), None, 0)
        self.table = table

    def tau_params(self, z: float):
        t = self.table
        lt = np.interp(z, t.redshift[::-1], t.log_tau[::-1])
        return lt


def generatePerturbationGrid(cosmo: Cosmology, spline: Spline, grf, grid, title: str,
                             rescale: float = 1.0):
    _check(load().generatePerturbationGrid(ctypes.byref(cosmo), ctypes.byref(spline.sp),
                                           ctypes.byref(grf), ctypes.byref(grid), title.encode(),
                                           b"", ctypes.c_double(rescale)))


def cic_deposit_dg(rho, pos: np.ndarray, mass: float) -> float:
    pos = np.ascontiguousarray(pos, np.float32)
    tot = ctypes.c_double()
    _check(load().cic_deposit_dg(ctypes.byref(rho), pos.ctypes.data_as(_fp), ctypes.c_long(len(pos)),
                                 ctypes.c_double(mass), ctypes.byref(tot)))
    return tot.value


# ---- fused pipeline --------------------------------------------------------------------------
def ic_config(N, M, boxlen, seed, table, method=METHOD_2LPT, pk_bins=32, pk_linear=True,
              precision=FP32, z_ini=31.0, ma_cycles=0, ma_tol=0.0, index_src=0, index_vel=None,
              thermal=0, thermal_M_eV=0.0, thermal_T_eV=0.0, speed_of_light=0.0,
              thermal_draw_offset=0, particle_mass=1.0, id_first_particle=0) -> ICConfig:
    """index_vel: the velocity transfer function (default: the table's ``t_cdm`` when it has one);
    thermal: FERMION or BOSON adds thermal motion to the velocities (0: none)"""
    if index_vel is None:
        index_vel = table.index_of("t_cdm") if "t_cdm" in getattr(table, "titles", []) else -1
    return ICConfig(N, M, boxlen, seed, table.A_s, table.n_s, table.k_pivot, z_ini, index_src,
                    method, ma_cycles, ma_tol, pk_bins, int(pk_linear), precision, 0, index_vel,
                    int(thermal), thermal_M_eV, thermal_T_eV, speed_of_light, thermal_draw_offset,
                    particle_mass, id_first_particle)


def thermal_sampler(kind: int, T_eV: float) -> Sampler:
    """thermal_sampler_init: the inverse-CDF sampler of fd_pdf (FERMION) or be_pdf (BOSON)"""
    s = Sampler()
    _check(load().thermal_sampler_init(ctypes.byref(s), int(kind), ctypes.c_double(T_eV)))
    return s


def thermal_sampler_free(s: Sampler) -> None:
    load().thermal_sampler_free(ctypes.byref(s))


def sampler_rows(s: Sampler) -> np.ndarray:
    """the sampler's pieces as rows [l r Fl Fr a0 a1 a2 a3]"""
    rows = np.zeros((s.intervalNum, 8))
    for j in range(s.intervalNum):
        iv = s.intervals[j]
        rows[j] = (iv.l, iv.r, iv.Fl, iv.Fr, iv.a0, iv.a1, iv.a2, iv.a3)
    return rows


def sampler_index(s: Sampler) -> np.ndarray:
    return np.array([s.index[i] for i in range(s.I_max)], dtype=np.int64)


def thermal_velocities(s: Sampler, state: np.ndarray, vel, M_eV: float, a_ini: float, c: float,
                       stride: int = 3, n: int | None = None, offset: int = 0) -> np.ndarray:
    """thermal_velocities on vel (host float32 array or a device tensor, updated in place): n particles
    (default: size // stride) whose components start at float `offset` and lie `stride` floats apart;
    state (four uint64) is advanced by 7 n draws.  Returns the new state."""
    st = RngState()
    for i in range(4):
        st.s[i] = int(state[i])
    if hasattr(vel, "data_ptr"):
        n = vel.numel() // stride if n is None else n
        ptr = ctypes.cast(vel.data_ptr() + 4 * offset, _fp)
    else:
        assert vel.dtype == np.float32 and vel.flags.c_contiguous
        n = vel.size // stride if n is None else n
        ptr = ctypes.cast(vel.ctypes.data + 4 * offset, _fp)
    _check(load().thermal_velocities(ctypes.byref(s), ctypes.byref(st), ctypes.c_long(n), ctypes.c_double(M_eV),
                                     ctypes.c_double(a_ini), ctypes.c_double(c), ptr, ctypes.c_long(stride)))
    return np.array([st.s[i] for i in range(4)], dtype=np.uint64)


def calc_bispectrum(g, bins, bins3, volume_mode=False, btype=0, theta=0.0, k3=0.0) -> dict:
    """calc_bispectrum_dg on a momentum-space grid (either precision)"""
    k1, k2, k3o, b = (np.zeros(bins) for _ in range(4))
    _check(load().calc_bispectrum_dg(ctypes.byref(g), bins, bins3, k1.ctypes.data_as(_dp), k2.ctypes.data_as(_dp),
                                     k3o.ctypes.data_as(_dp), b.ctypes.data_as(_dp), int(volume_mode), int(btype),
                                     ctypes.c_double(theta), ctypes.c_double(k3)))
    return {"k1": k1, "k2": k2, "k3": k3o, "B": b}


def ic_pipeline_run(cfg: ICConfig, spline: Spline, want_pos: bool = False, want_vel: bool = False,
                    want_snapshot: bool = False) -> dict:
    """want_snapshot: the snapshot datasets coords, vels (with index_vel), masses and ids"""
    bins = cfg.pk_bins
    k = np.zeros(bins)
    p = np.zeros(bins)
    o = np.zeros(bins, np.int64)
    n = cfg.M ** 3
    pos = np.zeros((n, 3), np.float32) if want_pos else None
    vel = np.zeros((n, 3), np.float32) if want_vel else None
    snap = {}
    if want_snapshot:
        snap = {"coords": np.zeros((n, 3)), "masses": np.zeros(n), "ids": np.zeros(n, np.int64)}
        if cfg.index_vel >= 0:
            snap["vels"] = np.zeros((n, 3))
    res = ICResult(k.ctypes.data_as(_dp), p.ctypes.data_as(_dp), o.ctypes.data_as(_lp),
                   pos.ctypes.data_as(_fp) if pos is not None else None, 0, 0.0,
                   vel.ctypes.data_as(_fp) if vel is not None else None)
    if snap:
        res.coords = snap["coords"].ctypes.data_as(_dp)
        res.masses = snap["masses"].ctypes.data_as(_dp)
        res.ids = snap["ids"].ctypes.data_as(ctypes.POINTER(ctypes.c_longlong))
        if "vels" in snap:
            res.vels = snap["vels"].ctypes.data_as(_dp)
    _check(load().ic_pipeline_run(ctypes.byref(cfg), ctypes.byref(spline.sp), ctypes.byref(res)))
    out = {"pk_k": k, "pk_p": p, "pk_obs": o, "ma_iterations": res.ma_iterations,
           "ma_residual": res.ma_residual}
    if pos is not None:
        out["pos"] = pos
    if vel is not None:
        out["vel"] = vel
    out.update(snap)
    return out


class SnapshotHeader(ctypes.Structure):
    _fields_ = [("BoxSize", ctypes.c_double * 3), ("Dimension", ctypes.c_int), ("Redshift", ctypes.c_double),
                ("Flag_Entropy_ICs", ctypes.c_int), ("NumFilesPerSnapshot", ctypes.c_int),
                ("NumPart_Total", ctypes.c_long * 7), ("NumPart_Total_HighWord", ctypes.c_long * 7),
                ("MassTable", ctypes.c_double * 7), ("Cosmology_Redshift", ctypes.c_double),
                ("Unit_mass_cgs", ctypes.c_double), ("Unit_length_cgs", ctypes.c_double),
                ("Unit_time_cgs", ctypes.c_double), ("Unit_temperature_cgs", ctypes.c_double),
                ("Unit_current_cgs", ctypes.c_double)]


# (group, attribute name) of writeHeaderAttributes (src/header.c:26-175) -> SnapshotHeader field
HEADER_ATTRIBUTES = {
    ("/Header", "BoxSize"): "BoxSize", ("/Header", "Dimension"): "Dimension",
    ("/Header", "Redshift"): "Redshift", ("/Header", "Flag_Entropy_ICs"): "Flag_Entropy_ICs",
    ("/Header", "NumFilesPerSnapshot"): "NumFilesPerSnapshot", ("/Header", "NumPart_Total"): "NumPart_Total",
    ("/Header", "NumPart_Total_HighWord"): "NumPart_Total_HighWord", ("/Header", "MassTable"): "MassTable",
    ("/Cosmology", "Redshift"): "Cosmology_Redshift",
    ("/Units", "Unit mass in cgs (U_M)"): "Unit_mass_cgs", ("/Units", "Unit length in cgs (U_L)"): "Unit_length_cgs",
    ("/Units", "Unit time in cgs (U_t)"): "Unit_time_cgs",
    ("/Units", "Unit temperature in cgs (U_T)"): "Unit_temperature_cgs",
    ("/Units", "Unit current in cgs (U_I)"): "Unit_current_cgs"}


def snapshot_header(boxlen: float, z_ini: float, types, units) -> dict:
    """types: [(ExportName, TotalNumber)]; units: (kg, m, s, K, A) of the internal unit system.
    Returns {(group, name): list of values} as writeHeaderAttributes writes them."""
    n = len(types)
    names = (ctypes.c_char_p * max(n, 1))(*[t[0].encode() for t in types])
    tot = (ctypes.c_longlong * max(n, 1))(*[int(t[1]) for t in types])
    h = SnapshotHeader()
    _check(load().snapshot_header_attributes(ctypes.c_double(boxlen), ctypes.c_double(z_ini), n, names, tot,
                                             *[ctypes.c_double(u) for u in units], ctypes.byref(h)))
    out = {}
    for key, f in HEADER_ATTRIBUTES.items():
        v = getattr(h, f)
        out[key] = list(v) if hasattr(v, "__len__") else [v]
    return out


def field_to_host(dg) -> np.ndarray:
    """dg_field_to_host: the /Field/Field dataset (N, N, N + 2) doubles of a real-space grid"""
    out = np.zeros((dg.N, dg.N, dg.N + 2))
    _check(load().dg_field_to_host(ctypes.byref(dg), out.ctypes.data_as(_dp)))
    return out


def stage_times() -> np.ndarray:
    ms = np.zeros(16)
    n = load().mitos_stage_times(ms.ctypes.data_as(_dp), 16)
    return ms[:n]


def timer_start() -> None:
    _check(load().mitos_timer_start())


def timer_stop() -> float:
    return float(load().mitos_timer_stop())


def kernel_timing(on: bool) -> None:
    load().mitos_kernel_timing(int(on))


def kernel_times(max_n: int = 4096):
    names = (ctypes.c_char_p * max_n)()
    ms = np.zeros(max_n)
    n = load().mitos_kernel_times(names, ms.ctypes.data_as(_dp), max_n)
    return [(names[i].decode(), float(ms[i])) for i in range(n)]


# ---- learned Monge-Ampere warm start -------------------------------------------------------
MANET_PARAMS = 27712


class Manet(ctypes.Structure):
    """struct manet: input / output scales, Adam step count, device state."""
    _fields_ = [("scale_in", ctypes.c_float * 3), ("scale_out", ctypes.c_float), ("steps", ctypes.c_int),
                ("priv", ctypes.c_void_p)]


def _vp(p):
    """a device pointer from an int, a c_void_p, or a DistributedGrid (its real box)"""
    if isinstance(p, DistributedGrid):
        return ctypes.c_void_p(p.box)
    if isinstance(p, ctypes.c_void_p):
        return p
    return ctypes.c_void_p(int(p))


def manet_init(seed: int = 1) -> Manet:
    net = Manet()
    _check(load().manet_init(ctypes.byref(net), ctypes.c_ulonglong(seed)))
    return net


def manet_free(net: Manet) -> None:
    load().manet_free(ctypes.byref(net))


def manet_params(net: Manet) -> np.ndarray:
    out = np.zeros(MANET_PARAMS, np.float32)
    _check(load().manet_get_params(ctypes.byref(net), out.ctypes.data_as(_fp)))
    return out


def manet_set_params(net: Manet, p: np.ndarray) -> None:
    p = np.ascontiguousarray(p, np.float32)
    assert p.size == MANET_PARAMS
    _check(load().manet_set_params(ctypes.byref(net), p.ctypes.data_as(_fp)))


def manet_grads(net: Manet) -> np.ndarray:
    out = np.zeros(MANET_PARAMS, np.float32)
    _check(load().manet_get_grads(ctypes.byref(net), out.ctypes.data_as(_fp)))
    return out


def manet_loss_grad(net: Manet, N: int, pitch: int, delta, phi1, phi2, target) -> float:
    loss = ctypes.c_double(0)
    _check(load().manet_loss_grad(ctypes.byref(net), N, pitch, _vp(delta), _vp(phi1), _vp(phi2), _vp(target),
                                  ctypes.byref(loss)))
    return loss.value


def manet_train_step(net: Manet, N: int, pitch: int, delta, phi1, phi2, target, lr: float) -> float:
    loss = ctypes.c_double(0)
    _check(load().manet_train_step(ctypes.byref(net), N, pitch, _vp(delta), _vp(phi1), _vp(phi2), _vp(target),
                                   ctypes.c_float(lr), ctypes.byref(loss)))
    return loss.value


def manet_infer(net: Manet, N: int, pitch: int, delta, phi1, phi2, out) -> None:
    _check(load().manet_infer(ctypes.byref(net), N, pitch, _vp(delta), _vp(phi1), _vp(phi2), _vp(out)))


def manet_set_warm_grid(net: Manet, Nw: int) -> None:
    """run the warm start's network on an Nw grid (0: the solve's own grid)"""
    _check(load().manet_set_warm_grid(ctypes.byref(net), Nw))


def manet_layers(p: np.ndarray):
    """split a parameter vector into per-layer (w[27][16][16], b[16]) arrays"""
    ppl = MANET_PARAMS // 4
    return [(p[l * ppl:l * ppl + 27 * 256].reshape(27, 16, 16), p[l * ppl + 27 * 256:(l + 1) * ppl])
            for l in range(4)]


class MAStats(ctypes.Structure):
    _fields_ = [("cycles", ctypes.c_int), ("evaluations", ctypes.c_int), ("rel", ctypes.c_double),
                ("eps", ctypes.c_double), ("rel_first", ctypes.c_double), ("rel_second", ctypes.c_double),
                ("ms", ctypes.c_double), ("ms_warm", ctypes.c_double)]

    def as_dict(self) -> dict:
        return {n: getattr(self, n) for n, _ in self._fields_}


def solveMongeAmpereTol(pot, dens, work, tol: float, max_cycles: int, net: Manet | None = None) -> dict:
    """Monge-Ampere to a relative rms residual tol; returns the statistics (converged: status 0)."""
    st = MAStats()
    s = load().solveMongeAmpereTol(ctypes.byref(pot), ctypes.byref(dens), ctypes.byref(work), ctypes.c_double(tol),
                                   max_cycles, ctypes.byref(net) if net is not None else None, ctypes.byref(st))
    if s not in (0, 7):
        _check(s)
    d = st.as_dict()
    d["converged"] = s == 0
    return d


def manet_training_pair(pot, dens, work, cycles: int, delta, phi1, phi2, sigma) -> dict:
    st = MAStats()
    _check(load().manet_training_pair(ctypes.byref(pot), ctypes.byref(dens), ctypes.byref(work), cycles,
                                      _vp(delta), _vp(phi1), _vp(phi2), _vp(sigma), ctypes.byref(st)))
    return st.as_dict()


# ---- ensembles in one CUDA graph, FFT tile autotuner -----------------------------------------
class Ensemble:
    """ic_ensemble_create / run / result / destroy over a list of ICConfig"""

    def __init__(self, cfgs, spline: Spline, streams: int = 8, max_batch: int = 0):
        """max_batch: realisations per batched unit (1: none; 0: the library's default)"""
        self.n = len(cfgs)
        self.cfgs = (ICConfig * self.n)(*cfgs)
        self.spline = spline
        self.h = ctypes.c_void_p()
        _check(load().ic_ensemble_create_batched(ctypes.byref(self.h), self.cfgs, self.n, ctypes.byref(spline.sp),
                                                 streams, max_batch))

    def run(self) -> float:
        ms = ctypes.c_double(0)
        _check(load().ic_ensemble_run(self.h, ctypes.byref(ms)))
        return ms.value

    def launches(self) -> int:
        return load().ic_ensemble_launches(self.h)

    def units(self) -> int:
        return load().ic_ensemble_units(self.h)

    def result(self, i: int) -> dict:
        bins = self.cfgs[i].pk_bins
        k, p, o = np.zeros(bins), np.zeros(bins), np.zeros(bins, np.int64)
        r = ICResult(k.ctypes.data_as(_dp), p.ctypes.data_as(_dp), o.ctypes.data_as(_lp), None, 0, 0.0)
        _check(load().ic_ensemble_result(self.h, i, ctypes.byref(r)))
        return {"pk_k": k, "pk_p": p, "pk_obs": o}

    def close(self) -> None:
        if self.h:
            load().ic_ensemble_destroy(self.h)
            self.h = ctypes.c_void_p()


def autotune(cfg: ICConfig, spline: Spline) -> tuple:
    pxy, pz, ms = ctypes.c_int(0), ctypes.c_int(0), ctypes.c_double(0)
    _check(load().mitos_autotune(ctypes.byref(cfg), ctypes.byref(spline.sp), ctypes.byref(pxy), ctypes.byref(pz),
                                 ctypes.byref(ms)))
    return pxy.value, pz.value, ms.value


def set_tiles(N: int, precision: int, pxy: int, pz: int) -> None:
    _check(load().mitos_set_tiles(N, precision, pxy, pz))


def set_radix(N: int, precision: int, rad_n, rad_h) -> None:
    a = (ctypes.c_int * len(rad_n))(*rad_n)
    b = (ctypes.c_int * len(rad_h))(*rad_h)
    _check(load().mitos_set_radix(N, precision, a, len(rad_n), b, len(rad_h)))


def get_radix(N: int, precision: int) -> tuple:
    """(radices of the length-N transforms, radices of the length-N/2 transforms)"""
    a, b = (ctypes.c_int * 12)(), (ctypes.c_int * 12)()
    na, nb = ctypes.c_int(), ctypes.c_int()
    _check(load().mitos_get_radix(N, precision, a, ctypes.byref(na), b, ctypes.byref(nb)))
    return list(a[:na.value]), list(b[:nb.value])


def get_tiles(N: int, precision: int) -> tuple:
    pxy, pz = ctypes.c_int(0), ctypes.c_int(0)
    _check(load().mitos_get_tiles(N, precision, ctypes.byref(pxy), ctypes.byref(pz)))
    return pxy.value, pz.value


# ---- N-GenIC-like field --------------------------------------------------------------------
def generate_ngeniclike_grf_dg(grf: DistributedGrid, seed: int) -> None:
    _check(load().generate_ngeniclike_grf_dg(ctypes.byref(grf), ctypes.c_long(seed)))


def ranlxd1_uniforms(seed: int, n: int) -> np.ndarray:
    out = np.zeros(n)
    _check(load().mitos_ranlxd1_uniforms(ctypes.c_ulong(seed), ctypes.c_long(n), out.ctypes.data_as(_dp)))
    return out


# ---- asynchronous IC submission --------------------------------------------------------------
def ic_pipeline_submit(cfg: ICConfig, spline: Spline, res: ICResult) -> None:
    """enqueue one IC; res (and its arrays) must stay alive until ic_pipeline_wait returns"""
    _check(load().ic_pipeline_submit(ctypes.byref(cfg), ctypes.byref(spline.sp), ctypes.byref(res)))


def ic_pipeline_wait() -> None:
    _check(load().ic_pipeline_wait())


def set_cluster_fft(mode: int) -> int:
    """the one-pass cluster Z + Y step of the FP32 r2c (256^3, 512^3): 0 off, 1-3 a cluster shape;
    returns the previous mode"""
    return int(load().mitos_set_cluster_fft(int(mode)))


def set_lattice_tma(on: bool) -> bool:
    """tensor-copy staging of the lattice deposit's tiles on or off; the previous setting"""
    return bool(load().mitos_set_lattice_tma(1 if on else 0))


def set_lattice_order(regions: bool) -> bool:
    """the lattice deposit's brick order: 8 x 8 x 4 regions (True) or rows; the previous setting"""
    return bool(load().mitos_set_lattice_order(1 if regions else 0))


def set_stream(stream_handle: int = 0, asynchronous: bool = False) -> None:
    """launch this thread's library work on a caller's CUDA stream (its handle, e.g.
    torch.cuda.Stream().cuda_stream; 0: the library's stream); asynchronous: return without
    synchronising (device-only entry points)"""
    _check(load().mitos_set_stream(ctypes.c_void_p(stream_handle or None), 1 if asynchronous else 0))
