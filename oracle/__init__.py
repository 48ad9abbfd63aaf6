"""ctypes bindings of the CPU oracle (liborc.so) and of the reference build (_ref/).

TEST INFRASTRUCTURE ONLY: imported by tests/, __graft_entry__.smoke() and bench.py's CPU
baseline / reference arm.  The GPU library never imports this package.
"""
from __future__ import annotations

import ctypes
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "liborc.so")
REF_PATH = os.path.join(HERE, "_ref", "libmitos_ref.so")
# the reference checkout beside this repository, unless MITOS_REF_DIR names another
REF_DIR = os.environ.get("MITOS_REF_DIR") or os.path.normpath(os.path.join(HERE, "..", "..", "reference"))

_dp = ctypes.POINTER(ctypes.c_double)
_fp = ctypes.POINTER(ctypes.c_float)
_lp = ctypes.POINTER(ctypes.c_long)
_up = ctypes.POINTER(ctypes.c_uint64)

_lib = None
_ref = None


def build(ref: bool = True) -> None:
    """Compile liborc.so (always) and _ref/libmitos_ref.so (when the reference tree exists)."""
    subprocess.run(["make", "-s", "-C", HERE, "liborc.so"], check=True)
    if ref and os.path.isdir(os.path.join(REF_DIR, "src")):
        subprocess.run(["make", "-s", "-C", HERE, "ref", f"REF_DIR={REF_DIR}"], check=True)


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            build(ref=False)
        _lib = ctypes.CDLL(LIB_PATH)
        _lib.orc_rng_next.restype = ctypes.c_uint64
        _lib.orc_sample_norm.restype = ctypes.c_double
        _lib.orc_tsc_gather.restype = ctypes.c_double
        _lib.orc_cic_deposit.restype = ctypes.c_double
        _lib.orc_log_tau_at_redshift.restype = ctypes.c_double
        _lib.orc_growth_at_log_tau.restype = ctypes.c_double
        _lib.orc_primordial_power.restype = ctypes.c_double
    return _lib


def ref_lib():
    """The reference build, or None when it was not built (no reference tree here)."""
    global _ref
    if _ref is None and os.path.exists(REF_PATH):
        _ref = ctypes.CDLL(REF_PATH)
    return _ref


def P(a, t=_dp):
    return None if a is None else a.ctypes.data_as(t)


# ---- structs mirrored from mitos_oracle.h ----------------------------------------------
class OrcPerturb(ctypes.Structure):
    _fields_ = [("k_size", ctypes.c_int), ("tau_size", ctypes.c_int), ("n_functions", ctypes.c_int),
                ("k", _dp), ("log_tau", _dp), ("redshift", _dp), ("D_growth", _dp),
                ("f_growth", _dp), ("H_Hubble", _dp), ("delta", _dp),
                ("k_acc_size", ctypes.c_int), ("k_acc", _dp)]


class OrcCosmo(ctypes.Structure):
    _fields_ = [("A_s", ctypes.c_double), ("n_s", ctypes.c_double), ("k_pivot", ctypes.c_double)]


class OrcICParams(ctypes.Structure):
    _fields_ = [("N", ctypes.c_int), ("M", ctypes.c_int), ("boxlen", ctypes.c_double),
                ("seed", ctypes.c_uint64), ("cosmo", OrcCosmo),
                ("sp", ctypes.POINTER(OrcPerturb)), ("index_src", ctypes.c_int),
                ("z_ini", ctypes.c_double), ("lpt_order", ctypes.c_int),
                ("ma_cycles", ctypes.c_int), ("pk_bins", ctypes.c_int),
                ("pk_linear", ctypes.c_int), ("mass", ctypes.c_double), ("index_vel", ctypes.c_int),
                ("thermal", ctypes.c_int), ("thermal_T_eV", ctypes.c_double),
                ("thermal_M_eV", ctypes.c_double), ("speed_of_light", ctypes.c_double),
                ("thermal_draw_offset", ctypes.c_uint64)]


class OrcICOut(ctypes.Structure):
    _fields_ = [("grf", _dp), ("delta_k", _dp), ("phi_k", _dp), ("disp", _dp * 3), ("pos", _fp),
                ("rho", _dp), ("pk_k", _dp), ("pk_p", _dp), ("pk_obs", _lp), ("ma_eps", _dp),
                ("vel", _fp)]


class Spline:
    """Keeps the table arrays alive for an OrcPerturb."""

    def __init__(self, table):
        self.arrays = [np.ascontiguousarray(a, dtype=np.float64) for a in
                       (table.k, table.log_tau, table.redshift, table.D_growth, table.f_growth,
                        table.H_Hubble, table.delta)]
        k, lt, z, D, f, H, d = self.arrays
        self.s = OrcPerturb(table.k_size, table.tau_size, table.n_functions, P(k), P(lt), P(z),
                            P(D), P(f), P(H), P(d), 0, None)
        lib().orc_spline_init(ctypes.byref(self.s), 1000)

    def __del__(self):
        try:
            lib().orc_spline_free(ctypes.byref(self.s))
        except Exception:
            pass


# ---- helpers ---------------------------------------------------------------------------
def draws(seed: int, n: int) -> np.ndarray:
    out = np.empty(n, np.uint64)
    lib().orc_draws(ctypes.c_uint64(seed), ctypes.c_int64(n), P(out, _up))
    return out


def norms(seed: int, n: int) -> np.ndarray:
    out = np.empty(n, np.float64)
    lib().orc_norms(ctypes.c_uint64(seed), ctypes.c_int64(n), P(out))
    return out


def to_complex(buf: np.ndarray) -> np.ndarray:
    return buf[..., 0] + 1j * buf[..., 1]


def grf(N: int, boxlen: float, seed: int, hermitian: bool = True) -> np.ndarray:
    buf = np.zeros((N, N, N // 2 + 1, 2))
    lib().orc_generate_grf(N, ctypes.c_double(boxlen), ctypes.c_uint64(seed), P(buf))
    if hermitian:
        lib().orc_enforce_hermiticity(N, P(buf))
    return to_complex(buf)


def fft_r2c(N: int, boxlen: float, real_padded: np.ndarray) -> np.ndarray:
    src = np.ascontiguousarray(real_padded, np.float64).reshape(N, N, -1)
    out = np.zeros((N, N, N // 2 + 1, 2))
    lib().orc_fft_r2c(N, ctypes.c_double(boxlen), P(src), ctypes.c_long(src.shape[2]), P(out))
    return to_complex(out)


def fft_c2r(N: int, boxlen: float, fbox: np.ndarray, pitch: int | None = None) -> np.ndarray:
    buf = np.ascontiguousarray(np.stack([fbox.real, fbox.imag], -1))
    pitch = N + 2 if pitch is None else pitch
    out = np.zeros((N, N, pitch))
    lib().orc_fft_c2r(N, ctypes.c_double(boxlen), P(buf), P(out), ctypes.c_long(pitch))
    return out


KERNELS = {"constant": 0, "lowpass": 1, "hipass": 2, "tophat": 3, "elliptic_tophat": 4,
           "translate": 5, "gaussian": 6, "gaussian_inv": 7, "inv_poisson": 8, "dx": 9, "dy": 10,
           "dz": 11, "power_no_transfer": 12, "transfer": 13, "inv_transfer": 14,
           "undo_hermite": 15}


class TransferParams(ctypes.Structure):
    _fields_ = [("sp", ctypes.POINTER(OrcPerturb)), ("index_src", ctypes.c_int),
                ("tau_index", ctypes.c_int), ("u_tau", ctypes.c_double)]


class HermiteParams(ctypes.Structure):
    _fields_ = [("order", ctypes.c_int), ("N", ctypes.c_int), ("boxlen", ctypes.c_double)]


def apply_kernel(N: int, boxlen: float, fbox: np.ndarray, name: str, params=None) -> np.ndarray:
    src = np.ascontiguousarray(np.stack([fbox.real, fbox.imag], -1))
    out = np.zeros_like(src)
    if params is None:
        pp = None
    elif isinstance(params, ctypes.Structure):
        pp = ctypes.cast(ctypes.byref(params), ctypes.c_void_p)
    else:
        arr = np.ascontiguousarray(np.atleast_1d(params), np.float64)
        pp = ctypes.cast(P(arr), ctypes.c_void_p)
    err = lib().orc_apply_kernel(N, ctypes.c_double(boxlen), P(out), P(src), KERNELS[name], pp)
    assert err == 0
    return to_complex(out)


def transfer_params(spline: Spline, z: float, index_src: int = 0) -> TransferParams:
    l = lib()
    lt = l.orc_log_tau_at_redshift(ctypes.byref(spline.s), ctypes.c_double(z))
    ti = ctypes.c_int()
    ut = ctypes.c_double()
    l.orc_spline_find_tau(ctypes.byref(spline.s), ctypes.c_double(lt), ctypes.byref(ti),
                          ctypes.byref(ut))
    return TransferParams(ctypes.pointer(spline.s), index_src, ti.value, ut.value)


def powerspec(N: int, boxlen: float, f1: np.ndarray, f2: np.ndarray, bins: int, linear: bool):
    a = np.ascontiguousarray(np.stack([f1.real, f1.imag], -1))
    b = np.ascontiguousarray(np.stack([f2.real, f2.imag], -1))
    k = np.zeros(bins)
    p = np.zeros(bins)
    o = np.zeros(bins, np.int64)
    fn = lib().orc_powerspec_lin if linear else lib().orc_powerspec_log
    with np.errstate(all="ignore"):
        fn(N, ctypes.c_double(boxlen), P(a), P(b), bins, P(k), P(p), P(o, _lp))
    return k, p, o


def _float_slab_args(box1, box2):
    a = np.ascontiguousarray(np.stack([box1.real, box1.imag], -1).astype(np.float32))
    b = np.ascontiguousarray(np.stack([box2.real, box2.imag], -1).astype(np.float32))
    return a, b


def powerspec_float_slab(N: int, X0: int, NX: int, boxlen: float, box1: np.ndarray, box2: np.ndarray, bins: int):
    """calc_cross_powerspec_float_mpi on one rank; box1/box2: complex64 slabs (NX, N, N/2+1)"""
    a, b = _float_slab_args(box1, box2)
    k, p, o = np.zeros(bins), np.zeros(bins), np.zeros(bins, np.int64)
    with np.errstate(all="ignore"):
        lib().orc_powerspec_float_slab(ctypes.c_long(N), ctypes.c_long(X0), ctypes.c_long(NX), ctypes.c_double(boxlen),
                                       P(a, _fp), P(b, _fp), bins, P(k), P(p), P(o, _lp))
    return k, p, o


def ref_powerspec_float_slab(N: int, X0: int, NX: int, boxlen: float, box1: np.ndarray, box2: np.ndarray, bins: int):
    """the reference build's calc_cross_powerspec_float_mpi (one rank), or None without it"""
    r = ref_lib()
    if r is None:
        return None
    a, b = _float_slab_args(box1, box2)
    k, p, o = np.zeros(bins), np.zeros(bins), np.zeros(bins, np.int64)
    with np.errstate(all="ignore"):
        r.calc_cross_powerspec_float_mpi(ctypes.c_long(N), ctypes.c_long(X0), ctypes.c_long(NX), ctypes.c_double(boxlen),
                                         P(a, _fp), P(b, _fp), bins, P(k), P(p), P(o, _lp))
    return k, p, o


def ref_header_attributes(boxlen: float, z_ini: float, types, units):
    """the attributes the reference's writeHeaderAttributes (src/header.c:26-175) writes, recorded by
    the HDF5 stand-in: {(group, name): list of values}; None without the reference build"""
    r = ref_lib()
    if r is None:
        return None
    n = len(types)
    names = (ctypes.c_char_p * max(n, 1))(*[t[0].encode() for t in types])
    tot = (ctypes.c_longlong * max(n, 1))(*[int(t[1]) for t in types])
    u = (ctypes.c_double * 5)(*units)
    assert r.ref_header_attributes(ctypes.c_double(boxlen), ctypes.c_double(z_ini), n, names, tot, u) == 0
    out = {}
    g, nm = ctypes.create_string_buffer(32), ctypes.create_string_buffer(64)
    ty, cnt = ctypes.c_int(), ctypes.c_int()
    d, l = (ctypes.c_double * 8)(), (ctypes.c_longlong * 8)()
    for i in range(r.orc_h5_count()):
        r.orc_h5_get(i, g, nm, ctypes.byref(ty), ctypes.byref(cnt), d, l)
        vals = [d[j] for j in range(cnt.value)] if ty.value == 1 else [l[j] for j in range(cnt.value)]
        out[(g.value.decode(), nm.value.decode())] = vals
    return out


def ic_params(N, M, boxlen, seed, table, lpt_order=2, ma_cycles=0, pk_bins=32, pk_linear=True,
              z_ini=31.0, mass=1.0, index_src=0, index_vel=-1, thermal=0, thermal_T_eV=0.0,
              thermal_M_eV=0.0, speed_of_light=0.0, thermal_draw_offset=0):
    return dict(N=N, M=M, boxlen=boxlen, seed=seed, table=table, lpt_order=lpt_order,
                ma_cycles=ma_cycles, pk_bins=pk_bins, pk_linear=pk_linear, z_ini=z_ini, mass=mass,
                index_src=index_src, index_vel=index_vel, thermal=thermal, thermal_T_eV=thermal_T_eV,
                thermal_M_eV=thermal_M_eV, speed_of_light=speed_of_light,
                thermal_draw_offset=thermal_draw_offset)


def _thermal_args(prm):
    return (int(prm.get("thermal", 0)), ctypes.c_double(prm.get("thermal_T_eV", 0.0)),
            ctypes.c_double(prm.get("thermal_M_eV", 0.0)), ctypes.c_double(prm.get("speed_of_light", 0.0)),
            ctypes.c_uint64(prm.get("thermal_draw_offset", 0)))


def _alloc_outputs(N, M, bins, want, ma_cycles):
    H = N // 2 + 1
    o = {"pk_k": np.zeros(bins), "pk_p": np.zeros(bins), "pk_obs": np.zeros(bins, np.int64)}
    if "grf" in want: o["grf"] = np.zeros((N, N, H, 2))
    if "delta_k" in want: o["delta_k"] = np.zeros((N, N, H, 2))
    if "phi_k" in want: o["phi_k"] = np.zeros((N, N, H, 2))
    if "disp" in want:
        for i in range(3): o[f"disp{i}"] = np.zeros((N, N, N + 2))
    if "pos" in want: o["pos"] = np.zeros((M * M * M, 3), np.float32)
    if "vel" in want: o["vel"] = np.zeros((M * M * M, 3), np.float32)
    if "rho" in want: o["rho"] = np.zeros((N, N, N))
    if ma_cycles: o["ma_eps"] = np.zeros(ma_cycles)
    return o


def _finish(o):
    for key in ("grf", "delta_k", "phi_k"):
        if key in o: o[key] = to_complex(o[key])
    return o


def ic_pipeline(prm: dict, want=("pk",)) -> dict:
    """Run the oracle pipeline; returns the requested intermediates and the P(k) bins."""
    N, M, bins = prm["N"], prm["M"], prm["pk_bins"]
    sp = Spline(prm["table"])
    t = prm["table"]
    o = _alloc_outputs(N, M, bins, want, prm["ma_cycles"])
    p = OrcICParams(N, M, prm["boxlen"], prm["seed"], OrcCosmo(t.A_s, t.n_s, t.k_pivot),
                    ctypes.pointer(sp.s), prm["index_src"], prm["z_ini"], prm["lpt_order"],
                    prm["ma_cycles"], bins, int(prm["pk_linear"]), prm["mass"], prm.get("index_vel", -1),
                    *_thermal_args(prm))
    out = OrcICOut()
    out.grf, out.delta_k, out.phi_k = P(o.get("grf")), P(o.get("delta_k")), P(o.get("phi_k"))
    for i in range(3):
        out.disp[i] = P(o.get(f"disp{i}"))
    out.pos = P(o.get("pos"), _fp)
    out.rho = P(o.get("rho"))
    out.pk_k, out.pk_p, out.pk_obs = P(o["pk_k"]), P(o["pk_p"]), P(o["pk_obs"], _lp)
    out.ma_eps = P(o.get("ma_eps"))
    out.vel = P(o.get("vel"), _fp)
    with np.errstate(all="ignore"):
        err = lib().orc_ic_pipeline(ctypes.byref(p), ctypes.byref(out))
    assert err == 0, err
    return _finish(o)


def ref_ic_pipeline(prm: dict, want=("pk",)) -> dict:
    """Run the same pipeline through the reference's own functions (needs the _ref build)."""
    r = ref_lib()
    if r is None:
        raise RuntimeError("reference build missing (oracle/_ref/libmitos_ref.so)")
    N, M, bins, t = prm["N"], prm["M"], prm["pk_bins"], prm["table"]
    o = _alloc_outputs(N, M, bins, want, 0)
    arrs = [np.ascontiguousarray(a, np.float64) for a in
            (t.k, t.log_tau, t.redshift, t.D_growth, t.f_growth, t.H_Hubble, t.delta)]
    r.ref_ic_pipeline.restype = ctypes.c_int
    err = r.ref_ic_pipeline(
        N, M, ctypes.c_double(prm["boxlen"]), ctypes.c_uint64(prm["seed"]), ctypes.c_double(t.A_s),
        ctypes.c_double(t.n_s), ctypes.c_double(t.k_pivot), t.k_size, t.tau_size, t.n_functions,
        *[P(a) for a in arrs], prm["index_src"], ctypes.c_double(prm["z_ini"]), prm["lpt_order"],
        prm["ma_cycles"], bins, int(prm["pk_linear"]), ctypes.c_double(prm["mass"]),
        P(o.get("grf")), P(o.get("delta_k")), P(o.get("phi_k")), P(o.get("disp0")),
        P(o.get("disp1")), P(o.get("disp2")), P(o.get("pos"), _fp), P(o.get("rho")),
        P(o["pk_k"]), P(o["pk_p"]), P(o["pk_obs"], _lp), prm.get("index_vel", -1), P(o.get("vel"), _fp),
        *_thermal_args(prm))
    assert err == 0, err
    return _finish(o)


# ---- thermal-motion sampler (thermal_oracle.c) ----------------------------------------------
FERMION, BOSON = 1, 2


def _state(st):
    a = np.ascontiguousarray(np.asarray(st, dtype=np.uint64).reshape(4))
    return a


def _table_call(fn, kind, T_eV):
    rows = np.zeros((4096, 8))
    table = np.zeros(1000, np.int32)
    norm = ctypes.c_double(0)
    fn.restype = ctypes.c_int
    with np.errstate(all="ignore"):
        n = fn(int(kind), ctypes.c_double(T_eV), 4096, P(rows), table.ctypes.data_as(ctypes.POINTER(ctypes.c_int)),
               ctypes.byref(norm))
    assert 0 < n <= 4096, n
    return {"pieces": rows[:n].copy(), "table": table, "norm": norm.value}


def sampler_table(kind: int, T_eV: float) -> dict:
    """The sampler's pieces (rows l r Fl Fr a0 a1 a2 a3, sorted by Fl), start table and norm."""
    return _table_call(lib().orc_sampler_table, kind, T_eV)


def ref_sampler_table(kind: int, T_eV: float) -> dict:
    return _table_call(ref_lib().ref_sampler_table, kind, T_eV)


def _draws_call(fn, kind, T_eV, st0, n):
    out = np.zeros(n)
    st = _state(st0)
    assert fn(int(kind), ctypes.c_double(T_eV), P(st, _up), ctypes.c_long(n), P(out)) == 0
    return out


def sampler_draws(kind: int, T_eV: float, st0, n: int) -> np.ndarray:
    """n momenta (eV) drawn from start state st0 (four uint64)."""
    return _draws_call(lib().orc_sampler_draws, kind, T_eV, st0, n)


def ref_sampler_draws(kind: int, T_eV: float, st0, n: int) -> np.ndarray:
    return _draws_call(ref_lib().ref_sampler_draws, kind, T_eV, st0, n)


def thermal(kind, T_eV, M_eV, a_ini, c, st0, vel, stride=3) -> np.ndarray:
    """vel (float32, particles x stride, updated copy returned) plus the thermal motion of
    src/mitos.c:928-1062 from start state st0."""
    v = np.array(vel, dtype=np.float32, copy=True, order="C")
    n = v.shape[0]
    st = _state(st0)
    with np.errstate(all="ignore"):
        e = lib().orc_thermal(int(kind), ctypes.c_double(T_eV), ctypes.c_double(M_eV), ctypes.c_double(a_ini),
                              ctypes.c_double(c), P(st, _up), ctypes.c_long(n), P(v, _fp), ctypes.c_long(stride))
    assert e == 0, e
    return v


def ref_thermal(kind, T_eV, M_eV, a_ini, c, st0, vel) -> np.ndarray:
    v = np.array(vel, dtype=np.float32, copy=True, order="C")
    st = _state(st0)
    with np.errstate(all="ignore"):
        e = ref_lib().ref_thermal(int(kind), ctypes.c_double(T_eV), ctypes.c_double(M_eV), ctypes.c_double(a_ini),
                                  ctypes.c_double(c), P(st, _up), ctypes.c_long(v.shape[0]), P(v, _fp))
    assert e == 0, e
    return v


def rng_state(seed: int, advance: int = 0) -> np.ndarray:
    """xoshiro256** state of Seed after `advance` draws (sequential stepping)."""
    st = np.zeros(4, np.uint64)
    lib().orc_rng_init(ctypes.c_uint64(seed), P(st, _up))
    if advance:
        lib().orc_rng_advance(P(st, _up), ctypes.c_uint64(advance))
    return st


def _bispec_args(N, bins):
    return [np.zeros(bins) for _ in range(4)]


def bispectrum(N, boxlen, fbox, bins, bins3, volume_mode=False, btype=0, theta=0.0, k3=0.0) -> dict:
    """orc_bispectrum (src/calc_powerspec.c:295-508 restated); fbox complex (N, N, N/2+1)"""
    buf = None if fbox is None else np.ascontiguousarray(np.stack([fbox.real, fbox.imag], -1), np.float64)
    k1, k2, k3o, b = _bispec_args(N, bins)
    if buf is None:
        buf = np.zeros((N, N, N // 2 + 1, 2))
    lib().orc_bispectrum(N, ctypes.c_double(boxlen), P(buf), bins, bins3, P(k1), P(k2), P(k3o), P(b),
                         int(volume_mode), int(btype), ctypes.c_double(theta), ctypes.c_double(k3))
    return {"k1": k1, "k2": k2, "k3": k3o, "B": b}


def ref_bispectrum(N, boxlen, fbox, bins, bins3, volume_mode=False, btype=0, theta=0.0, k3=0.0) -> dict:
    """the reference's own calc_bispectrum (needs the _ref build)"""
    buf = np.zeros((N, N, N // 2 + 1, 2)) if fbox is None else \
        np.ascontiguousarray(np.stack([fbox.real, fbox.imag], -1), np.float64)
    k1, k2, k3o, b = _bispec_args(N, bins)
    ref_lib().calc_bispectrum(N, ctypes.c_double(boxlen), None if fbox is None else P(buf), bins, bins3,
                              P(k1), P(k2), P(k3o), P(b), int(volume_mode), int(btype), ctypes.c_double(theta),
                              ctypes.c_double(k3))
    return {"k1": k1, "k2": k2, "k3": k3o, "B": b}


def ref_grf(N: int, boxlen: float, seed: int, hermitian: bool = True) -> np.ndarray:
    buf = np.zeros((N, N, N // 2 + 1, 2))
    ref_lib().ref_grf(N, ctypes.c_double(boxlen), ctypes.c_uint64(seed), int(hermitian), P(buf))
    return to_complex(buf)


def ref_draws(seed: int, n: int) -> np.ndarray:
    out = np.empty(n, np.uint64)
    ref_lib().ref_draws(ctypes.c_uint64(seed), ctypes.c_int64(n), P(out, _up))
    return out


def ref_norms(seed: int, n: int) -> np.ndarray:
    out = np.empty(n, np.float64)
    ref_lib().ref_norms(ctypes.c_uint64(seed), ctypes.c_int64(n), P(out))
    return out


# ---- Monge-Ampere warm-start network (manet_oracle.c) ----------------------------------------
MANET_CIN = (3, 16, 16, 16)
MANET_COUT = (16, 16, 16, 1)


def bf16(x: np.ndarray) -> np.ndarray:
    """round to bfloat16 (through float32, ties to even), as float64"""
    f = lib().orc_bf16
    f.restype = ctypes.c_double
    f.argtypes = [ctypes.c_double]
    return np.vectorize(f)(np.asarray(x, np.float64))


def manet_loss_grad(x: np.ndarray, target: np.ndarray, layers, round_bf16: bool = True):
    """FP64 forward, MSE loss and gradients of the 4-layer network.
    x: [N, N, N, 3]; target: [N, N, N]; layers: [(w [27, cin, cout], b [cout])] with the real
    channel counts.  Returns (loss, pred [N, N, N], [(dw, db)])."""
    N = x.shape[0]
    xs = np.ascontiguousarray(x, np.float64)
    ts = np.ascontiguousarray(target, np.float64)
    ws = [np.ascontiguousarray(w, np.float64) for w, _ in layers]
    bs = [np.ascontiguousarray(b, np.float64) for _, b in layers]
    dws = [np.zeros_like(w) for w in ws]
    dbs = [np.zeros_like(b) for b in bs]
    pred = np.zeros((N, N, N))
    arr = lambda lst: (_dp * 4)(*[a.ctypes.data_as(_dp) for a in lst])
    f = lib().orc_manet_loss_grad
    f.restype = ctypes.c_double
    loss = f(N, xs.ctypes.data_as(_dp), ts.ctypes.data_as(_dp), arr(ws), arr(bs), int(round_bf16),
             pred.ctypes.data_as(_dp), arr(dws), arr(dbs))
    return loss, pred, list(zip(dws, dbs))


# ---- N-GenIC-like field (ngenic_oracle.c; parity with libgsl unpinned) -----------------------
class OrcRanlxd(ctypes.Structure):
    _fields_ = [("x", ctypes.c_uint64 * 12), ("carry", ctypes.c_int), ("i", ctypes.c_int), ("left", ctypes.c_int)]


def ranlxd1_uniforms(seed: int, n: int) -> np.ndarray:
    r = OrcRanlxd()
    L = lib()
    L.orc_ranlxd1_set(ctypes.byref(r), ctypes.c_ulong(seed))
    f = L.orc_ranlxd1_uniform
    f.restype = ctypes.c_double
    return np.array([f(ctypes.byref(r)) for _ in range(n)])


def ngenic_seedtable(N: int, seed: int) -> np.ndarray:
    t = np.zeros(N * N, np.uint32)
    lib().orc_ngenic_seedtable(N, ctypes.c_ulong(seed), t.ctypes.data_as(ctypes.POINTER(ctypes.c_uint32)))
    return t.reshape(N, N)


def ngeniclike_grf(N: int, boxlen: float, seed: int) -> np.ndarray:
    """complex [N, N, N/2+1] field of src/grf_ngeniclike.c on one rank"""
    buf = np.zeros(N * N * (N // 2 + 1) * 2)
    s = lib().orc_ngeniclike_grf(N, ctypes.c_double(boxlen), ctypes.c_ulong(seed), buf.ctypes.data_as(_dp))
    assert s == 0
    b = buf.reshape(N, N, N // 2 + 1, 2)
    return b[..., 0] + 1j * b[..., 1]
