"""Synthetic perturbation table in the layout of the reference's perturbation file.

The reference reads transfer functions T(k, tau) and background tables from an HDF5 file
(src/perturb_data.c:29-226, struct perturb_data in include/perturb_data.h:28-53).  No such file
ships with the reference, so this module builds an equivalent table:

* wavenumbers: ``k_size`` log-spaced values in [k_min, k_max] (h/Mpc; lengths are Mpc/h),
* times: ``tau_size`` scale factors log-spaced in [a_min, 1], flat LCDM background
  (Omega_m, Omega_Lambda = 1 - Omega_m, no radiation), conformal time in Mpc/h (c = 1),
* transfer function ``d_cdm``: the BBKS fit (Bardeen, Bond, Kaiser & Szalay 1986, eq. G3)
  with the Sugiyama (1995) shape parameter Gamma = Omega_m h exp(-Omega_b - sqrt(2h) Omega_b /
  Omega_m), scaled by the linear growth factor D(a) / D(1),
* A_s chosen so that sigma_8 (top hat, R = 8 Mpc/h) equals ``sigma8`` at z = 0 for the power
  spectrum the reference realises, P(k) = primordialPower(k) T(k)^2
  (src/primordial.c:25-33, include/fft_kernels.h:116-155).
* transfer function ``t_cdm`` (the velocity divergence, added at load time from the stored arrays):
  linear continuity, theta = -delta' = -f (a H / c) d_cdm in h/Mpc, with conformal time in Mpc/h.
  The reference builds the particle velocities from such a function (``TransferFunctionVelocity``,
  src/mitos.c:425-490).

The table is written once to ``data/perturb_bbks.npz`` and loaded from there, so every machine
uses the same bits.
"""
from __future__ import annotations

import os
from dataclasses import dataclass

import numpy as np

DATA_FILE = os.path.join(os.path.dirname(__file__), "data", "perturb_bbks.npz")
C_KMS = 299792.458


@dataclass
class PerturbTable:
    k: np.ndarray          # (k_size,)
    log_tau: np.ndarray    # (tau_size,)
    redshift: np.ndarray   # (tau_size,)
    D_growth: np.ndarray   # (tau_size,)
    f_growth: np.ndarray   # (tau_size,)
    H_Hubble: np.ndarray   # (tau_size,)
    delta: np.ndarray      # (n_functions, tau_size, k_size)
    titles: list
    A_s: float
    n_s: float
    k_pivot: float
    sigma8: float
    Omega_m: float
    Omega_b: float
    h: float

    @property
    def k_size(self) -> int:
        return int(self.k.shape[0])

    @property
    def tau_size(self) -> int:
        return int(self.log_tau.shape[0])

    @property
    def n_functions(self) -> int:
        return int(self.delta.shape[0])

    def index_of(self, title: str) -> int:
        return self.titles.index(title)


def bbks(k, Omega_m, Omega_b, h):
    gamma = Omega_m * h * np.exp(-Omega_b - np.sqrt(2.0 * h) * Omega_b / Omega_m)
    q = k / gamma
    return (np.log1p(2.34 * q) / (2.34 * q)
            * (1.0 + 3.89 * q + (16.1 * q) ** 2 + (5.46 * q) ** 3 + (6.71 * q) ** 4) ** -0.25)


def _background(a, Omega_m):
    from scipy.integrate import quad
    OL = 1.0 - Omega_m
    E = lambda x: np.sqrt(Omega_m / x**3 + OL)
    H0 = 100.0  # km/s/(Mpc/h)
    tau = np.array([quad(lambda x: C_KMS / (x * x * H0 * E(x)), 0.0, ai, limit=200)[0] for ai in a])
    I = np.array([quad(lambda x: 1.0 / (x * E(x)) ** 3, 0.0, ai, limit=200)[0] for ai in a])
    Ea = E(a)
    D = 2.5 * Omega_m * Ea * I
    dlnE = -1.5 * Omega_m / a**3 / Ea**2
    f = dlnE + 1.0 / (a**2 * Ea**3 * I)
    return tau, D, f, H0 * Ea


def build_table(Omega_m=0.31, Omega_b=0.049, h=0.67, n_s=0.965, sigma8=0.81, k_pivot=0.05,
                k_size=500, k_min=1e-5, k_max=10.0, tau_size=32, a_min=1e-3) -> PerturbTable:
    from scipy.integrate import quad
    k = np.logspace(np.log10(k_min), np.log10(k_max), k_size)
    a = np.logspace(np.log10(a_min), 0.0, tau_size)
    tau, D, f, H = _background(a, Omega_m)
    T0 = bbks(k, Omega_m, Omega_b, h)
    delta = (T0[None, :] * (D / D[-1])[:, None])[None, :, :]

    R = 8.0

    def integrand(lnk):
        kk = np.exp(lnk)
        x = kk * R
        W = 3.0 * (np.sin(x) - x * np.cos(x)) / x**3
        T = bbks(kk, Omega_m, Omega_b, h)
        return kk**4 * (kk / k_pivot) ** (n_s - 1.0) * T * T * W * W

    I = quad(integrand, np.log(1e-6), np.log(1e3), limit=500)[0]
    A_s = sigma8**2 / I
    return PerturbTable(k=k, log_tau=np.log(tau), redshift=1.0 / a - 1.0, D_growth=D, f_growth=f,
                        H_Hubble=H, delta=np.ascontiguousarray(delta), titles=["d_cdm"], A_s=A_s,
                        n_s=n_s, k_pivot=k_pivot, sigma8=sigma8, Omega_m=Omega_m, Omega_b=Omega_b,
                        h=h)


def save_table(t: PerturbTable, path: str = DATA_FILE) -> None:
    os.makedirs(os.path.dirname(path), exist_ok=True)
    np.savez(path, k=t.k, log_tau=t.log_tau, redshift=t.redshift, D_growth=t.D_growth,
             f_growth=t.f_growth, H_Hubble=t.H_Hubble, delta=t.delta,
             titles=np.array(t.titles), scalars=np.array([t.A_s, t.n_s, t.k_pivot, t.sigma8,
                                                          t.Omega_m, t.Omega_b, t.h]))


def velocity_transfer(t: PerturbTable) -> np.ndarray:
    """t_cdm(tau, k) = -f(tau) a(tau) H(tau) / c * d_cdm(tau, k) (h/Mpc)"""
    a = 1.0 / (1.0 + t.redshift)
    rate = -(t.f_growth * a * t.H_Hubble / C_KMS)
    return rate[:, None] * t.delta[t.index_of("d_cdm")]


def load_table(path: str = DATA_FILE) -> PerturbTable:
    z = np.load(path)
    A_s, n_s, k_pivot, sigma8, Om, Ob, h = [float(v) for v in z["scalars"]]
    t = PerturbTable(k=z["k"], log_tau=z["log_tau"], redshift=z["redshift"],
                     D_growth=z["D_growth"], f_growth=z["f_growth"], H_Hubble=z["H_Hubble"],
                     delta=np.ascontiguousarray(z["delta"]), titles=[str(s) for s in z["titles"]],
                     A_s=A_s, n_s=n_s, k_pivot=k_pivot, sigma8=sigma8, Omega_m=Om, Omega_b=Ob,
                     h=h)
    if "t_cdm" not in t.titles:
        t.delta = np.ascontiguousarray(np.concatenate([t.delta, velocity_transfer(t)[None]], axis=0))
        t.titles = t.titles + ["t_cdm"]
    return t


if __name__ == "__main__":
    tab = build_table()
    save_table(tab)
    print("wrote", DATA_FILE, "A_s =", tab.A_s)
