"""Exactly rounded log, cos and sampleNorm in pure Python (decimal, 60-90 digits), to classify the
values where the host libm and the correctly rounded GPU noise differ.  No third-party modules, so
it runs on every machine the tests run on."""
import math
from decimal import Decimal, localcontext

import numpy as np

RMAX = 18446744073709551616.0
TWO_PI = 2 * 3.14159265358979323846  # the double 2 * M_PI of src/random.c:45


def exact_log(x: float) -> float:
    """the double nearest to log(x): a 60-digit correctly rounded decimal logarithm, rounded once more
    (60 digits lie far below the 2^-118 that the hardest double-precision inputs need)"""
    with localcontext() as c:
        c.prec = 60
        return float(Decimal(x).ln())


def exact_cos(y: float) -> float:
    """the double nearest to cos(y), |y| < 8: Taylor series in 90-digit decimal arithmetic"""
    with localcontext() as c:
        c.prec = 90
        x = Decimal(y)
        x2 = x * x
        term = Decimal(1)
        s = Decimal(1)
        n = 0
        eps = Decimal(10) ** -88
        while True:
            n += 2
            term = -term * x2 / (n * (n - 1))
            s += term
            if abs(term) < eps:
                break
        return float(s)


def uniforms(A: np.ndarray) -> np.ndarray:
    """sampleUniform (src/random.c:27-31): (A + 0.5) / 2^64 with A rounded to double first"""
    return (A.astype(np.float64) + 0.5) / RMAX


def sample_norm_parts(A: int, B: int):
    """(u, y): the arguments of log and cos in sampleNorm (src/random.c:44-45)"""
    u = (float(A) + 0.5) / RMAX
    v = (float(B) + 0.5) / RMAX
    return u, TWO_PI * v


def sample_norm_exact(A: int, B: int) -> float:
    """sqrt(-2 log u) cos(2 pi v) with exactly rounded log and cos (sqrt and the products are IEEE)"""
    u, y = sample_norm_parts(A, B)
    return math.sqrt(-2.0 * exact_log(u)) * exact_cos(y)


def sample_norm_libm(A: int, B: int) -> float:
    """the same with this machine's libm (the reference's arithmetic)"""
    u, y = sample_norm_parts(A, B)
    return math.sqrt(-2.0 * math.log(u)) * math.cos(y)


def libm_misrounds(A: int, B: int) -> bool:
    """whether the host libm misrounds the log or the cos of this draw pair"""
    u, y = sample_norm_parts(A, B)
    return math.log(u) != exact_log(u) or math.cos(y) != exact_cos(y)


def ulps(got: np.ndarray, ref: np.ndarray) -> np.ndarray:
    """|got - ref| in units of the last place of ref (same dtype)"""
    got = np.asarray(got)
    ref = np.asarray(ref, dtype=got.dtype)
    sp = np.spacing(np.abs(ref).astype(got.dtype))
    return np.abs(got.astype(np.float64) - ref.astype(np.float64)) / sp.astype(np.float64)
