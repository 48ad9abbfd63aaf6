"""Write crmath_tables.h: the constants of the correctly rounded FP64 log and cos (crmath.cuh).

Run once with mpmath available (it is not needed at build time; the header is committed):
    python mitos_gb300/csrc/gen_crmath_tables.py
Every constant is a mathematical value (log, sin, cos, pi/2, ln 2, 1/n, 1/n!) evaluated with 400
bits and split into doubles; nothing is taken from another library.
"""
import os

import mpmath as mp

mp.mp.prec = 400
HERE = os.path.dirname(os.path.abspath(__file__))
OUT = os.path.join(HERE, "crmath_tables.h")


def rn(v, bits=53):
    """v rounded to nearest with `bits` significant bits, as an exact Python float"""
    with mp.workprec(bits):
        r = +mp.mpf(v)
    f = float(r)
    assert mp.mpf(f) == r
    return f


def split(v, widths=(53, 53, 53)):
    """v = c0 + c1 + c2 (+ a remainder below the last part), each c_i of widths[i] bits"""
    out, rest = [], mp.mpf(v)
    for w in widths:
        c = rn(rest, w)
        out.append(c)
        rest -= mp.mpf(c)
    return out


def hx(x):
    return "0.0" if x == 0 else float(x).hex()


lines = ["// crmath_tables.h -- generated by gen_crmath_tables.py (mpmath, 400 bits); do not edit.",
         "// Triple-double constants of the correctly rounded log and cos of crmath.cuh.", "#pragma once", ""]


def emit(name, vals, per=3):
    body = ",\n    ".join(", ".join(hx(v) for v in vals[i:i + per]) for i in range(0, len(vals), per))
    lines.append(f"#define {name} {{ \\\n    " + body.replace("\n", " \\\n") + " }")
    lines.append("")


# ---- log: x = 2^K m r_i^-1 (1 + z); log x = K ln 2 + L_i + log1p(z) ----------------------
# index i: the top 7 fraction bits of m in [1, 2).  r_i ~ 1 / (1 + (i + 1/2)/128) with 8 significant
# bits (so z = m r_i - 1 is exact with one FMA); r_0 = 1.  For i >= 53 (m >= 1.4140625) the
# exponent is raised by one and L_i = -log(2 r_i), so that x just below 1 (m near 2, K = 0) gives
# L = 0 and log x = log1p(z) with no cancellation.
LOG_SPLIT = 53
rtab, ltab = [], []
zmax = mp.mpf(0)
for i in range(128):
    if i == 0:
        r = 1.0
    else:
        c = 1 + (mp.mpf(i) + 0.5) / 128
        r = float(mp.nint(256 / c)) / 256
    rtab.append(r)
    lv = -mp.log(mp.mpf(r)) if i < LOG_SPLIT else -mp.log(2 * mp.mpf(r))
    ltab += split(lv)
    lo, hi = 1 + mp.mpf(i) / 128, 1 + mp.mpf(i + 1) / 128
    zmax = max(zmax, abs(lo * r - 1), abs(hi * r - 1))
    # exactness of z = fma(m, r, -1): m r is a multiple of 2^-60 below 2, |m r - 1| < 2^-7
    assert float(mp.nint(r * 256)) == r * 256
# the bound is reached only at an interval's open upper end (i = 0: m -> 1 + 1/128), so |z| < 2^-7
assert zmax <= mp.mpf(2) ** -7, zmax
lines.append(f"// sup |z| over the table: {float(zmax):.6g} (2^{float(mp.log(zmax, 2)):.3f}), not attained")
lines.append(f"#define CR_LOG_SPLIT {LOG_SPLIT}")
emit("CR_LOG_R_INIT", rtab, per=4)
emit("CR_LOG_L_INIT", ltab)
# ln 2 with two 42-bit leading parts, so K ln2_0 and K ln2_1 are exact for |K| < 2^11
for n, v in enumerate(split(mp.log(2), (42, 42, 53))):
    lines.append(f"#define CR_LN2_{n} {hx(v)}")
lines.append("")
# 1/n, n = 1 .. 24, as triple-doubles (log1p series)
inv = []
for n in range(1, 25):
    inv += split(mp.mpf(1) / n)
emit("CR_INV_N_INIT", inv)

# ---- cos: y = k pi/2 + t, t = +-(j/128 + b) ---------------------------------------------
# pi/2 in parts of 50, 50, 50 and 53 bits: k P1, k P2, k P3 are exact for k < 8
for n, v in enumerate(split(mp.pi / 2, (50, 50, 50, 53))):
    lines.append(f"#define CR_PIO2_{n} {hx(v)}")
lines.append(f"#define CR_2_OVER_PI {hx(rn(2 / mp.pi))}")
lines.append("")
NJ = 106  # j <= 105: |t| up to 0.82 > pi/4 + the rounding of k
sc = []
for j in range(NJ):
    a = mp.mpf(j) / 128
    sc += split(mp.sin(a)) + split(mp.cos(a))
lines.append(f"#define CR_COS_NJ {NJ}")
emit("CR_SINCOS_INIT", sc, per=6)
# 1/n!, n = 0 .. 16 (sin and cos series)
fac = []
for n in range(17):
    fac += split(1 / mp.factorial(n))
emit("CR_INV_FACT_INIT", fac)

with open(OUT, "w") as f:
    f.write("\n".join(lines) + "\n")
print("wrote", OUT, "zmax 2^%.3f" % float(mp.log(zmax, 2)))
