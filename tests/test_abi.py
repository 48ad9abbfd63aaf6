"""CPU tests of the C ABI library: it loads, exports every function include/*.h declares, and its
host-side jump-ahead reproduces the sequential xoshiro256** stream.  No GPU work is issued."""
import ctypes
import glob
import os
import re

import numpy as np

import oracle
import mitos_gb300.lib as ml

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_functions():
    names = set()
    for h in glob.glob(os.path.join(ROOT, "include", "*.h")):
        src = open(h).read()
        src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
        # function declarations (typedefs of function pointers are types, not exports)
        for m in re.finditer(r"^\s*(?!typedef\b)(?:const\s+)?[A-Za-z_][\w\s\*]*?\b([A-Za-z_]\w*)\s*\(", src, re.M):
            name = m.group(1)
            if name not in ("if", "while", "for", "return", "sizeof", "defined"):
                names.add(name)
    return names


def test_library_exports_every_declared_function():
    lib = ml.load()
    names = declared_functions()
    assert len(names) >= 40
    missing = [n for n in sorted(names) if not hasattr(lib, n)]
    assert not missing, missing
    assert set(ml.EXPORTS) <= names


def _next(s):
    M = (1 << 64) - 1
    rot = lambda x, k: ((x << k) | (x >> (64 - k))) & M
    r = rot((s[1] * 5) & M, 7) * 9 & M
    t = (s[1] << 17) & M
    s[2] ^= s[0]; s[3] ^= s[1]; s[1] ^= s[2]; s[0] ^= s[3]; s[2] ^= t; s[3] = rot(s[3], 45)
    return r


def test_jump_ahead_matches_sequential_stream():
    lib = ml.load()
    for seed in (42, 7, 1000):
        s0 = list(ml.rng_init(seed).s)
        d = oracle.draws(seed, 20001)
        for n in (0, 1, 17, 1028, 20000):
            arr = (ctypes.c_uint64 * 4)(*s0)
            lib.mitos_rng_jump(arr, ctypes.c_ulonglong(n))
            assert _next(list(arr)) == int(d[n])


def test_noise_column_start_offsets():
    """column c = x N + y starts at draw 0 (c = 0) or 4 (c (N/2+1) - 1), src/grf.c:47-63."""
    lib = ml.load()
    s0 = list(ml.rng_init(42).s)
    for N in (16, 96):
        T = 4 * (N // 2 + 1)
        cols = [0, 1, 2, N + 3, N * N - 1]
        d = oracle.draws(42, T * N * N)
        for c in cols:
            out = (ctypes.c_uint64 * 4)()
            lib.mitos_noise_column_state(N, ctypes.c_long(c), (ctypes.c_uint64 * 4)(*s0), out)
            off = 0 if c == 0 else T * c - 4
            assert _next(list(out)) == int(d[off])


def test_host_kernel_callbacks_follow_reference():
    lib = ml.load()
    k = ml.Kernel(0.1, -0.2, 0.3, np.sqrt(0.14), (0.0, 0.0), None)
    lib.kernel_inv_poisson(ctypes.byref(k))
    assert k.kern[0] == -1.0 / k.k / k.k and k.kern[1] == 0
    lib.kernel_dy(ctypes.byref(k))
    assert k.kern[0] == 0 and k.kern[1] == -0.2


def _check_layouts(tmp_path, include_dir, header, structs):
    """compile a program printing sizeof / offsetof of each struct against `header` and compare them
    with the ctypes mirrors"""
    import shutil
    import subprocess
    import pytest
    cc = shutil.which("gcc") or shutil.which("cc")
    if cc is None:
        pytest.skip("no C compiler")
    lines = ["#include <stdio.h>", "#include <stddef.h>", f'#include "{header}"', "int main(void) {"]
    for cname, py in structs.items():
        lines.append(f'printf("{cname} size %zu\\n", sizeof(struct {cname}));')
        for fname, _ in py._fields_:
            lines.append(f'printf("{cname} {fname} %zu\\n", offsetof(struct {cname}, {fname}));')
    lines += ["return 0;", "}"]
    src = tmp_path / "layout.c"
    src.write_text("\n".join(lines) + "\n")
    exe = tmp_path / "layout"
    subprocess.run([cc, "-std=c11", "-I", include_dir, str(src), "-o", str(exe)], check=True)
    got = {}
    for line in subprocess.run([str(exe)], check=True, capture_output=True, text=True).stdout.splitlines():
        c, f, v = line.split()
        got[(c, f)] = int(v)
    for cname, py in structs.items():
        assert got[(cname, "size")] == ctypes.sizeof(py), cname
        for fname, _ in py._fields_:
            assert got[(cname, fname)] == getattr(py, fname).offset, (cname, fname)


def test_struct_layouts_match_ctypes(tmp_path):
    """every struct the Python binding mirrors has the header's field offsets and size"""
    _check_layouts(tmp_path, os.path.join(ROOT, "include"), "mitos_gb300.h",
                   {"distributed_grid": ml.DistributedGrid, "ic_config": ml.ICConfig, "ic_result": ml.ICResult,
                    "interval": ml.Interval, "sampler": ml.Sampler, "xoshiro256ss_state": ml.RngState})


def test_oracle_struct_layouts_match_ctypes(tmp_path):
    """the oracle's parameter and output structs as the test binding mirrors them"""
    _check_layouts(tmp_path, os.path.join(ROOT, "oracle"), "mitos_oracle.h",
                   {"orc_ic_params": oracle.OrcICParams, "orc_ic_out": oracle.OrcICOut})
