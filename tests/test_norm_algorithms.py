"""The integer algorithms of csrc/tk_norm.cu, restated in Python and checked on
the CPU against what they stand in for: printf's "%g" and "%.1f" (the
decimal digits of a float, rounded half to even on its binary value, and the
double Perl reads back from that text), the speculative chunked two-cursor
merge of nbkc_merge_left_right_stats.pl against the plain sequential walk,
and drand48's jump-ahead against stepping it draw by draw.  The GPU parity
tests (tests/test_gpu_norm.py) check the CUDA code itself."""
import bisect
import math
import random
import struct

import numpy as np


# ---- g6: 6 significant digits of (double)f, exactly (tk_norm.cu g6/scaled_rne)

def _shr_rne(a, sh):
    q, r, h = a >> sh, a & ((1 << sh) - 1), 1 << (sh - 1)
    return q + 1 if r > h or (r == h and q & 1) else q


def _div_rne(a, d):
    q = a // d
    r = a - q * d
    return q + 1 if r > d - r or (r == d - r and q & 1) else q


def _scaled_rne(m, q, s):
    if s >= 0:
        a = m * 10 ** s
        return a << q if q >= 0 else _shr_rne(a, -q)
    t = -s
    return _div_rne(m << q, 10 ** t) if q >= 0 else _div_rne(m, (10 ** t) << (-q))


def g6(f):
    if f == 0:
        return 0, 0
    bits = struct.unpack("<I", struct.pack("<f", f))[0]
    be = (bits >> 23) & 0xFF
    m, q = (bits & 0x7FFFFF) | 0x800000, be - 150
    x = ((be - 127) * 1233) >> 12          # floor(log10 f) to within one
    for _ in range(4):
        d = _scaled_rne(m, q, 5 - x)
        if d >= 10 ** 6:
            x += 1
        elif d < 10 ** 5:
            x -= 1
        else:
            return d, x
    raise AssertionError("no exponent")


def g6_text(D, X):
    if D == 0:
        return "0"
    d = "%06d" % D
    nz = 6
    while nz > 1 and d[nz - 1] == "0":
        nz -= 1
    if X < -4 or X >= 6:
        return d[0] + ("." + d[1:nz] if nz > 1 else "") + "e" + ("-" if X < 0 else "+") + "%02d" % abs(X)
    if X >= 0:
        return d[:X + 1] + ("." + d[X + 1:nz] if nz > X + 1 else "")
    return "0." + "0" * (-X - 1) + d[:nz]


def g6_value(D, X):
    if D == 0:
        return 0.0
    e = X - 5
    return float(D) * 10.0 ** e if e >= 0 else float(D) / 10.0 ** (-e)


def fix1(y):
    if y == 0:
        return 0
    bits = struct.unpack("<Q", struct.pack("<d", y))[0]
    be, M = (bits >> 52) & 0x7FF, bits & ((1 << 52) - 1)
    Q = -1074 if be == 0 else be - 1075
    if be:
        M |= 1 << 52
    W, sh = 10 * M, -Q
    return 0 if sh >= 64 else _shr_rne(W, sh)


def test_g6_matches_printf_g():
    rng = np.random.default_rng(3)
    vals = np.float32(rng.uniform(0, 1, 20000) * 10.0 ** rng.integers(-17, 19, 20000))
    vals = list(vals) + [np.float32(v) for v in (1, 0.5, 1.25, 999999.5, 9999995, 1e-5, 123456789, 1e6, 99999.95)]
    vals += list(np.float32(rng.integers(1, 2000, 20000) / np.float32(rng.integers(1, 200, 20000))))
    for f in vals:
        f = float(f)
        if not (1e-17 <= f < 1.8e19):
            continue
        D, X = g6(f)
        want = "%g" % f
        assert g6_text(D, X) == want, (f, D, X)
        assert g6_value(D, X) == float(want)


def test_fix1_matches_printf_1f():
    rng = random.Random(5)
    for _ in range(20000):
        a = float("%g" % float(np.float32(rng.uniform(0, 1000))))
        b = float("%g" % float(np.float32(rng.uniform(0, 1000))))
        y = (a + b) / 2
        N = fix1(y)
        assert "%d.%d" % (N // 10, N % 10) == "%.1f" % y
    for y in (0.25, 0.35, 0.05, 0.15, 1.25, 2.5, 0.45, 1e-300):
        N = fix1(y)
        assert "%d.%d" % (N // 10, N % 10) == "%.1f" % y


# ---- the merge: speculative chunks (tk_norm.cu k_merge_run / k_merge_repair)

def _core(a):
    return a[:-2] if len(a) >= 3 and a[-2:-1] == b"/" and a[-1:].isdigit() else a


def _walk(L, R, i=0, j=0):
    out = []
    while i < len(L) and j < len(R):
        if _core(L[i]) == _core(R[j]):
            out.append((i, j))
            i += 1
            j += 1
        elif L[i] < R[j]:
            i += 1
        else:
            j += 1
    return out


def _speculative(L, R, C):
    nL, nR = len(L), len(R)
    if not nL or not nR:
        return []
    nch = (nL + C - 1) // C
    js = [0] + [bisect.bisect_left(R, L[k * C]) for k in range(1, nch)]
    res = []
    for k in range(nch):
        last = k + 1 == nch
        ti, tj = (nL, nR) if last else ((k + 1) * C, js[k + 1])
        i, j, rows, st = k * C, js[k], [], "end"
        while i < nL and j < nR:
            if not last:
                if i == ti and j == tj:
                    st = "reached"
                    break
                if i > ti or j > tj:
                    st = "fail"
                    break
            if _core(L[i]) == _core(R[j]):
                rows.append((i, j))
                i += 1
                j += 1
            elif L[i] < R[j]:
                i += 1
            else:
                j += 1
        if len(rows) > C + 1:
            st = "fail"
        res.append((st, rows))
    f = next(k for k, (st, _) in enumerate(res) if st != "reached")
    out = [r for k in range(f + (res[f][0] == "end")) for r in res[k][1]]
    if res[f][0] == "fail":
        out += _walk(L, R, f * C, js[f])
    return out


def test_speculative_merge_equals_the_sequential_walk():
    rnd = random.Random(5)
    alpha = [b"a", b"b", b"/", b".", b"0", b"1", b"2", b"-", b"_"]
    seen = set()
    for _ in range(1500):
        names = sorted({b"r" + b"".join(rnd.choice(alpha) for _ in range(rnd.randint(0, 4)))
                        for _ in range(rnd.randint(0, 200))})
        L, R = [], []
        for nm in names:
            p = rnd.random()
            if p < 0.7:
                L.append(nm + b"/1")
                R.append(nm + b"/2")
            elif p < 0.8:
                L.append(nm + b"/1")
            elif p < 0.9:
                R.append(nm + b"/2")
            else:
                L.append(nm)
                R.append(nm + b"/" + rnd.choice([b"1", b"2", b"3"]))
        if L and rnd.random() < 0.3:
            L.append(rnd.choice(L))
        L.sort()
        R.sort()
        C = rnd.choice([1, 2, 3, 8])
        assert _speculative(L, R, C) == _walk(L, R)
        seen.add(len(L) > C)
    assert seen == {True, False}


# ---- drand48 jump-ahead (tk_norm.cu lcg_tables / lcg_jump)

def test_drand48_jump_ahead():
    a, c, mask = 0x5DEECE66D, 0xB, (1 << 48) - 1
    A, Cc = [a], [c]
    for _ in range(47):
        Cc.append((A[-1] * Cc[-1] + Cc[-1]) & mask)
        A.append((A[-1] * A[-1]) & mask)

    def jump(x0, steps):
        ma, mc = 1, 0
        for b in range(48):
            if steps >> b & 1:
                mc = (A[b] * mc + Cc[b]) & mask
                ma = (A[b] * ma) & mask
        return (ma * x0 + mc) & mask

    x0 = (12345 << 16) | 0x330E
    x = x0
    for k in range(1, 3000):
        x = (a * x + c) & mask
        assert jump(x0, k) == x
    assert math.isclose(jump(x0, 1) / 2 ** 48, 0.22532851279629895, rel_tol=0, abs_tol=0)
