"""The integer algorithms of csrc/tk_norm.cu and csrc/tk_parse.cu, restated in
Python and checked on the CPU against what they stand in for: printf's "%g"
and "%.1f" (the decimal digits of a float, rounded half to even on its binary
value, and the double Perl reads back from that text), the speculative
chunked two-cursor merge of nbkc_merge_left_right_stats.pl against the plain
sequential walk, drand48's jump-ahead against stepping it draw by draw, and
the word-wise byte movement of the parse and the extraction against plain
copies.  The GPU parity tests (tests/test_gpu_norm.py, test_gpu_count.py,
test_gpu_prep.py) check the CUDA code itself."""
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


# ---- byte-movement algorithms of the parse and the extraction

M32 = 0xFFFFFFFF


def _fold_and_ws(x):
    """tk_parse.cu copy_group: 4 bytes upper-cased, and whether any is
    whitespace (' ' or 9..13), with SIMD bit tricks on one 32-bit word."""
    t = x & 0x7F7F7F7F
    lower = ((t + 0x1F1F1F1F) & M32) & (~((t + 0x05050505) & M32) & M32) & (~x & M32) & 0x80808080
    sp = x ^ 0x20202020
    zsp = (~((((sp & 0x7F7F7F7F) + 0x7F7F7F7F) & M32) | sp) & M32) & 0x80808080
    rng = ((t + 0x77777777) & M32) & (~((t + 0x72727272) & M32) & M32) & (~x & M32) & 0x80808080
    return x ^ (lower >> 2), (zsp | rng) != 0


def test_simd_case_fold_and_whitespace():
    rnd = random.Random(11)
    cases = [[c, f, f, f] for c in range(256) for f in (0x41, 0x00, 0xFF, 0x20, 0x61)]
    cases += [[rnd.randrange(256) for _ in range(4)] for _ in range(50000)]
    for bs in cases:
        x = sum(b << (8 * i) for i, b in enumerate(bs))
        up, ws = _fold_and_ws(x)
        assert up == sum((b - 32 if 97 <= b <= 122 else b) << (8 * i) for i, b in enumerate(bs))
        assert ws == any(b == 32 or 9 <= b <= 13 for b in bs)


def test_word_copy_of_lines():
    """Aligned 4-byte output words per line, source words by funnel shift,
    partial words at the line's ends byte by byte (line_word / copy_group)."""
    rnd = random.Random(3)
    for _ in range(2000):
        L = rnd.randint(1, 400)
        text = bytes(rnd.choice(b"acgtACGTN") for _ in range(L))
        S = rnd.randrange(0, L)
        n = rnd.randint(1, L - S)
        d0 = rnd.randrange(0, 50)
        out = bytearray(d0 + n + 8)
        want = bytearray(out)
        want[d0:d0 + n] = text[S:S + n].upper()
        for w in range(((d0 + n + 3) >> 2) - (d0 >> 2)):
            so = 4 * w - (d0 & 3)
            a = S + so
            if a >= 0 and (a & ~3) + 8 <= L:
                bs = list(text[a & ~3:(a & ~3) + 8][a & 3:(a & 3) + 4])
            else:
                bs = [text[S + so + i] if 0 <= so + i < n else 0x41 for i in range(4)]
            bs = [bs[i] if 0 <= so + i < n else 0x41 for i in range(4)]
            up, _ = _fold_and_ws(sum(b << (8 * i) for i, b in enumerate(bs)))
            o = (d0 & ~3) + 4 * w
            for i in range(4):
                if 0 <= so + i < n:
                    out[o + i] = (up >> (8 * i)) & 0xFF
        assert out == want


def test_chunked_record_copy():
    """tk_norm.cu k_extract_copy: a block's records as aligned 16-byte
    chunks, the holding record by binary search, boundary chunks byte by byte."""
    rnd = random.Random(9)
    EX = 256
    for _ in range(150):
        n = rnd.randint(1, 900)
        lens = [rnd.randint(1, 60) for _ in range(n)]
        pos = rnd.randint(0, 7)
        text = bytearray(rnd.getrandbits(8) for _ in range(pos))
        name_off = []
        for ln in lens:
            name_off.append(pos + 1)
            text += bytes(rnd.getrandbits(8) for _ in range(ln))
            pos += ln
        text += bytes(rnd.getrandbits(8) for _ in range(rnd.randint(0, 30)))
        rec = [ln if rnd.random() < 0.6 else 0 for ln in lens]
        off = [0]
        for ln in rec:
            off.append(off[-1] + ln)
        base = rnd.randint(0, 40)
        out = bytearray(b"\xee" * (base + off[-1] + 64))
        want = bytearray(out)
        for i in range(n):
            want[base + off[i]:base + off[i] + rec[i]] = text[name_off[i] - 1:name_off[i] - 1 + rec[i]]
        for blk in range((n + EX - 1) // EX):
            r0 = blk * EX
            m = min(n - r0, EX)
            s_off = [base + off[r0 + i] for i in range(m + 1)]
            s_src = [name_off[r0 + i] - 1 for i in range(m)]
            O0, O1 = s_off[0], s_off[m]
            for cidx in range(O0 >> 4, (O1 + 15) >> 4) if O1 > O0 else ():
                b = 16 * cidx
                key = max(b, O0)
                lo, hi = 0, m
                while hi - lo > 1:
                    mid = (lo + hi) >> 1
                    lo, hi = (mid, hi) if s_off[mid] <= key else (lo, mid)
                a = s_src[lo] + (b - s_off[lo])
                if b >= O0 and b + 16 <= s_off[lo + 1] and (a & ~3) + 20 <= len(text):
                    out[b:b + 16] = text[a:a + 16]
                else:
                    r = lo
                    for i in range(16):
                        q = b + i
                        if q < O0 or q >= O1:
                            continue
                        while q >= s_off[r + 1]:
                            r += 1
                        out[q] = text[s_src[r] + (q - s_off[r])]
        assert out == want
