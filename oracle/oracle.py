"""ctypes wrapper of the CPU oracle (oracle.c) -- TEST INFRASTRUCTURE ONLY.

Imported by tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg,
and there only as the checker or the timed CPU reference; the package
``trinityrnaseq_gb300`` never imports it.  See oracle.h for what is pinned
against the reference and what is a documented decision ("parity unpinned").
"""
from __future__ import annotations

import ctypes as C
import subprocess
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
LIB = HERE / "_build" / "liborc.so"

_lib = None


def build() -> Path:
    subprocess.run(["make", "-s", "-C", str(HERE)], check=True)
    return LIB


def load() -> C.CDLL:
    global _lib
    if _lib is not None:
        return _lib
    if not LIB.exists():
        build()
    lib = C.CDLL(str(LIB))
    vp, u64, P = C.c_void_p, C.c_uint64, C.POINTER
    lib.orc_count.argtypes = [vp, C.c_size_t, C.c_int, C.c_int, C.c_int, C.c_int, P(vp), P(vp), P(u64)]
    lib.orc_count_sized.argtypes = [vp, C.c_size_t, C.c_int, C.c_int, C.c_int, C.c_int, u64, P(vp), P(vp), P(u64)]
    lib.orc_fastq_to_fasta.argtypes = [vp, C.c_size_t, C.c_int, C.c_int, P(vp), P(C.c_size_t), P(u64)]
    lib.orc_histo.argtypes = [vp, u64, u64, u64, vp]
    lib.orc_histo.restype = None
    lib.orc_dump.argtypes = [vp, vp, u64, C.c_int, C.c_uint32, P(vp), P(C.c_size_t)]
    lib.orc_load_dump.argtypes = [vp, C.c_size_t, C.c_int, C.c_int, P(vp), P(vp), P(u64)]
    lib.orc_cov_stats.argtypes = [vp, C.c_size_t, vp, vp, u64, C.c_int, C.c_int, C.c_int, C.c_int, P(vp),
                                  P(C.c_size_t)]
    lib.orc_cov_values.argtypes = [vp, C.c_size_t, vp, vp, u64, C.c_int, C.c_int, C.c_int, P(u64), P(vp), P(vp),
                                   P(vp)]
    lib.orc_r2t.argtypes = [vp, C.c_size_t, vp, C.c_size_t, C.c_int, C.c_int, C.c_int, C.c_int, P(vp),
                            P(C.c_size_t)]
    lib.orc_r2t_values.argtypes = [vp, C.c_size_t, vp, C.c_size_t, C.c_int, C.c_int, C.c_int, P(u64), P(vp),
                                   P(vp), P(vp)]
    lib.orc_records.argtypes = [vp, C.c_size_t, P(vp), P(C.c_size_t)]
    lib.orc_debruijn.argtypes = [vp, C.c_size_t, C.c_int, C.c_int, C.c_int, P(vp), P(C.c_size_t)]
    lib.orc_norm.argtypes = [vp, C.c_size_t, vp, C.c_size_t, C.c_int, C.c_int, C.c_int, P(vp), P(C.c_size_t), P(vp),
                             P(C.c_size_t), P(u64)]
    lib.orc_norm_extract.argtypes = [vp, C.c_size_t, vp, C.c_size_t, P(vp), P(C.c_size_t), P(u64)]
    lib.orc_free.argtypes = [vp]
    lib.orc_free.restype = None
    _lib = lib
    return lib


def _buf(text):
    """(pointer, length) of a bytes object or a contiguous uint8 numpy array,
    so that large texts reach the library without a copy."""
    if isinstance(text, np.ndarray):
        a = np.ascontiguousarray(text).view(np.uint8)
        return C.c_void_p(a.ctypes.data if a.size else None), a.size
    return text, len(text)


def _chk(st: int, what: str) -> None:
    if st != 0:
        raise RuntimeError(f"oracle {what} failed with status {st}")


def _take(ptr: C.c_void_p, n: int, dtype) -> np.ndarray:
    lib = load()
    if n == 0:
        lib.orc_free(ptr)
        return np.zeros(0, dtype=dtype)
    nbytes = n * np.dtype(dtype).itemsize
    a = np.ctypeslib.as_array((C.c_uint8 * nbytes).from_address(ptr.value)).view(dtype).copy()
    lib.orc_free(ptr)
    return a


def _take_bytes(ptr: C.c_void_p, n: int) -> bytes:
    lib = load()
    # (string_at takes a C int size: texts of 2 GB and more go through an array)
    b = (C.c_char * n).from_address(ptr.value).raw if n else b""
    lib.orc_free(ptr)
    return b


FA_REV, FA_IGNORE_DIRTY, FA_IF_MISSING = 1, 2, 4


def fastq_to_fasta(text: bytes, append: int = -1, flags: int = 0) -> bytes:
    """FASTQ -> FASTA as util/support_scripts/fastQ_to_fastA.pl prints it;
    raises ValueError(record number) on a poorly formed record unless
    FA_IGNORE_DIRTY."""
    lib = load()
    p, n, bad = C.c_void_p(), C.c_size_t(), C.c_uint64()
    st = lib.orc_fastq_to_fasta(text, len(text), append, flags, C.byref(p), C.byref(n), C.byref(bad))
    if st == -4:
        raise ValueError(bad.value)
    _chk(st, "fastq_to_fasta")
    return _take_bytes(p, n.value)


def norm(left_stats: bytes, right_stats=None, max_cov: int = 200, min_cov: int = 1, max_cv: int = 10000):
    """(table, accs, counts) of the normalization tail of
    util/insilico_read_normalization.pl over coverage-stats tables: each side
    sorted with `sort -k1,1`, nbkc_merge_left_right_stats.pl --sorted when
    right_stats is given, nbkc_normalize.pl.  counts = (rows, selected,
    aberrant, below min_cov)."""
    lib = load()
    tp, tn, ap, an = C.c_void_p(), C.c_size_t(), C.c_void_p(), C.c_size_t()
    cnt = (C.c_uint64 * 4)()
    r = right_stats if right_stats is not None else None
    _chk(lib.orc_norm(left_stats, len(left_stats), r, len(r) if r is not None else 0, max_cov, min_cov, max_cv,
                      C.byref(tp), C.byref(tn), C.byref(ap), C.byref(an), cnt), "norm")
    return _take_bytes(tp, tn.value), _take_bytes(ap, an.value), tuple(int(v) for v in cnt)


def norm_extract(fastq: bytes, accs: bytes) -> bytes:
    """The FASTQ records the accs select (make_normalized_reads_file);
    raises ValueError(number of selected names without a record) or on a
    malformed record (ValueError(0))."""
    lib = load()
    p, n, miss = C.c_void_p(), C.c_size_t(), C.c_uint64()
    fp, fl = _buf(fastq)
    st = lib.orc_norm_extract(fp, fl, accs, len(accs), C.byref(p), C.byref(n), C.byref(miss))
    if st == -4:
        raise ValueError(miss.value)
    _chk(st, "norm_extract")
    return _take_bytes(p, n.value)


def records(text: bytes) -> bytes:
    """"acc\\tsequence\\n" per record, as PerlLib/Fasta_reader.pm parses them."""
    lib = load()
    p, n = C.c_void_p(), C.c_size_t()
    _chk(lib.orc_records(text, len(text), C.byref(p), C.byref(n)), "records")
    return _take_bytes(p, n.value)


def count(text, k: int = 25, canonical: bool = True, threads: int = 0, sorted_: bool = True,
          distinct_hint: int = 0):
    """(keys, counts) of every k-mer, sorted by key (jellyfish count).  With
    distinct_hint the table is sized for about that many distinct k-mers
    (retried at full size when it was too small)."""
    lib = load()
    kp, cp, n = C.c_void_p(), C.c_void_p(), C.c_uint64()
    p, ln = _buf(text)
    st = lib.orc_count_sized(p, ln, k, int(canonical), threads, int(sorted_), distinct_hint, C.byref(kp),
                             C.byref(cp), C.byref(n))
    if st == -5 and distinct_hint:
        st = lib.orc_count_sized(p, ln, k, int(canonical), threads, int(sorted_), 0, C.byref(kp), C.byref(cp),
                                 C.byref(n))
    _chk(st, "count")
    return _take(kp, n.value, np.uint64), _take(cp, n.value, np.uint32)


def histo(counts: np.ndarray, low: int = 1, high: int = 10000) -> np.ndarray:
    lib = load()
    c = np.ascontiguousarray(counts, dtype=np.uint32)
    h = np.zeros(high - low + 3, dtype=np.uint64)
    lib.orc_histo(c.ctypes.data, c.size, low, high, h.ctypes.data)
    return h


def dump(keys: np.ndarray, counts: np.ndarray, k: int = 25, min_count: int = 1) -> bytes:
    lib = load()
    kk = np.ascontiguousarray(keys, dtype=np.uint64)
    cc = np.ascontiguousarray(counts, dtype=np.uint32)
    p, n = C.c_void_p(), C.c_size_t()
    _chk(lib.orc_dump(kk.ctypes.data, cc.ctypes.data, kk.size, k, min_count, C.byref(p), C.byref(n)), "dump")
    return _take_bytes(p, n.value)


def load_dump(text: bytes, k: int = 25, canonical: bool = True):
    lib = load()
    kp, cp, n = C.c_void_p(), C.c_void_p(), C.c_uint64()
    _chk(lib.orc_load_dump(text, len(text), k, int(canonical), C.byref(kp), C.byref(cp), C.byref(n)), "load_dump")
    return _take(kp, n.value, np.uint64), _take(cp, n.value, np.uint32)


def cov_stats(reads: bytes, keys, counts, k: int = 25, ds: bool = True, capture: bool = False,
              threads: int = 0) -> bytes:
    lib = load()
    kk = np.ascontiguousarray(keys, dtype=np.uint64)
    cc = np.ascontiguousarray(counts, dtype=np.uint32)
    p, n = C.c_void_p(), C.c_size_t()
    rp, rl = _buf(reads)
    _chk(lib.orc_cov_stats(rp, rl, kk.ctypes.data, cc.ctypes.data, kk.size, k, int(ds), int(capture),
                           threads, C.byref(p), C.byref(n)), "cov_stats")
    return _take_bytes(p, n.value)


def cov_values(reads: bytes, keys, counts, k: int = 25, ds: bool = True, threads: int = 0):
    lib = load()
    kk = np.ascontiguousarray(keys, dtype=np.uint64)
    cc = np.ascontiguousarray(counts, dtype=np.uint32)
    nr, mp, ap, sp = C.c_uint64(), C.c_void_p(), C.c_void_p(), C.c_void_p()
    rp, rl = _buf(reads)
    _chk(lib.orc_cov_values(rp, rl, kk.ctypes.data, cc.ctypes.data, kk.size, k, int(ds), threads,
                            C.byref(nr), C.byref(mp), C.byref(ap), C.byref(sp)), "cov_values")
    n = nr.value
    return _take(mp, n, np.uint32), _take(ap, n, np.float32), _take(sp, n, np.float32)


def r2t(reads: bytes, bundle: bytes, k: int = 25, strand: bool = False, min_pct: int = 0, threads: int = 0) -> bytes:
    lib = load()
    p, n = C.c_void_p(), C.c_size_t()
    _chk(lib.orc_r2t(reads, len(reads), bundle, len(bundle), k, int(strand), min_pct, threads, C.byref(p),
                     C.byref(n)), "r2t")
    return _take_bytes(p, n.value)


def r2t_values(reads: bytes, bundle: bytes, k: int = 25, strand: bool = False, threads: int = 0):
    lib = load()
    nr, rp, hp, wp = C.c_uint64(), C.c_void_p(), C.c_void_p(), C.c_void_p()
    ip, il = _buf(reads)
    bp, bl = _buf(bundle)
    _chk(lib.orc_r2t_values(ip, il, bp, bl, k, int(strand), threads, C.byref(nr),
                            C.byref(rp), C.byref(hp), C.byref(wp)), "r2t_values")
    n = nr.value
    return _take(rp, n, np.int32), _take(hp, n, np.uint32), _take(wp, n, np.uint32)


def debruijn(bundle, K: int = 24, ss: bool = False, threads: int = 0) -> bytes:
    """FastaToDeBruijn --graph_per_record -K K [--SS] output (decision D8)."""
    lib = load()
    p, n = C.c_void_p(), C.c_size_t()
    bp, bl = _buf(bundle)
    _chk(lib.orc_debruijn(bp, bl, K, int(ss), threads, C.byref(p), C.byref(n)), "debruijn")
    return _take_bytes(p, n.value)
