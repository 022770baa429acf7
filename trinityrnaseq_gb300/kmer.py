"""Host-side mirror of the three reference tools over the C ABI.

``KmerTable`` is ``jellyfish count/histo/dump`` (Trinity:2612-2638),
``coverage_stats`` is Inchworm's ``fastaToKmerCoverageStats``
(util/insilico_read_normalization.pl:837-846) and ``ReadsToTranscripts`` is
Chrysalis' ``ReadsToTranscripts`` (Trinity:2237-2251).  The ``format_*``
helpers write the reference's text formats; the C++ drop-in executables under
``tools/`` write the same bytes.
"""
from __future__ import annotations

import atexit
import ctypes as C
from typing import Optional, Sequence, Tuple, Union

import numpy as np

from . import native as N

# At interpreter exit the library is not called any more: handles still alive
# are left to the process teardown (the driver reclaims the device memory),
# so that no CUDA state another library in the process (PyTorch) still uses
# is released under it while that library tears down its own objects.
_exiting = False


@atexit.register
def _at_exit() -> None:
    global _exiting
    _exiting = True


def _live() -> bool:
    return not _exiting


Buffer = Union[bytes, bytearray, memoryview, np.ndarray]


def _host_ptr(buf: Buffer) -> Tuple[int, int, object]:
    """(address, length, keep-alive) of a host buffer."""
    if isinstance(buf, np.ndarray):
        a = np.ascontiguousarray(buf)
        return a.ctypes.data, a.nbytes, a
    if isinstance(buf, (bytes, bytearray)):
        a = np.frombuffer(buf, dtype=np.uint8)
        return (a.ctypes.data if a.size else 0), a.size, (buf, a)
    if isinstance(buf, memoryview):
        a = np.frombuffer(buf, dtype=np.uint8)
        return (a.ctypes.data if a.size else 0), a.size, (buf, a)
    raise TypeError(f"unsupported buffer type {type(buf)}")


def split_records(text: Buffer, n_chunks: int) -> list:
    """n_chunks + 1 record-aligned cut offsets of a host FASTA/FASTQ text
    (tk_split_records; host code, no GPU needed)."""
    lib = N.load()
    ptr, n, keep = _host_ptr(text)
    cuts = (C.c_uint64 * (n_chunks + 1))()
    st = lib.tk_split_records(C.c_void_p(ptr), n, n_chunks, cuts)
    if st != N.TK_OK:
        raise N.TrinkmerError(st, "tk_split_records")
    return list(cuts)


class Context:
    """A CUDA device context with its own stream (tk_ctx).  close() destroys
    the stream: objects of other libraries that used it (e.g. PyTorch tensors
    allocated or copied under a torch.cuda.ExternalStream of `stream`) must be
    released first."""

    def __init__(self, device: int = 0):
        self.lib = N.load()
        h = C.c_void_p()
        st = self.lib.tk_ctx_create(device, C.byref(h))
        N.check(st, "tk_ctx_create")
        self.h = h
        self.device = device

    def close(self) -> None:
        if getattr(self, "h", None) and _live():
            self.lib.tk_ctx_destroy(self.h)
        self.h = None

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def check(self, st: int, where: str) -> None:
        N.check(st, where, self.h)

    @property
    def stream(self) -> int:
        return self.lib.tk_ctx_stream(self.h) or 0

    def synchronize(self) -> None:
        self.check(self.lib.tk_ctx_synchronize(self.h), "tk_ctx_synchronize")

    def set_profiling(self, on: bool) -> None:
        self.check(self.lib.tk_ctx_set_profiling(self.h, int(on)), "tk_ctx_set_profiling")

    def reset_profile(self) -> None:
        self.check(self.lib.tk_ctx_reset_profile(self.h), "tk_ctx_reset_profile")

    def profile(self, kernel: str) -> Tuple[float, int, int]:
        ms, ln, un = C.c_double(), C.c_uint64(), C.c_uint64()
        self.check(self.lib.tk_ctx_profile(self.h, N.KID[kernel], C.byref(ms), C.byref(ln), C.byref(un)),
                   "tk_ctx_profile")
        return ms.value, ln.value, un.value

    @property
    def kernel_launches(self) -> int:
        return int(self.lib.tk_ctx_kernel_launches(self.h))

    def set_reprobes(self, n: int) -> None:
        self.check(self.lib.tk_ctx_set_reprobes(self.h, int(n)), "tk_ctx_set_reprobes")

    def random_access_rate(self, table_bytes: int, atomics: bool = False) -> float:
        """Measured random 8-byte accesses/s into a table of about table_bytes."""
        r = C.c_double()
        self.check(self.lib.tk_ctx_random_access_rate(self.h, table_bytes, int(atomics), C.byref(r)),
                   "tk_ctx_random_access_rate")
        return r.value

    def trim(self) -> None:
        """Gives the context's cached device blocks back to the driver (tk_ctx_trim)."""
        self.check(self.lib.tk_ctx_trim(self.h), "tk_ctx_trim")

    def mem_info(self) -> Tuple[int, int]:
        f, t = C.c_uint64(), C.c_uint64()
        self.check(self.lib.tk_ctx_mem_info(self.h, C.byref(f), C.byref(t)), "tk_ctx_mem_info")
        return f.value, t.value


class ReadSet:
    """FASTA/FASTQ text parsed into a device-resident read set (tk_reads).

    ``text`` is a host buffer, or a device address (int) with ``length`` and
    ``device=True``; a device text must outlive the read set."""

    def __init__(self, ctx: Context, text, length: Optional[int] = None, device: bool = False):
        self.ctx = ctx
        self.lib = ctx.lib
        h = C.c_void_p()
        if device:
            ptr, n, keep = int(text), int(length), None
            where = N.TK_DEVICE
        else:
            ptr, n, keep = _host_ptr(text)
            where = N.TK_HOST
        self._keep = keep if device else None   # a host text is copied; a device text is aliased
        self._host_text = None if device else text
        ctx.check(self.lib.tk_reads_parse(ctx.h, C.c_void_p(ptr), n, where, C.byref(h)), "tk_reads_parse")
        self._adopt(h)

    def _adopt(self, h) -> None:
        self.h = h
        nr, nb, ml, fm = C.c_uint64(), C.c_uint64(), C.c_uint32(), C.c_int()
        self.ctx.check(self.lib.tk_reads_info(h, C.byref(nr), C.byref(nb), C.byref(ml), C.byref(fm)), "tk_reads_info")
        self.n_reads, self.n_bases, self.max_len, self.format = nr.value, nb.value, ml.value, fm.value

    @classmethod
    def parse_many(cls, ctx: Context, texts: list) -> list:
        """Host texts -> read sets, the upload of each text overlapping the
        parse of the ones before it (tk_reads_parse_many)."""
        n = len(texts)
        ptrs, lens, keep = (C.c_void_p * n)(), (C.c_uint64 * n)(), []
        for i, t in enumerate(texts):
            ptr, ln, k = _host_ptr(t)
            ptrs[i], lens[i] = ptr, ln
            keep.append(k)
        hs = (C.c_void_p * n)()
        ctx.check(ctx.lib.tk_reads_parse_many(ctx.h, ptrs, lens, n, N.TK_HOST, hs), "tk_reads_parse_many")
        return [cls._adopted(ctx, C.c_void_p(hs[i]), texts[i]) for i in range(n)]

    @classmethod
    def _adopted(cls, ctx: Context, h, text) -> "ReadSet":
        """A read set around a handle the library returned for host text `text`."""
        rs = cls.__new__(cls)
        rs.ctx, rs.lib, rs._keep, rs._host_text = ctx, ctx.lib, None, text
        rs._adopt(h)
        return rs

    def free(self) -> None:
        if getattr(self, "h", None) and _live():
            self.lib.tk_reads_free(self.h)
            self.h = None

    def __del__(self):
        try:
            self.free()
        except Exception:
            pass

    def names(self) -> Tuple[np.ndarray, np.ndarray]:
        off = np.zeros(self.n_reads, dtype=np.uint64)
        ln = np.zeros(self.n_reads, dtype=np.uint32)
        if self.n_reads:
            self.ctx.check(self.lib.tk_reads_names(self.h, off.ctypes.data, ln.ctypes.data), "tk_reads_names")
        return off, ln

    def accessions(self) -> list:
        assert self._host_text is not None, "accessions need the host text"
        off, ln = self.names()
        t = bytes(self._host_text) if not isinstance(self._host_text, bytes) else self._host_text
        return [t[o:o + l] for o, l in zip(off.tolist(), ln.tolist())]

    def offsets(self) -> np.ndarray:
        off = np.zeros(self.n_reads + 1, dtype=np.uint64)
        self.ctx.check(self.lib.tk_reads_offsets(self.h, off.ctypes.data), "tk_reads_offsets")
        return off

    def packed(self) -> bytes:
        n = self.n_bases + self.n_reads
        buf = np.zeros(max(n, 1), dtype=np.uint8)
        self.ctx.check(self.lib.tk_reads_copy_seq(self.h, buf.ctypes.data, n), "tk_reads_copy_seq")
        return buf[:n].tobytes()

    @staticmethod
    def _fa_flags(revcomp: bool, ignore_dirty: bool, if_missing: bool) -> int:
        return (N.TK_FA_REVCOMP if revcomp else 0) | (N.TK_FA_IGNORE_DIRTY if ignore_dirty else 0) | \
               (N.TK_FA_IF_MISSING if if_missing else 0)

    def fasta_len(self, append: int = -1, revcomp: bool = False, ignore_dirty: bool = False,
                  if_missing: bool = False) -> int:
        """Converts on the device (kept with the read set); returns the FASTA size."""
        n = C.c_uint64()
        self.ctx.check(self.lib.tk_reads_to_fasta(self.h, append, self._fa_flags(revcomp, ignore_dirty, if_missing),
                                                  N.TK_HOST, None, 0, C.byref(n)), "tk_reads_to_fasta")
        return n.value

    def fasta_into(self, ptr: int, cap: int, append: int = -1, revcomp: bool = False, ignore_dirty: bool = False,
                   if_missing: bool = False, device: bool = False) -> int:
        """The FASTA text into a caller buffer (host or device address)."""
        n = C.c_uint64()
        self.ctx.check(self.lib.tk_reads_to_fasta(self.h, append, self._fa_flags(revcomp, ignore_dirty, if_missing),
                                                  N.TK_DEVICE if device else N.TK_HOST, C.c_void_p(ptr), cap,
                                                  C.byref(n)), "tk_reads_to_fasta")
        return n.value

    def to_fasta(self, append: int = -1, revcomp: bool = False, ignore_dirty: bool = False,
                 if_missing: bool = False) -> bytes:
        """FASTQ read set -> FASTA text (tk_reads_to_fasta; the read prep of
        util/support_scripts/fastQ_to_fastA.pl / seqtk-trinity seq -A)."""
        n = self.fasta_len(append, revcomp, ignore_dirty, if_missing)
        buf = np.zeros(max(n, 1), dtype=np.uint8)
        m = self.fasta_into(buf.ctypes.data, buf.size, append, revcomp, ignore_dirty, if_missing)
        return buf[:m].tobytes()

    def sequences(self) -> list:
        off = self.offsets().tolist()
        s = self.packed()
        return [s[off[i]:off[i + 1] - 1] for i in range(self.n_reads)]


class KmerTable:
    """Device-resident k-mer -> count table (tk_table): jellyfish count/histo/dump."""

    def __init__(self, ctx: Context, k: int = 25, canonical: bool = True, capacity: int = 0):
        self.ctx, self.lib, self.k, self.canonical = ctx, ctx.lib, k, canonical
        h = C.c_void_p()
        ctx.check(self.lib.tk_table_create(ctx.h, k, int(canonical), capacity, C.byref(h)), "tk_table_create")
        self.h = h

    def free(self) -> None:
        if getattr(self, "h", None) and _live():
            self.lib.tk_table_free(self.h)
            self.h = None

    def __del__(self):
        try:
            self.free()
        except Exception:
            pass

    def add(self, reads: ReadSet) -> None:
        self.ctx.check(self.lib.tk_table_add_reads(self.h, reads.h), "tk_table_add_reads")

    def add_many(self, sets: Sequence["ReadSet"]) -> None:
        """Counts several read sets in one pass over the table."""
        arr = (C.c_void_p * len(sets))(*[s.h.value for s in sets])
        self.ctx.check(self.lib.tk_table_add_reads_multi(self.h, arr, len(sets)), "tk_table_add_reads_multi")

    def count_texts(self, texts: list) -> list:
        """Host texts -> read sets, counted into the table as they land
        (tk_table_count_texts: each text's first counting pass runs while the
        later texts upload).  Returns the read sets, in order."""
        n = len(texts)
        ptrs, lens, keep = (C.c_void_p * n)(), (C.c_uint64 * n)(), []
        for i, t in enumerate(texts):
            ptr, ln, k = _host_ptr(t)
            ptrs[i], lens[i] = ptr, ln
            keep.append(k)
        hs = (C.c_void_p * n)()
        self.ctx.check(self.lib.tk_table_count_texts(self.h, ptrs, lens, n, N.TK_HOST, hs), "tk_table_count_texts")
        return [ReadSet._adopted(self.ctx, C.c_void_p(hs[i]), texts[i]) for i in range(n)]

    def count_text(self, text: Buffer) -> None:
        ptr, n, keep = _host_ptr(text)
        self.ctx.check(self.lib.tk_table_count_text(self.h, C.c_void_p(ptr), n, N.TK_HOST), "tk_table_count_text")

    def info(self, distinct: bool = True) -> Tuple[int, int, int]:
        """(distinct k-mers, occurrences added, slots); distinct=False skips the
        table scan that counts distinct k-mers and reports -1."""
        d, t, c = C.c_uint64(), C.c_uint64(), C.c_uint64()
        self.ctx.check(self.lib.tk_table_info(self.h, C.byref(d) if distinct else None, C.byref(t), C.byref(c)),
                       "tk_table_info")
        return (d.value if distinct else -1), t.value, c.value

    def histo(self, low: int = 1, high: int = 10000) -> np.ndarray:
        h = np.zeros(high - low + 3, dtype=np.uint64)
        self.ctx.check(self.lib.tk_table_histo(self.h, low, high, h.ctypes.data), "tk_table_histo")
        return h

    def dump(self, min_count: int = 1) -> Tuple[np.ndarray, np.ndarray]:
        n = C.c_uint64()
        self.ctx.check(self.lib.tk_table_dump(self.h, min_count, N.TK_HOST, None, None, 0, C.byref(n)), "tk_table_dump")
        keys = np.zeros(max(n.value, 1), dtype=np.uint64)
        cnt = np.zeros(max(n.value, 1), dtype=np.uint32)
        m = C.c_uint64()
        self.ctx.check(self.lib.tk_table_dump(self.h, min_count, N.TK_HOST, keys.ctypes.data, cnt.ctypes.data,
                                              keys.size, C.byref(m)), "tk_table_dump")
        return keys[:m.value], cnt[:m.value]

    def dump_fasta_len(self, min_count: int = 1) -> int:
        """Formats the dump on the device (kept with the table); returns its size."""
        n = C.c_uint64()
        self.ctx.check(self.lib.tk_table_dump_fasta(self.h, min_count, N.TK_HOST, None, 0, C.byref(n)),
                       "tk_table_dump_fasta")
        return n.value

    def dump_fasta_into(self, min_count: int, ptr: int, cap: int, device: bool = False) -> int:
        """Copies the dump text to a caller buffer (host or device address)."""
        m = C.c_uint64()
        self.ctx.check(self.lib.tk_table_dump_fasta(self.h, min_count, N.TK_DEVICE if device else N.TK_HOST,
                                                    C.c_void_p(ptr), cap, C.byref(m)), "tk_table_dump_fasta")
        return m.value

    def dump_fasta_into_async(self, min_count: int, ptr: int, cap: int) -> int:
        """Starts the copy of the dump text to host memory at ``ptr`` on the
        context's copy stream; the text is there after ``Context.synchronize``."""
        m = C.c_uint64()
        self.ctx.check(self.lib.tk_table_dump_fasta_async(self.h, min_count, C.c_void_p(ptr), cap, C.byref(m)),
                       "tk_table_dump_fasta_async")
        return m.value

    def dump_fasta(self, min_count: int = 1) -> bytes:
        n = self.dump_fasta_len(min_count)
        buf = np.zeros(max(n, 1), dtype=np.uint8)
        m = self.dump_fasta_into(min_count, buf.ctypes.data, buf.size)
        return buf[:m].tobytes()

    def load_pairs(self, keys: np.ndarray, counts: np.ndarray) -> None:
        k = np.ascontiguousarray(keys, dtype=np.uint64)
        c = np.ascontiguousarray(counts, dtype=np.uint32)
        self.ctx.check(self.lib.tk_table_load_pairs(self.h, k.ctypes.data, c.ctypes.data, k.size, N.TK_HOST),
                       "tk_table_load_pairs")

    def load_dump_fasta(self, text: Buffer) -> None:
        ptr, n, keep = _host_ptr(text)
        self.ctx.check(self.lib.tk_table_load_dump_fasta(self.h, C.c_void_p(ptr), n, N.TK_HOST),
                       "tk_table_load_dump_fasta")


def coverage_stats(table: KmerTable, reads: ReadSet) -> Tuple[np.ndarray, np.ndarray, np.ndarray]:
    """Per-read (median, mean, stdev) of k-mer coverage, in read order."""
    n = reads.n_reads
    med = np.zeros(max(n, 1), dtype=np.uint32)
    mean = np.zeros(max(n, 1), dtype=np.float32)
    sd = np.zeros(max(n, 1), dtype=np.float32)
    table.ctx.check(table.lib.tk_coverage_stats(table.h, reads.h, N.TK_HOST, med.ctypes.data, mean.ctypes.data,
                                                sd.ctypes.data), "tk_coverage_stats")
    return med[:n], mean[:n], sd[:n]


def coverage_stats_into(table: KmerTable, reads: ReadSet, median_ptr: int, mean_ptr: int, stdev_ptr: int,
                        device: bool = True) -> None:
    """coverage_stats writing n_reads entries to caller arrays (device addresses by default)."""
    table.ctx.check(table.lib.tk_coverage_stats(table.h, reads.h, N.TK_DEVICE if device else N.TK_HOST,
                                                C.c_void_p(median_ptr), C.c_void_p(mean_ptr),
                                                C.c_void_p(stdev_ptr)), "tk_coverage_stats")


class ReadsToTranscripts:
    """Bundle k-mer table and read-to-component vote (tk_r2t)."""

    def __init__(self, ctx: Context, bundle: Buffer, k: int = 25, strand: bool = False):
        self.ctx, self.lib, self.k, self.strand = ctx, ctx.lib, k, strand
        ptr, n, keep = _host_ptr(bundle)
        h = C.c_void_p()
        ctx.check(self.lib.tk_r2t_create(ctx.h, C.c_void_p(ptr), n, N.TK_HOST, k, int(strand), C.byref(h)),
                  "tk_r2t_create")
        self.h = h
        nr, nk = C.c_uint64(), C.c_uint64()
        ctx.check(self.lib.tk_r2t_info(h, C.byref(nr), C.byref(nk)), "tk_r2t_info")
        self.n_records, self.n_kmers = nr.value, nk.value
        ids = np.zeros(max(self.n_records, 1), dtype=np.uint64)
        ctx.check(self.lib.tk_r2t_component_ids(h, ids.ctypes.data), "tk_r2t_component_ids")
        self.component_ids = ids[:self.n_records]

    def free(self) -> None:
        if getattr(self, "h", None) and _live():
            self.lib.tk_r2t_free(self.h)
            self.h = None

    def __del__(self):
        try:
            self.free()
        except Exception:
            pass

    def assign_into(self, reads: ReadSet, rec_ptr: int, hits_ptr: int, nwin_ptr: int, device: bool = True) -> None:
        """assign() writing n_reads entries to caller arrays (device addresses by default)."""
        self.ctx.check(self.lib.tk_r2t_assign(self.h, reads.h, N.TK_DEVICE if device else N.TK_HOST,
                                              C.c_void_p(rec_ptr), C.c_void_p(hits_ptr), C.c_void_p(nwin_ptr)),
                       "tk_r2t_assign")

    def assign(self, reads: ReadSet) -> Tuple[np.ndarray, np.ndarray, np.ndarray]:
        n = reads.n_reads
        rec = np.zeros(max(n, 1), dtype=np.int32)
        hits = np.zeros(max(n, 1), dtype=np.uint32)
        nwin = np.zeros(max(n, 1), dtype=np.uint32)
        self.ctx.check(self.lib.tk_r2t_assign(self.h, reads.h, N.TK_HOST, rec.ctypes.data, hits.ctypes.data,
                                              nwin.ctypes.data), "tk_r2t_assign")
        return rec[:n], hits[:n], nwin[:n]


class DeBruijnGraphs:
    """Per-record de Bruijn graphs of a bundle (tk_dbg; Inchworm's
    FastaToDeBruijn --graph_per_record, Trinity:2298-2302).  `bundle` is a host
    buffer, or a device address with `length` and device=True."""

    def __init__(self, ctx: Context, bundle, K: int = 24, strand: bool = False, length: Optional[int] = None,
                 device: bool = False):
        self.ctx, self.lib, self.K, self.strand = ctx, ctx.lib, K, strand
        if device:
            ptr, n, where = int(bundle), int(length), N.TK_DEVICE
        else:
            ptr, n, _ = _host_ptr(bundle)
            where = N.TK_HOST
        h = C.c_void_p()
        ctx.check(self.lib.tk_dbg_create(ctx.h, C.c_void_p(ptr), n, where, K, int(strand), C.byref(h)),
                  "tk_dbg_create")
        self.h = h
        nc, nn, nt = C.c_uint64(), C.c_uint64(), C.c_uint64()
        ctx.check(self.lib.tk_dbg_info(h, C.byref(nc), C.byref(nn), C.byref(nt)), "tk_dbg_info")
        self.n_components, self.n_nodes, self.text_len = nc.value, nn.value, nt.value

    def text_into(self, ptr: int, cap: int, device: bool = False) -> int:
        self.ctx.check(self.lib.tk_dbg_text(self.h, N.TK_DEVICE if device else N.TK_HOST, C.c_void_p(ptr), cap),
                       "tk_dbg_text")
        return self.text_len

    def text(self) -> bytes:
        buf = np.zeros(max(self.text_len, 1), dtype=np.uint8)
        self.text_into(buf.ctypes.data, buf.size)
        return buf[:self.text_len].tobytes()

    def free(self) -> None:
        if getattr(self, "h", None) and _live():
            self.lib.tk_dbg_free(self.h)
            self.h = None

    def __del__(self):
        try:
            self.free()
        except Exception:
            pass


class Normalization:
    """In-silico normalization over coverage statistics (tk_norm): the sort,
    pair merge and selection util/insilico_read_normalization.pl runs through
    `sort -k1,1`, nbkc_merge_left_right_stats.pl --sorted and nbkc_normalize.pl,
    and its extraction of the selected FASTQ records.

    left_stats / right_stats are (median, mean, stdev) per read as
    coverage_stats returns them (host numpy arrays), or device addresses
    (median_ptr, mean_ptr, stdev_ptr) with device=True.  A side may be a list
    of read sets (pieces of one file; statistics in the same order).
    right=None selects on one side alone.  The read sets must outlive this
    object."""

    def __init__(self, ctx: Context, left: ReadSet, left_stats, right: Optional[ReadSet] = None, right_stats=None,
                 max_cov: int = 200, min_cov: int = 1, max_cv: int = 10000, device: bool = False):
        self.ctx, self.lib, self.h = ctx, ctx.lib, None
        self._reads = (left, right)
        keep = []

        def ptrs(stats, n):
            if stats is None:
                return (None, None, None)
            if device:
                return tuple(C.c_void_p(int(p)) for p in stats)
            med = np.ascontiguousarray(stats[0], dtype=np.uint32)
            mean = np.ascontiguousarray(stats[1], dtype=np.float32)
            sd = np.ascontiguousarray(stats[2], dtype=np.float32)
            if not (len(med) == len(mean) == len(sd) == n):
                raise ValueError("statistics must have one entry per read")
            keep.extend((med, mean, sd))
            return tuple(C.c_void_p(a.ctypes.data) for a in (med, mean, sd))

        lsets = list(left) if isinstance(left, (list, tuple)) else [left]
        rsets = (list(right) if isinstance(right, (list, tuple)) else [right]) if right is not None else []
        lp = ptrs(left_stats, sum(r.n_reads for r in lsets))
        rp = ptrs(right_stats, sum(r.n_reads for r in rsets)) if rsets else (None, None, None)
        lh = (C.c_void_p * len(lsets))(*[r.h for r in lsets])
        rh = (C.c_void_p * max(len(rsets), 1))(*[r.h for r in rsets]) if rsets else None
        h = C.c_void_p()
        ctx.check(self.lib.tk_norm_select_multi(ctx.h, lh, len(lsets), *lp, rh, len(rsets), *rp,
                                                N.TK_DEVICE if device else N.TK_HOST, max_cov, min_cov, max_cv,
                                                C.byref(h)), "tk_norm_select")
        self.h = h
        cnt = (C.c_uint64 * 4)()
        alen = C.c_uint64()
        ctx.check(self.lib.tk_norm_info(h, cnt, C.byref(alen)), "tk_norm_info")
        self.counts = {"rows": cnt[0], "selected": cnt[1], "aberrant": cnt[2], "below_min": cnt[3]}
        self.accs_len = alen.value

    def free(self) -> None:
        if getattr(self, "h", None) and _live():
            self.lib.tk_norm_free(self.h)
            self.h = None

    def __del__(self):
        try:
            self.free()
        except Exception:
            pass

    def accs(self) -> bytes:
        """nbkc_normalize.pl's output: the selected accs, one per line."""
        buf = C.create_string_buffer(max(self.accs_len, 1))
        self.ctx.check(self.lib.tk_norm_accs(self.h, N.TK_HOST, buf, self.accs_len), "tk_norm_accs")
        return buf.raw[:self.accs_len]

    def table(self) -> bytes:
        """The table nbkc_normalize.pl reads (merged pairs or sorted stats)."""
        n = C.c_uint64()
        self.ctx.check(self.lib.tk_norm_table(self.h, N.TK_HOST, None, 0, C.byref(n)), "tk_norm_table")
        buf = C.create_string_buffer(max(n.value, 1))
        self.ctx.check(self.lib.tk_norm_table(self.h, N.TK_HOST, buf, n.value, C.byref(n)), "tk_norm_table")
        return buf.raw[:n.value]

    def extract_into(self, fastq, ptr: Optional[int] = None, cap: int = 0, device: bool = False,
                     overlap: bool = False) -> int:
        """Runs the extraction (the text stays on the device) and returns its
        length; with ptr, also copies it there (host, or device address).
        fastq may be a list of read sets (one side's files or pieces).  With
        overlap (host ptr, page-locked) the copy runs on the context's copy
        stream behind later work and has landed once ctx.synchronize()
        returns (tk_norm_extract_copy_async)."""
        n = C.c_uint64()
        sets = list(fastq) if isinstance(fastq, (list, tuple)) else [fastq]
        hs = (C.c_void_p * len(sets))(*[r.h for r in sets])
        self.ctx.check(self.lib.tk_norm_extract_multi(self.h, hs, len(sets), C.byref(n)), "tk_norm_extract")
        if ptr is not None and overlap and not device:
            self.ctx.check(self.lib.tk_norm_extract_copy_async(self.h, C.c_void_p(ptr), cap),
                           "tk_norm_extract_copy_async")
        elif ptr is not None:
            self.ctx.check(self.lib.tk_norm_extract_copy(self.h, N.TK_DEVICE if device else N.TK_HOST,
                                                         C.c_void_p(ptr), cap), "tk_norm_extract_copy")
        return n.value

    def extract(self, fastq) -> bytes:
        """The selected records of a FASTQ read set, verbatim, in input order."""
        n = self.extract_into(fastq)
        buf = C.create_string_buffer(max(n, 1))
        self.ctx.check(self.lib.tk_norm_extract_copy(self.h, N.TK_HOST, buf, n), "tk_norm_extract_copy")
        return buf.raw[:n]


def count_bins(ctx: Context, text: Buffer, bin_off, k: int = 25, canonical: bool = True,
               min_count: int = 1, out: Optional[np.ndarray] = None) -> Tuple[bytes, np.ndarray, int]:
    """Per-bin k-mer dumps of back-to-back FASTA bins in one batched GPU pass
    (tk_count_bins).  Returns (dump text, n_bins + 1 byte offsets, k-mers counted);
    with `out` (a uint8 array, e.g. page-locked, large enough) the text is
    copied there and a view of it is returned instead of bytes.  The call's
    block size, slice load factor and relaunches (tk_bins_tuning) are left in
    count_bins.last_tuning."""
    ptr, n, keep = _host_ptr(text)
    off = np.ascontiguousarray(bin_off, dtype=np.uint64)
    nb = off.size - 1
    h = C.c_void_p()
    ctx.check(ctx.lib.tk_count_bins(ctx.h, C.c_void_p(ptr), n, N.TK_HOST, off.ctypes.data, nb, k, int(canonical),
                                    min_count, C.byref(h)), "tk_count_bins")
    try:
        tl, km = C.c_uint64(), C.c_uint64()
        ctx.check(ctx.lib.tk_bins_info(h, C.byref(tl), C.byref(km)), "tk_bins_info")
        offs = np.zeros(nb + 1, dtype=np.uint64)
        ctx.check(ctx.lib.tk_bins_dump_offsets(h, offs.ctypes.data), "tk_bins_dump_offsets")
        blk, lpm, rl = C.c_int(), C.c_int(), C.c_int()
        ctx.check(ctx.lib.tk_bins_tuning(h, C.byref(blk), C.byref(lpm), C.byref(rl)), "tk_bins_tuning")
        count_bins.last_tuning = {"block": blk.value, "load": lpm.value / 1000.0, "relaunches": rl.value}
        if out is not None and out.size >= tl.value:
            ctx.check(ctx.lib.tk_bins_dump_text(h, out.ctypes.data, out.size), "tk_bins_dump_text")
            return out[:tl.value], offs, km.value
        buf = np.zeros(max(tl.value, 1), dtype=np.uint8)
        ctx.check(ctx.lib.tk_bins_dump_text(h, buf.ctypes.data, buf.size), "tk_bins_dump_text")
        return buf[:tl.value].tobytes(), offs, km.value
    finally:
        ctx.lib.tk_bins_free(h)


count_bins.last_tuning = None


# ---------------------------------------------------------------- text formats

def format_histo(hist: np.ndarray, low: int = 1, high: int = 10000, full: bool = False) -> bytes:
    """``jellyfish histo`` lines "<count> <n>": bin 0 is labelled low-1, the
    overflow bin high+1 (util/misc/insilico_norm_kmer_hists/kmer_histo.all.txt);
    empty bins are skipped unless ``full``."""
    out = []
    labels = [low - 1] + list(range(low, high + 1)) + [high + 1]
    for lab, v in zip(labels, hist.tolist()):
        if v or full:
            if lab == low - 1 and not v:
                continue
            out.append(f"{lab} {v}\n")
    return "".join(out).encode()


def format_stats(accs: Sequence[bytes], med, mean, sd, header: bool = True) -> bytes:
    """fastaToKmerCoverageStats rows: acc, median_cov, mean_cov, stdev."""
    rows = [b"acc\tmedian_cov\tmean_cov\tstdev\n"] if header else []
    for a, m, u, s in zip(accs, med.tolist(), mean.tolist(), sd.tolist()):
        rows.append(a + (f"\t{m}\t{u:g}\t{s:g}\n").encode())
    return b"".join(rows)


def format_r2t(accs: Sequence[bytes], seqs: Sequence[bytes], comp_ids, rec, hits, nwin, min_pct: int = 0) -> bytes:
    """readsToComponents rows: comp_id, '>'acc, pct, SEQ (Trinity:2474)."""
    rows = []
    for a, s, r, h, w in zip(accs, seqs, rec.tolist(), hits.tolist(), nwin.tolist()):
        if r < 0 or w == 0:
            continue
        pct = (100 * h) // w
        if min_pct > 0 and pct < min_pct:
            continue
        rows.append(b"%d\t>%s\t%d\t%s\n" % (int(comp_ids[r]), a, pct, s))
    return b"".join(rows)
