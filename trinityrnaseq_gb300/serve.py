"""Python side of the job server (tk_server_* in include/trinkmer.h)."""
from __future__ import annotations

import ctypes as C
from typing import Dict, List, Optional, Tuple

import numpy as np

from . import native as N
from .kmer import _host_ptr, _live


class Server:
    """Continuous-batching job server: `slots` concurrent jobs on one GPU,
    admitted by an HBM budget in bytes (0 = 80% of free memory)."""

    def __init__(self, device: int = 0, slots: int = 4, hbm_budget: int = 0):
        self.lib = N.load()
        h = C.c_void_p()
        N.check(self.lib.tk_server_create(device, slots, hbm_budget, C.byref(h)), "tk_server_create")
        self.h = h
        self._keep: Dict[int, object] = {}

    def close(self) -> None:
        if getattr(self, "h", None) and _live():
            self.lib.tk_server_destroy(self.h)
        self.h = None

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def _submit(self, kind, text, text2=b"", k=25, canonical=True, strand=False, min_count=1, norm=(0, 0, 0)) -> int:
        p1, n1, k1 = _host_ptr(text)
        p2, n2, k2 = _host_ptr(text2)
        spec = N.JobSpec(kind, k, int(canonical), int(strand), min_count, p1, n1, p2, n2, *norm)
        jid = C.c_uint64()
        N.check(self.lib.tk_server_submit(self.h, C.byref(spec), C.byref(jid)), "tk_server_submit")
        self._keep[jid.value] = (text, text2, k1, k2)   # inputs must outlive the job
        return jid.value

    def submit_count(self, reads, k=25, canonical=True, min_count=1) -> int:
        return self._submit(N.TK_JOB_COUNT, reads, b"", k, canonical, False, min_count)

    def submit_normalize(self, left, right, k=25, canonical=True, max_cov=0, min_cov=1, max_cv=10000) -> int:
        """Coverage statistics of both mates; with max_cov >= 2 also the pair
        selection and the selected records (outputs 10-13)."""
        return self._submit(N.TK_JOB_NORMALIZE, left, right, k, canonical, norm=(max_cov, min_cov, max_cv))

    def submit_r2t(self, reads, bundle, k=25, strand=False) -> int:
        return self._submit(N.TK_JOB_R2T, reads, bundle, k, not strand, strand)

    def wait(self, jid: int) -> Tuple[int, float, float]:
        st, lat, q = C.c_int(), C.c_uint64(), C.c_uint64()
        N.check(self.lib.tk_server_wait(self.h, jid, C.byref(st), C.byref(lat), C.byref(q)), "tk_server_wait")
        return st.value, lat.value / 1e6, q.value / 1e6

    def output(self, jid: int, which: int, dtype=np.uint8):
        p, n = C.c_void_p(), C.c_uint64()
        N.check(self.lib.tk_job_output(self.h, jid, which, C.byref(p), C.byref(n)), "tk_job_output")
        if dtype is None:
            return C.string_at(p, n.value) if n.value else b""
        a = np.empty(n.value // np.dtype(dtype).itemsize, dtype=dtype)
        if n.value:
            C.memmove(a.ctypes.data, p, n.value)
        return a

    def result(self, jid: int, kind: int):
        """Outputs of a completed job as Python objects (see include/trinkmer.h)."""
        if kind == N.TK_JOB_COUNT:
            return self.output(jid, 0, None), self.output(jid, 1, np.uint64)
        if kind == N.TK_JOB_NORMALIZE:
            d = (np.uint32, np.float32, np.float32, np.uint32, np.float32, np.float32)
            return tuple(self.output(jid, i, t) for i, t in enumerate(d))
        if kind == "normalize_select":
            return (self.output(jid, 10, None), tuple(int(v) for v in self.output(jid, 11, np.uint64)),
                    self.output(jid, 12, None), self.output(jid, 13, None))
        return self.output(jid, 0, np.int32), self.output(jid, 1, np.uint32), self.output(jid, 2, np.uint32)

    def error(self, jid: int) -> str:
        return (self.lib.tk_job_error(self.h, jid) or b"").decode()

    def release(self, jid: int) -> None:
        N.check(self.lib.tk_job_release(self.h, jid), "tk_job_release")
        self._keep.pop(jid, None)

    def batched_jobs(self) -> int:
        n = C.c_uint64()
        N.check(self.lib.tk_server_batched_jobs(self.h, C.byref(n)), "tk_server_batched_jobs")
        return n.value

    def held_by_free_memory(self) -> int:
        """Admission passes that left a job queued for lack of free GPU memory."""
        n = C.c_uint64()
        N.check(self.lib.tk_server_held_by_free_memory(self.h, C.byref(n)), "tk_server_held_by_free_memory")
        return n.value

    def stats(self) -> Tuple[int, int, int]:
        b, u, m = C.c_uint64(), C.c_uint64(), C.c_int()
        N.check(self.lib.tk_server_stats(self.h, C.byref(b), C.byref(u), C.byref(m)), "tk_server_stats")
        return b.value, u.value, m.value


def plain_run(ctx, kind, text, text2=b"", k=25, canonical=True, strand=False, min_count=1, norm=(200, 1, 10000)):
    """The same job through the plain single-job calls (the reference point
    a served result must equal)."""
    from .kmer import KmerTable, ReadSet, ReadsToTranscripts, coverage_stats
    if kind == N.TK_JOB_COUNT:
        t = KmerTable(ctx, k, canonical)
        t.count_text(text)
        return t.dump_fasta(min_count), t.histo(1, 10000)
    if kind == N.TK_JOB_NORMALIZE:
        rl, rr = ReadSet(ctx, text), ReadSet(ctx, text2)
        t = KmerTable(ctx, k, canonical)
        t.add_many([rl, rr])
        return coverage_stats(t, rl) + coverage_stats(t, rr)
    if kind == "normalize_select":
        from .kmer import Normalization
        rl, rr = ReadSet(ctx, text), ReadSet(ctx, text2)
        t = KmerTable(ctx, k, canonical)
        t.add_many([rl, rr])
        nm = Normalization(ctx, rl, coverage_stats(t, rl), rr, coverage_stats(t, rr), *norm)
        c = nm.counts
        return (nm.accs(), (c["rows"], c["selected"], c["aberrant"], c["below_min"]), nm.extract(rl), nm.extract(rr))
    z = ReadsToTranscripts(ctx, text2, k, strand)
    return z.assign(ReadSet(ctx, text))
