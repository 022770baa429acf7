"""tk_coverage_stats_noalloc: the coverage statistics for callers that cannot
allocate device memory while computing (their HBM is already divided among
jobs, or an allocation failure or cudaMalloc's implicit synchronisation is not
acceptable mid-run).  Checked through the C ABI against the allocating entry
point, bit for bit, on two calls in a row that share the static scratch slab.

This file is collected last on purpose, so a failure here leaves every other
test already run."""
import ctypes as C

import numpy as np
import pytest

from trinityrnaseq_gb300 import KmerTable, ReadSet, coverage_stats, native, synth

pytestmark = pytest.mark.gpu


def _reads() -> bytes:
    short = synth.transcriptome_reads(seed=31, n_reads=20000).tobytes()
    rnd = np.random.default_rng(7)
    longs = []
    for i in range(12):  # reads above 256 windows go through the static slab
        L = int(rnd.integers(300, 5000))
        s = rnd.choice(np.frombuffer(b"ACGT", dtype=np.uint8), L)
        s[rnd.integers(0, L, 2)] = ord("N")
        longs.append(b">long%d\n" % i + s.tobytes() + b"\n")
    return short[:900000] + b"".join(longs) + short[900000:]


def _call(lib, table, rs, torch, dev):
    n = rs.n_reads
    med = torch.full((n,), 0x5EED, dtype=torch.int32, device=dev)        # poisoned: every entry must be written
    mean = torch.full((n,), float("nan"), dtype=torch.float32, device=dev)
    sd = torch.full((n,), float("nan"), dtype=torch.float32, device=dev)
    torch.cuda.synchronize(dev)
    st = lib.tk_coverage_stats_noalloc(table.h, rs.h, C.c_void_p(med.data_ptr()), C.c_void_p(mean.data_ptr()),
                                       C.c_void_p(sd.data_ptr()))
    assert st == native.TK_OK, lib.tk_ctx_last_error(table.ctx.h)
    return (med.cpu().numpy().view(np.uint32), mean.cpu().numpy(), sd.cpu().numpy())


def test_noalloc_matches_allocating_path_twice(ctx):
    torch = pytest.importorskip("torch")
    dev = torch.device(f"cuda:{ctx.device}")
    lib = native.load()
    text = _reads()
    table = KmerTable(ctx, 25, True)
    table.count_text(text + text[:200000])
    rs = ReadSet(ctx, text)
    assert rs.max_len > 280
    want = coverage_stats(table, rs)
    for _ in range(2):
        got = _call(lib, table, rs, torch, dev)
        np.testing.assert_array_equal(got[0], want[0])
        np.testing.assert_array_equal(got[1].view(np.uint32), want[1].view(np.uint32))
        np.testing.assert_array_equal(got[2].view(np.uint32), want[2].view(np.uint32))


def test_noalloc_rejects_reads_beyond_its_limit(ctx):
    torch = pytest.importorskip("torch")
    dev = torch.device(f"cuda:{ctx.device}")
    lib = native.load()
    text = b">huge\n" + b"ACGT" * 33000 + b"\n"        # 132,000 bases: 131,976 windows > 131,072
    table = KmerTable(ctx, 25, True)
    rs = ReadSet(ctx, text)
    out = torch.zeros(3, dtype=torch.int32, device=dev)
    st = lib.tk_coverage_stats_noalloc(table.h, rs.h, C.c_void_p(out.data_ptr()), C.c_void_p(out.data_ptr()),
                                       C.c_void_p(out.data_ptr()))
    assert st == native.TK_E_RANGE
    assert b"131072" in lib.tk_ctx_last_error(ctx.h)
