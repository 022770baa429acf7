"""tk_coverage_stats_noalloc: the coverage statistics for callers that cannot
allocate device memory while computing (their HBM is already divided among
jobs, or an allocation failure or cudaMalloc's implicit synchronisation is not
acceptable mid-run).  Checked through the C ABI against the allocating entry
point and the oracle, bit for bit, on two calls in a row that share the static
scratch slab.

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
    # reads above 256 windows go through the static slab: a dozen of 300 to
    # 5000 bases, one of exactly 257 windows and one at the slab's limit of
    # 131,072 windows (k = 25)
    lens = [int(x) for x in rnd.integers(300, 5000, 12)] + [257 + 24, 131072 + 24]
    for i, L in enumerate(lens):
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


def test_noalloc_matches_allocating_path_twice(ctx, oracle):
    """Two calls in a row against the allocating entry point and against the
    oracle's statistics of the same text (the long-read path of both entry
    points shares its helpers, so the oracle is the independent check)."""
    torch = pytest.importorskip("torch")
    dev = torch.device(f"cuda:{ctx.device}")
    lib = native.load()
    text = _reads()
    catalogue = text + text[:200000]
    table = KmerTable(ctx, 25, True)
    table.count_text(catalogue)
    rs = ReadSet(ctx, text)
    assert rs.max_len == 131072 + 24
    want = coverage_stats(table, rs)
    keys, counts = oracle.count(catalogue, 25, True)
    om, oa, osd = oracle.cov_values(text, keys, counts, 25, True)
    np.testing.assert_array_equal(want[0], om)
    for _ in range(2):
        got = _call(lib, table, rs, torch, dev)
        for g, w, o in zip(got, want, (om, oa, osd)):
            np.testing.assert_array_equal(g.view(np.uint32), w.view(np.uint32))
            np.testing.assert_array_equal(g.view(np.uint32), o.view(np.uint32))


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
