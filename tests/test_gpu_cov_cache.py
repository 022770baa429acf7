"""The coverage cache: before the first coverage pass over a large table, the
k-mers with the highest counts are copied into an L2-sized table that the
lookups try first.  A lookup that misses it reads the count table, so the
statistics must be bit-identical to the oracle's whatever the cache holds.
TRINKMER_COV_CACHE_MB=8 makes the cache 8 MB so that it is used on tables of
32 MB and more (by default it is 64 MB and serves tables of 256 MB and more).
An entry keeps 32 bits of the key's hash below its bucket index, so a cache
of 2^h buckets serves k <= (h + 32) / 2: k <= 25 at 8 MB, k <= 26 at 64 MB."""
import numpy as np
import pytest

from trinityrnaseq_gb300 import KmerTable, ReadSet, coverage_stats, synth
from tests.test_gpu_coverage_r2t import assert_stats, long_reads, window_class_reads

pytestmark = pytest.mark.gpu


@pytest.fixture
def small_cache(monkeypatch):
    monkeypatch.setenv("TRINKMER_COV_CACHE_MB", "8")


def cache_builds(ctx, fn):
    """Runs fn with profiling on; returns (fn's result, cache builds launched)."""
    ctx.set_profiling(True)
    ctx.reset_profile()
    try:
        out = fn()
        return out, ctx.profile("cov_cache")[1]
    finally:
        ctx.set_profiling(False)


def mixed_reads(k, seed=5):
    return (synth.transcriptome_reads(seed=seed, n_reads=60000).tobytes() + window_class_reads(seed, k)
            + long_reads(seed, 8, 260, 1500))


@pytest.mark.parametrize("k", [17, 25, 31])
@pytest.mark.parametrize("ds", [True, False])
def test_cache_path_matches_oracle(ctx, oracle, small_cache, k, ds):
    text = mixed_reads(k)
    keys, counts = oracle.count(text, k, ds)
    t = KmerTable(ctx, k, ds)
    t.count_text(text)
    rs = ReadSet(ctx, text)
    _, _, cap = t.info(distinct=False)
    assert cap * 16 >= 32 << 20
    got, builds = cache_builds(ctx, lambda: coverage_stats(t, rs))
    assert builds == (1 if k <= 25 else 0)      # k = 31 needs a larger cache: the table alone serves it
    assert_stats(got, oracle.cov_values(text, keys, counts, k, ds))
    # the second pass over the same table reuses the cache
    got2, builds2 = cache_builds(ctx, lambda: coverage_stats(t, rs))
    assert builds2 == 0
    assert_stats(got2, got)


def test_very_high_counts(ctx, oracle, small_cache):
    """A k-mer counted 135,000 times (poly-A reads) sits in the cache with its
    full 32-bit count, beside ordinary ones."""
    k = 25
    text = mixed_reads(k, 9) + b"".join(b">poly%d\n" % i + b"A" * 300 + b"\n" for i in range(500))
    keys, counts = oracle.count(text, k, True)
    assert counts.max() > (1 << 17)
    t = KmerTable(ctx, k, True)
    t.count_text(text)
    rs = ReadSet(ctx, text)
    got, builds = cache_builds(ctx, lambda: coverage_stats(t, rs))
    assert builds == 1
    assert_stats(got, oracle.cov_values(text, keys, counts, k, True))


def test_cache_is_rebuilt_after_the_table_changes(ctx, oracle, small_cache):
    a = mixed_reads(25, 11)
    b = synth.transcriptome_reads(seed=12, n_reads=40000).tobytes()
    t = KmerTable(ctx, 25, True)
    t.count_text(a)
    rs = ReadSet(ctx, a)
    coverage_stats(t, rs)
    t.count_text(b)
    got, builds = cache_builds(ctx, lambda: coverage_stats(t, rs))
    assert builds == 1
    keys, counts = oracle.count(a + b, 25, True)
    assert_stats(got, oracle.cov_values(a, keys, counts, 25, True))


def test_cache_over_a_loaded_catalogue(ctx, oracle, small_cache):
    """fastaToKmerCoverageStats' own case: the -L 2 catalogue loaded from its
    dump text, the reads looked up in it (absent k-mers count 1)."""
    left, right = synth.gene_pairs(seed=14, n_genes=3000, n_pairs=300000, fastq=False)
    both = left.tobytes() + right.tobytes()
    keys, counts = oracle.count(both, 25, True)
    d2 = oracle.dump(keys, counts, 25, 2)
    t = KmerTable(ctx, 25, True)
    t.load_dump_fasta(d2)
    _, _, cap = t.info(distinct=False)
    rs = ReadSet(ctx, left.tobytes())
    got, builds = cache_builds(ctx, lambda: coverage_stats(t, rs))
    assert builds == (1 if cap * 16 >= 32 << 20 else 0)
    k2, c2 = oracle.load_dump(d2, 25, True)
    assert_stats(got, oracle.cov_values(left.tobytes(), k2, c2, 25, True))


def test_default_cache_serves_large_tables(ctx, oracle):
    """With the default 64 MB cache a table of 256 MB or more gets one."""
    text = synth.transcriptome_reads(seed=21, n_reads=1_500_000).tobytes()
    t = KmerTable(ctx, 25, True)
    t.count_text(text)
    _, _, cap = t.info(distinct=False)
    rs = ReadSet(ctx, text)
    got, builds = cache_builds(ctx, lambda: coverage_stats(t, rs))
    assert builds == (1 if cap * 16 >= 256 << 20 else 0)
    keys, counts = oracle.count(text, 25, True)
    assert_stats(got, oracle.cov_values(text, keys, counts, 25, True))
