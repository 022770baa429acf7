"""Batched per-bin counting (tk_count_bins): every bin's dump equals a
separate plain count + dump of that bin, on the GPU and in the oracle."""
import numpy as np
import pytest

from trinityrnaseq_gb300 import KmerTable, synth
from trinityrnaseq_gb300.kmer import count_bins

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("min_count", [1, 2])
def test_bins_equal_separate_plain_runs(ctx, oracle, min_count):
    text, off, reads = synth.power_law_bins(seed=3, n_bins=60, alpha=1.8, min_reads=5, max_reads=3000)
    t = text.tobytes()
    dump, toff, kmers = count_bins(ctx, t, off, 25, True, min_count)
    assert toff[0] == 0 and toff[-1] == len(dump)
    total = 0
    for b in range(len(off) - 1):
        bt = t[int(off[b]):int(off[b + 1])]
        got = dump[int(toff[b]):int(toff[b + 1])]
        keys, counts = oracle.count(bt, 25, True)
        total += int(counts.sum())
        assert got == oracle.dump(keys, counts, 25, min_count), f"bin {b}"
        if b % 15 == 0:
            plain = KmerTable(ctx, 25, True)
            plain.count_text(bt)
            assert got == plain.dump_fasta(min_count)
    assert kmers == total


def test_bins_with_empty_and_tiny_bins(ctx, oracle):
    parts = [b"", b">a\nACGTACGTACGTACGTACGTACGTACGT\n", b"", b">b\nNNNN\n>c\nACG\n",
             synth.transcriptome_reads(seed=9, n_reads=500).tobytes()]
    off = np.cumsum([0] + [len(p) for p in parts]).astype(np.uint64)
    dump, toff, _ = count_bins(ctx, b"".join(parts), off, 25, False, 1)
    for b, p in enumerate(parts):
        k, c = oracle.count(p, 25, False)
        assert dump[int(toff[b]):int(toff[b + 1])] == oracle.dump(k, c, 25, 1)


@pytest.mark.parametrize("k,n_bins,max_reads", [(25, 20000, 12), (31, 40, 400)])
def test_bins_whose_bin_and_kmer_exceed_one_word(ctx, oracle, k, n_bins, max_reads):
    # 2k + bits(bin) > 64: 20,000 bins at k = 25 (50 + 15 bits), 40 bins at
    # k = 31 (62 + 6 bits) take the two-sort (k-mer, then bin) order
    text, off, _ = synth.power_law_bins(seed=5, n_bins=n_bins, alpha=1.8, min_reads=1, max_reads=max_reads)
    t = text.tobytes()
    dump, toff, kmers = count_bins(ctx, t, off, k, True, 1)
    assert toff[0] == 0 and toff[-1] == len(dump)
    total = 0
    for b in range(n_bins):
        keys, counts = oracle.count(t[int(off[b]):int(off[b + 1])], k, True)
        total += int(counts.sum())
        assert dump[int(toff[b]):int(toff[b + 1])] == oracle.dump(keys, counts, k, 1), f"bin {b}"
    assert kmers == total


def test_load_factor_tuning_leaves_the_dumps_unchanged(ctx, oracle):
    """The first batch of at least 50M k-mers on a device times three slice
    load factors before counting; the chosen block size and load factor are
    reported, and the dumps equal those of the next (tuned) call and the
    oracle's per-bin counts."""
    text, off, _ = synth.power_law_bins(seed=17, n_bins=1000, alpha=1.8, min_reads=50, max_reads=200_000)
    t = text.tobytes()
    first, toff1, kmers = count_bins(ctx, t, off, 25, True, 1)
    tuning = count_bins.last_tuning
    assert tuning["block"] in (128, 256, 512)
    if kmers >= 50 << 20:
        assert tuning["load"] in (0.45, 0.6, 0.75)
    second, toff2, _ = count_bins(ctx, t, off, 25, True, 1)
    assert count_bins.last_tuning["load"] == tuning["load"]
    assert first == second and np.array_equal(toff1, toff2)
    for b in range(0, len(off) - 1, 97):
        keys, counts = oracle.count(t[int(off[b]):int(off[b + 1])], 25, True)
        assert first[int(toff1[b]):int(toff1[b + 1])] == oracle.dump(keys, counts, 25, 1), f"bin {b}"
