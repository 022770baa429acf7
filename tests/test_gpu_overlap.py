"""The overlapped host-transfer entry points: tk_reads_parse_many (uploads
queued on the copy stream, each text parsed as soon as it lands) and
tk_table_dump_fasta_async (the dump's download overlapping later work).
Their results must equal the one-at-a-time calls byte for byte."""
import numpy as np
import pytest

from trinityrnaseq_gb300 import KmerTable, ReadSet, coverage_stats, native, synth

pytestmark = pytest.mark.gpu


def same_reads(a, b):
    assert (a.n_reads, a.n_bases, a.max_len, a.format) == (b.n_reads, b.n_bases, b.max_len, b.format)
    np.testing.assert_array_equal(a.offsets(), b.offsets())
    assert a.packed() == b.packed()
    np.testing.assert_array_equal(a.names()[0], b.names()[0])
    np.testing.assert_array_equal(a.names()[1], b.names()[1])


def test_parse_many_equals_parse(ctx, golden):
    left, right = synth.gene_pairs(seed=31, n_genes=300, n_pairs=50000, fastq=True)
    texts = [left, right, (golden / "edge.fa").read_bytes(), b"", (golden / "edge.fq").read_bytes()]
    many = ReadSet.parse_many(ctx, texts)
    assert len(many) == len(texts)
    for t, rs in zip(texts, many):
        same_reads(rs, ReadSet(ctx, t))


def test_parse_many_counts_like_separate_sets(ctx, oracle):
    left, right = synth.gene_pairs(seed=32, n_genes=300, n_pairs=40000, fastq=True)
    a = KmerTable(ctx, 25, True)
    a.add_many(ReadSet.parse_many(ctx, [left, right]))
    b = KmerTable(ctx, 25, True)
    b.add_many([ReadSet(ctx, left), ReadSet(ctx, right)])
    assert a.dump_fasta(2) == b.dump_fasta(2)
    np.testing.assert_array_equal(a.histo(1, 10000), b.histo(1, 10000))


def test_parse_many_error_returns_no_sets(ctx, golden):
    bad = b"@r1\nACGT\nX\nIIII\n"   # third line of a FASTQ record must start with '+'
    with pytest.raises(native.TrinkmerError):
        ReadSet.parse_many(ctx, [(golden / "edge.fa").read_bytes(), bad])
    # the context stays usable
    assert ReadSet(ctx, (golden / "edge.fa").read_bytes()).n_reads > 0


def test_dump_async_equals_dump_and_survives_table_free(ctx):
    left, right = synth.gene_pairs(seed=33, n_genes=300, n_pairs=40000, fastq=True)
    rl, rr = ReadSet.parse_many(ctx, [left, right])
    t = KmerTable(ctx, 25, True)
    t.add_many([rl, rr])
    want = t.dump_fasta(2)
    buf = np.zeros(len(want) + 64, dtype=np.uint8)
    n = t.dump_fasta_into_async(2, buf.ctypes.data, buf.size)
    assert n == len(want)
    # later work on the context runs while the copy is in flight
    stats = coverage_stats(t, rl)
    t.free()
    ctx.synchronize()
    assert buf[:n].tobytes() == want
    assert len(stats[0]) == rl.n_reads


def test_dump_async_rejects_a_short_buffer(ctx):
    t = KmerTable(ctx, 25, True)
    t.count_text(b">a\n" + b"ACGT" * 20 + b"\n")
    buf = np.zeros(4, dtype=np.uint8)
    with pytest.raises(native.TrinkmerError):
        t.dump_fasta_into_async(1, buf.ctypes.data, buf.size)
