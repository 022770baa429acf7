"""GPU parity of parsing (K1), counting (K2), histo/dump (K3/K4) and
catalogue loading against the CPU oracle, through the C ABI.  Integer work:
bit-exact."""
import numpy as np
import pytest

from trinityrnaseq_gb300 import KmerTable, ReadSet, native, synth
from tests.helpers import dict_to_arrays, kmer_counter_to_canonical, read_gz

pytestmark = pytest.mark.gpu


def gpu_count(ctx, text, k=25, canonical=True, capacity=0):
    t = KmerTable(ctx, k, canonical, capacity)
    t.count_text(text)
    return t


def assert_pairs(got, want):
    np.testing.assert_array_equal(got[0], want[0])
    np.testing.assert_array_equal(got[1], want[1])


@pytest.mark.parametrize("name", ["edge", "bulk"])
def test_parse_matches_fasta_reader(ctx, golden, name):
    text = (golden / f"{name}.fa").read_bytes()
    rs = ReadSet(ctx, text)
    want = [l.split(b"\t") for l in (golden / f"{name}.fasta_reader.tsv").read_bytes().split(b"\n") if l]
    assert rs.n_reads == len(want)
    assert rs.accessions() == [w[0] for w in want]
    assert rs.sequences() == [w[1].upper() for w in want]


def test_parse_fastq(ctx, golden):
    rs = ReadSet(ctx, (golden / "edge.fq").read_bytes())
    assert rs.format == native.TK_FMT_FASTQ
    want = (golden / "edge.fastQ_to_fastA.fa").read_bytes().split(b"\n")
    assert rs.sequences() == [l for l in want[1::2] if l or True][:rs.n_reads]


@pytest.mark.parametrize("name", ["edge", "bulk"])
def test_count_matches_reference_perl_counter(ctx, golden, name):
    text = (golden / f"{name}.fa").read_bytes()
    want = dict_to_arrays(kmer_counter_to_canonical(read_gz(golden / f"{name}.kmer_counter.txt.gz")))
    assert_pairs(gpu_count(ctx, text).dump(1), want)


@pytest.mark.parametrize("k", [1, 5, 17, 24, 25, 31])
@pytest.mark.parametrize("canonical", [True, False])
def test_count_parity_k(ctx, oracle, golden, k, canonical):
    text = (golden / "edge.fa").read_bytes() + (golden / "bulk.fa").read_bytes()
    assert_pairs(gpu_count(ctx, text, k, canonical).dump(1), oracle.count(text, k, canonical))


def test_count_parity_transcriptome_1M(ctx, oracle):
    """Single-end 76-nt transcriptome workload at full size (1M reads)."""
    text = synth.transcriptome_reads(seed=1, n_reads=1_000_000).tobytes()
    t = gpu_count(ctx, text)
    want = oracle.count(text, 25, True)
    got = t.dump(1)
    assert_pairs(got, want)
    d, total, cap = t.info()
    assert d == len(want[0]) and total == int(want[1].sum()) == 52_000_000
    np.testing.assert_array_equal(t.histo(1, 10000), oracle.histo(want[1], 1, 10000))
    for L in (1, 2):
        assert t.dump_fasta(L) == oracle.dump(want[0], want[1], 25, L)


def test_count_fastq_pairs_with_n(ctx, oracle):
    left, right = synth.gene_pairs(seed=9, n_genes=300, n_pairs=20000, n_rate=0.01)
    text = left.tobytes() + right.tobytes()
    assert_pairs(gpu_count(ctx, text).dump(1), oracle.count(text, 25, True))


def test_batches_add_up(ctx, oracle):
    a = synth.transcriptome_reads(seed=3, n_reads=30000).tobytes()
    b = synth.transcriptome_reads(seed=4, n_reads=50000).tobytes()
    t = KmerTable(ctx, 25, True)
    t.count_text(a)
    t.count_text(b)
    assert_pairs(t.dump(1), oracle.count(a + b, 25, True))


def test_add_many_equals_concatenation(ctx, oracle):
    a = synth.transcriptome_reads(seed=13, n_reads=40000).tobytes()
    b, c = synth.gene_pairs(seed=14, n_genes=400, n_pairs=30000)
    sets = [ReadSet(ctx, x) for x in (a, b.tobytes(), b"", c.tobytes())]
    t = KmerTable(ctx, 25, True)
    t.add_many(sets)
    assert_pairs(t.dump(1), oracle.count(a + b.tobytes() + c.tobytes(), 25, True))
    # a second multi-set pass into the now non-empty table
    t.add_many(sets[:2])
    assert_pairs(t.dump(1), oracle.count(a + b.tobytes() + c.tobytes() + a + b.tobytes(), 25, True))


def test_large_partitioned_table(ctx, oracle):
    """Enough distinct k-mers for a multi-partition table (> 2M slots)."""
    text = synth.transcriptome_reads(seed=15, n_transcripts=4000, n_reads=600_000, err=0.02).tobytes()
    t = gpu_count(ctx, text)
    d, total, cap = t.info()
    assert cap > (1 << 21)
    assert_pairs(t.dump(1), oracle.count(text, 25, True))


def test_overflow_and_growth_are_exact(ctx, oracle):
    """Eight reprobes at up to 0.6 load: many inserts overflow, the table
    doubles and the overflow list is re-inserted; the counts stay exact."""
    text = synth.transcriptome_reads(seed=5, n_reads=3000).tobytes()
    ctx.set_reprobes(8)
    try:
        t = gpu_count(ctx, text, capacity=1024)
        got = t.dump(1)
    finally:
        ctx.set_reprobes(4096)
    assert_pairs(got, oracle.count(text, 25, True))


def test_empty_and_degenerate_inputs(ctx):
    for text in (b"", b"\n\n  \n", b">a\n\n>b\nNNNNNNNNNNNNNNNNNNNNNNNNNNNNNN\n", b">only_header"):
        t = gpu_count(ctx, text)
        k, c = t.dump(1)
        assert len(k) == 0
        assert t.dump_fasta(1) == b""
        assert int(t.histo().sum()) == 0


def test_malformed_fastq_is_an_error(ctx):
    with pytest.raises(native.TrinkmerError) as ei:
        ReadSet(ctx, b"@r1\nACGT\n+\nIIII\n@r2\nACGT\nIIII\n")
    assert ei.value.status == native.TK_E_PARSE
    with pytest.raises(native.TrinkmerError):
        ReadSet(ctx, b"@r1\nACGT\nXX\nIIII\n")


def test_load_dump_roundtrip(ctx, oracle, golden):
    text = (golden / "bulk.fa").read_bytes() + synth.transcriptome_reads(seed=8, n_reads=20000).tobytes()
    keys, counts = oracle.count(text, 25, True)
    d2 = oracle.dump(keys, counts, 25, 2)
    t = KmerTable(ctx, 25, True)
    t.load_dump_fasta(d2)
    assert_pairs(t.dump(1), oracle.load_dump(d2, 25, True))
    # a non-canonical dump loaded canonically merges strands
    kf, cf = oracle.count(text, 25, False)
    df = oracle.dump(kf, cf, 25, 1)
    t2 = KmerTable(ctx, 25, True)
    t2.load_dump_fasta(df)
    assert_pairs(t2.dump(1), oracle.load_dump(df, 25, True))


def test_load_pairs(ctx, oracle, golden):
    text = (golden / "bulk.fa").read_bytes()
    keys, counts = oracle.count(text, 25, True)
    t = KmerTable(ctx, 25, True)
    t.load_pairs(keys, counts)
    t.load_pairs(keys, counts)
    assert_pairs(t.dump(1), (keys, counts * 2))


def test_bad_dump_is_an_error(ctx):
    t = KmerTable(ctx, 25, True)
    with pytest.raises(native.TrinkmerError) as ei:
        t.load_dump_fasta(b">3\nACGTACGTACGTACGTACGTACGTA\n>x\nACGTACGTACGTACGTACGTACGTA\n")
    assert ei.value.status == native.TK_E_PARSE


def test_range_build_fallback_when_deferred_list_overruns(native_built, oracle):
    """A fresh table is built range by range in shared memory; keys whose probe
    leaves their range are deferred.  With the deferred list capped at one
    entry the build overruns it, the table is emptied and counted with global
    atomics instead: the result must not change."""
    import os
    import subprocess
    import sys
    code = (
        "import numpy as np, sys\n"
        "from trinityrnaseq_gb300 import Context, KmerTable, synth\n"
        "left, right = synth.gene_pairs(seed=41, n_genes=2000, n_pairs=300000, fastq=False)\n"
        "t = KmerTable(Context(0), 25, True)\n"
        "t.count_text(left.tobytes() + right.tobytes())\n"
        "sys.stdout.buffer.write(t.dump_fasta(1))\n")
    env = dict(os.environ, TRINKMER_DEFER_CAP="1")
    capped = subprocess.run([sys.executable, "-c", code], env=env, capture_output=True, timeout=600)
    assert capped.returncode == 0, capped.stderr[-2000:]
    left, right = synth.gene_pairs(seed=41, n_genes=2000, n_pairs=300000, fastq=False)
    keys, counts = oracle.count(left.tobytes() + right.tobytes(), 25, True)
    assert capped.stdout == oracle.dump(keys, counts, 25, 1)


def test_block_cache_trim_and_zero_cap(native_built, ctx, oracle):
    """Large blocks are cached per context after they are freed; tk_ctx_trim
    gives them back, and a zero cap (TRINKMER_BLOCK_CACHE_GB=0) frees them at
    once.  Counting is unchanged either way."""
    import os
    import subprocess
    import sys
    left, right = synth.gene_pairs(seed=43, n_genes=3000, n_pairs=1_500_000, fastq=False)
    t = KmerTable(ctx, 25, True)
    t.count_text(left.tobytes() + right.tobytes())
    assert t.info(distinct=False)[2] * 16 >= 256 << 20   # the table is a cached-size block
    t.free()
    free_before, _ = ctx.mem_info()
    ctx.trim()
    free_after, _ = ctx.mem_info()
    assert free_after >= free_before
    code = ("import sys\n"
            "from trinityrnaseq_gb300 import Context, KmerTable, synth\n"
            "left, right = synth.gene_pairs(seed=43, n_genes=3000, n_pairs=200000, fastq=False)\n"
            "t = KmerTable(Context(0), 25, True)\n"
            "t.count_text(left.tobytes() + right.tobytes())\n"
            "sys.stdout.buffer.write(t.dump_fasta(2))\n")
    p = subprocess.run([sys.executable, "-c", code], env=dict(os.environ, TRINKMER_BLOCK_CACHE_GB="0"),
                       capture_output=True, timeout=600)
    assert p.returncode == 0, p.stderr[-2000:]
    left, right = synth.gene_pairs(seed=43, n_genes=3000, n_pairs=200000, fastq=False)
    keys, counts = oracle.count(left.tobytes() + right.tobytes(), 25, True)
    assert p.stdout == oracle.dump(keys, counts, 25, 2)


def pieces_of(texts, n):
    from trinityrnaseq_gb300 import kmer
    out = []
    for a in texts:
        cuts = kmer.split_records(a, n)
        out += [a[int(cuts[i]):int(cuts[i + 1])] for i in range(n)]
    return out


def test_count_texts_equals_parse_then_add(ctx, oracle):
    """tk_table_count_texts: each host text's first counting pass runs as soon
    as it is parsed (per-text key buffers, the partitions read as one segment
    of each); the counts and the read sets equal parse_many + add_many."""
    left, right = synth.gene_pairs(seed=61, n_genes=1500, n_pairs=200000, fastq=True, n_rate=0.005)
    pieces = pieces_of((left, right), 3)
    pieces.insert(2, np.zeros(0, dtype=np.uint8))   # an empty text among them
    whole = left.tobytes() + right.tobytes()
    t = KmerTable(ctx, 25, True)
    sets = t.count_texts(pieces)
    assert_pairs(t.dump(1), oracle.count(whole, 25, True))
    ref = ReadSet.parse_many(ctx, pieces)
    assert [r.n_reads for r in sets] == [r.n_reads for r in ref]
    for a, b in zip(sets, ref):
        assert a.accessions() == b.accessions() and a.sequences() == b.sequences()
    # counted again into the now filled table (the atomic path over several key buffers)
    t.count_texts(pieces[:3])
    assert_pairs(t.dump(1), oracle.count(whole + b"".join(p.tobytes() for p in pieces[:3]), 25, True))


def test_count_texts_beyond_one_pass_of_sets(ctx, oracle):
    """More texts than one counting pass takes (64): parsed, then counted in groups."""
    text = synth.transcriptome_reads(seed=62, n_reads=70000).tobytes()
    arr = np.frombuffer(text, dtype=np.uint8)
    pieces = pieces_of((arr,), 70)
    t = KmerTable(ctx, 25, True)
    sets = t.count_texts(pieces)
    assert len(sets) == 70 and sum(r.n_reads for r in sets) == 70000
    assert_pairs(t.dump(1), oracle.count(text, 25, True))


def test_multi_set_partitioned_table_and_deferred_fallback(native_built, oracle):
    """Several read sets into a multi-partition table, by ranges and, with the
    deferred list capped at one entry, by the atomic fallback: both exact."""
    import os
    import subprocess
    import sys
    code = (
        "import sys\n"
        "from trinityrnaseq_gb300 import Context, KmerTable, ReadSet, synth\n"
        "ctx = Context(0)\n"
        "text = synth.transcriptome_reads(seed=63, n_transcripts=4000, n_reads=600_000, err=0.02).tobytes()\n"
        "q = len(text) // 3\n"
        "cut = [0, text.index(b'\\n>', q) + 1, text.index(b'\\n>', 2 * q) + 1, len(text)]\n"
        "sets = [ReadSet(ctx, text[cut[i]:cut[i + 1]]) for i in range(3)]\n"
        "t = KmerTable(ctx, 25, True)\n"
        "t.add_many(sets)\n"
        "assert t.info()[2] > (1 << 21)\n"
        "sys.stdout.buffer.write(t.dump_fasta(1))\n")
    text = synth.transcriptome_reads(seed=63, n_transcripts=4000, n_reads=600_000, err=0.02).tobytes()
    keys, counts = oracle.count(text, 25, True)
    want = oracle.dump(keys, counts, 25, 1)
    for cap in (None, "1"):
        env = dict(os.environ)
        if cap:
            env["TRINKMER_DEFER_CAP"] = cap
        run = subprocess.run([sys.executable, "-c", code], env=env, capture_output=True, timeout=600)
        assert run.returncode == 0, run.stderr[-2000:]
        assert run.stdout == want, cap


def test_count_texts_error_leaves_the_context_usable(ctx, oracle):
    """A malformed text among the pieces fails the call (no read set is
    returned, the key buffers of the texts before it are freed); the context
    and a new table still count exactly afterwards."""
    good = synth.transcriptome_reads(seed=64, n_reads=20000).tobytes()
    bad = b"@r1\nACGT\n+\nIIII\n@r2\nACGT\n"
    t = KmerTable(ctx, 25, True)
    with pytest.raises(native.TrinkmerError):
        t.count_texts([np.frombuffer(good, dtype=np.uint8), np.frombuffer(bad, dtype=np.uint8)])
    t2 = KmerTable(ctx, 25, True)
    sets = t2.count_texts([np.frombuffer(good, dtype=np.uint8)])
    assert sets[0].n_reads == 20000
    assert_pairs(t2.dump(1), oracle.count(good, 25, True))
