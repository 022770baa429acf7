"""GPU parity of coverage statistics (K5) and read-to-component assignment
(K6) against the CPU oracle through the C ABI.  Medians, hit counts and
records are integers (bit-exact); mean and stdev are the float32 values of
the documented double arithmetic and must match bit for bit as well."""
import numpy as np
import pytest

from trinityrnaseq_gb300 import KmerTable, ReadSet, ReadsToTranscripts, coverage_stats, format_r2t, format_stats, synth
from tests.helpers import sort_stats, trinity_r2t_sort

pytestmark = pytest.mark.gpu


def stats_gpu(ctx, table_text, reads_text, k=25, ds=True):
    t = KmerTable(ctx, k, ds)
    t.count_text(table_text)
    rs = ReadSet(ctx, reads_text)
    return rs, coverage_stats(t, rs)


def assert_stats(got, want):
    np.testing.assert_array_equal(got[0], want[0])
    np.testing.assert_array_equal(got[1].view(np.uint32), want[1].view(np.uint32))
    np.testing.assert_array_equal(got[2].view(np.uint32), want[2].view(np.uint32))


def long_reads(seed, n, lo, hi):
    rnd = np.random.default_rng(seed)
    out = []
    for i in range(n):
        L = int(rnd.integers(lo, hi))
        s = rnd.choice(np.frombuffer(b"ACGT", dtype=np.uint8), L)
        if i % 3 == 0:
            s[rnd.integers(0, L, 3)] = ord("N")
        out.append(b">long%d\n" % i + s.tobytes() + b"\n")
    return b"".join(out)


@pytest.mark.parametrize("ds", [True, False])
def test_stats_parity_golden(ctx, oracle, golden, ds):
    left = (golden / "left.fa").read_bytes()
    right = (golden / "right.fa").read_bytes()
    keys, counts = oracle.count(left + right, 25, ds)
    for txt in (left, right, (golden / "edge.fa").read_bytes()):
        rs, got = stats_gpu(ctx, left + right, txt, 25, ds)
        assert_stats(got, oracle.cov_values(txt, keys, counts, 25, ds))


def test_stats_table_bytes_match_the_fixture(ctx, golden):
    """The rows the reference's nbkc_merge_left_right_stats.pl consumed."""
    left = (golden / "left.fa").read_bytes()
    right = (golden / "right.fa").read_bytes()
    for side, txt in (("left", left), ("right", right)):
        rs, (m, a, s) = stats_gpu(ctx, left + right, txt)
        assert sort_stats(format_stats(rs.accessions(), m, a, s)) == (golden / f"{side}.stats").read_bytes()


def test_stats_from_catalogue_with_missing_kmers(ctx, oracle):
    left, right = synth.gene_pairs(seed=12, n_genes=500, n_pairs=40000, fastq=False)
    both = left.tobytes() + right.tobytes()
    keys, counts = oracle.count(both, 25, True)
    d2 = oracle.dump(keys, counts, 25, 2)
    t = KmerTable(ctx, 25, True)
    t.load_dump_fasta(d2)
    rs = ReadSet(ctx, left.tobytes())
    got = coverage_stats(t, rs)
    k2, c2 = oracle.load_dump(d2, 25, True)
    assert_stats(got, oracle.cov_values(left.tobytes(), k2, c2, 25, True))


def test_stats_long_and_odd_reads(ctx, oracle, golden):
    text = long_reads(1, 40, 200, 3000) + (golden / "edge.fa").read_bytes() + long_reads(2, 10, 281, 300)
    keys, counts = oracle.count(text + text[:5000], 25, True)
    rs, got = stats_gpu(ctx, text + text[:5000], text)
    assert_stats(got, oracle.cov_values(text, keys, counts, 25, True))


def window_class_reads(seed, k, n_per_len=3, nwins=None):
    """Reads whose window counts straddle every per-lane register class of the
    warp path (1, 2, 4, 8 values per lane) and the long-read path, a third of
    them with an N."""
    rnd = np.random.default_rng(seed)
    if nwins is None:
        nwins = [0, 1, 2, 31, 32, 33, 63, 64, 65, 76, 127, 128, 129, 200, 255, 256, 257, 300]
    out = []
    for nw in nwins:
        for i in range(n_per_len):
            L = max(1, nw + k - 1) if nw else max(1, k - 1 - i)
            s = rnd.choice(np.frombuffer(b"ACGT", dtype=np.uint8), L)
            if i == 2:
                s[rnd.integers(0, L)] = ord("N")
            out.append(b">w%d_%d\n" % (nw, i) + s.tobytes() + b"\n")
    return b"".join(out)


@pytest.mark.parametrize("k", [1, 7, 17, 25, 31])
@pytest.mark.parametrize("ds", [True, False])
def test_stats_every_window_class_and_k(ctx, oracle, k, ds):
    text = window_class_reads(k, k)
    catalogue = text + window_class_reads(100 + k, k)
    keys, counts = oracle.count(catalogue, k, ds)
    rs, got = stats_gpu(ctx, catalogue, text, k, ds)
    assert_stats(got, oracle.cov_values(text, keys, counts, k, ds))


@pytest.mark.parametrize("longest", [96, 128])
@pytest.mark.parametrize("ds", [True, False])
def test_stats_narrow_read_sets(ctx, oracle, longest, ds):
    """Read sets whose longest read has at most 96 or 128 windows go to the
    kernels compiled only for those classes (8 blocks per SM)."""
    nw = [w for w in (0, 1, 2, 31, 32, 33, 63, 64, 65, 76, 95, 96, 97, 127, 128) if w <= longest]
    text = window_class_reads(7, 25, 4, nw) + synth.transcriptome_reads(seed=8, n_reads=20000).tobytes()
    catalogue = text + window_class_reads(107, 25, 4, nw)
    keys, counts = oracle.count(catalogue, 25, ds)
    rs, got = stats_gpu(ctx, catalogue, text, 25, ds)
    assert_stats(got, oracle.cov_values(text, keys, counts, 25, ds))


def test_stats_parity_1M_reads(ctx, oracle):
    text = synth.transcriptome_reads(seed=1, n_reads=1_000_000).tobytes()
    keys, counts = oracle.count(text, 25, True)
    rs, got = stats_gpu(ctx, text, text)
    assert_stats(got, oracle.cov_values(text, keys, counts, 25, True))


@pytest.mark.parametrize("strand", [False, True])
def test_r2t_parity_golden(ctx, oracle, golden, strand):
    b = (golden / "r2t.bundle.fa").read_bytes()
    r = (golden / "r2t.reads.fa").read_bytes()
    z = ReadsToTranscripts(ctx, b, 25, strand)
    rs = ReadSet(ctx, r)
    got = z.assign(rs)
    want = oracle.r2t_values(r, b, 25, strand)
    for g, w in zip(got, want):
        np.testing.assert_array_equal(g, w)
    rows = format_r2t(rs.accessions(), rs.sequences(), z.component_ids, *got)
    assert rows == oracle.r2t(r, b, 25, strand, 0)
    if not strand:
        assert trinity_r2t_sort(rows) == (golden / "r2t.out.sort").read_bytes()


def test_r2t_parity_medium_and_long(ctx, oracle):
    b, r = synth.bundle_reads(seed=21, n_contigs=5000, n_components=1500, max_per_component=40, n_pairs=100000)
    b, r = b.tobytes(), r.tobytes()
    r = r + long_reads(3, 30, 250, 2000)
    z = ReadsToTranscripts(ctx, b)
    rs = ReadSet(ctx, r)
    got = z.assign(rs)
    want = oracle.r2t_values(r, b, 25, False)
    for g, w in zip(got, want):
        np.testing.assert_array_equal(g, w)
    for p in (0, 10, 50):
        assert format_r2t(rs.accessions(), rs.sequences(), z.component_ids, *got, min_pct=p) == \
            oracle.r2t(r, b, 25, False, p)


def test_r2t_first_record_owns_shared_kmer(ctx):
    shared = b"ACGTTGCAAGCTTAGCATCGATCGGATCCAGT"
    b = b">s_7\n" + shared + b"X" + b"T" * 30 + b"\n>s_3\n" + b"G" * 10 + shared + b"\n"
    z = ReadsToTranscripts(ctx, b)
    rs = ReadSet(ctx, b">q1\n" + shared + b"\n>q2\nGGGGGGGGGG\n")
    rec, hits, nwin = z.assign(rs)
    assert rec.tolist() == [0, -1] and hits.tolist() == [8, 0] and nwin.tolist() == [8, 0]
    assert z.component_ids.tolist() == [7, 3]
