"""Pins the CPU oracle against fixtures made by the reference's own code
(tests/golden/make_golden.py): PerlLib/Fasta_reader.pm, util/misc/print_kmers.pl,
util/misc/kmer_counter.pl, util/support_scripts/fastQ_to_fastA.pl and the
live consumers of the coverage-stats table.  CPU only."""
import numpy as np
import pytest

from tests.helpers import (canonical_counts_from_windows, dict_to_arrays, kmer_counter_to_canonical, read_gz,
                           sort_stats, trinity_r2t_sort)


@pytest.mark.parametrize("name", ["edge", "bulk"])
def test_records_match_fasta_reader(oracle, golden, name):
    text = (golden / f"{name}.fa").read_bytes()
    assert oracle.records(text) == (golden / f"{name}.fasta_reader.tsv").read_bytes()


@pytest.mark.parametrize("name", ["edge", "bulk"])
def test_count_matches_kmer_counter_pl(oracle, golden, name):
    text = (golden / f"{name}.fa").read_bytes()
    want = dict_to_arrays(kmer_counter_to_canonical(read_gz(golden / f"{name}.kmer_counter.txt.gz")))
    keys, counts = oracle.count(text, 25, True)
    np.testing.assert_array_equal(keys, want[0])
    np.testing.assert_array_equal(counts, want[1])


@pytest.mark.parametrize("name", ["edge", "bulk"])
@pytest.mark.parametrize("canonical", [True, False])
def test_count_matches_print_kmers_pl(oracle, golden, name, canonical):
    text = (golden / f"{name}.fa").read_bytes()
    windows = read_gz(golden / f"{name}.print_kmers.txt.gz").decode().split()
    want = dict_to_arrays(canonical_counts_from_windows(windows, canonical))
    keys, counts = oracle.count(text, 25, canonical)
    np.testing.assert_array_equal(keys, want[0])
    np.testing.assert_array_equal(counts, want[1])


def test_fastq_counts_like_its_fasta(oracle, golden):
    fq = (golden / "edge.fq").read_bytes()
    fa = (golden / "edge.fastQ_to_fastA.fa").read_bytes()
    a = oracle.count(fq, 25, True)
    b = oracle.count(fa, 25, True)
    np.testing.assert_array_equal(a[0], b[0])
    np.testing.assert_array_equal(a[1], b[1])


def test_coverage_stats_accepted_by_perl_consumers(oracle, golden):
    left = (golden / "left.fa").read_bytes()
    right = (golden / "right.fa").read_bytes()
    keys, counts = oracle.count(left + right, 25, True)
    for side, txt in (("left", left), ("right", right)):
        got = sort_stats(oracle.cov_stats(txt, keys, counts, 25, True))
        assert got == (golden / f"{side}.stats").read_bytes()
    # the merged table the reference's nbkc_merge_left_right_stats.pl wrote from them
    pairs = (golden / "pairs.stats").read_text().splitlines()
    assert pairs[0].split("\t")[0] == "acc" and len(pairs) == 201


def test_stats_from_dump_at_L2_equal_stats_from_full_table(oracle, golden):
    """A k-mer absent from the -L 2 catalogue counts 1 (Changelog.txt:536-538)."""
    left = (golden / "left.fa").read_bytes()
    right = (golden / "right.fa").read_bytes()
    keys, counts = oracle.count(left + right, 25, True)
    d2 = oracle.dump(keys, counts, 25, 2)
    k2, c2 = oracle.load_dump(d2, 25, True)
    assert (c2 >= 2).all()
    assert oracle.cov_stats(left, keys, counts) == oracle.cov_stats(left, k2, c2)


def test_r2t_sorted_like_trinity(oracle, golden):
    b = (golden / "r2t.bundle.fa").read_bytes()
    r = (golden / "r2t.reads.fa").read_bytes()
    rows = oracle.r2t(r, b, 25, False, 0)
    assert trinity_r2t_sort(rows) == (golden / "r2t.out.sort").read_bytes()


def test_histo_and_dump_roundtrip(oracle, golden):
    text = (golden / "bulk.fa").read_bytes()
    keys, counts = oracle.count(text, 25, True)
    h = oracle.histo(counts, 1, 10000)
    assert h.sum() == len(keys) and h[0] == 0
    assert h[1] == (counts == 1).sum()
    for L in (1, 2, 3):
        d = oracle.dump(keys, counts, 25, L)
        k2, c2 = oracle.load_dump(d, 25, True)
        sel = counts >= L
        np.testing.assert_array_equal(k2, keys[sel])
        np.testing.assert_array_equal(c2, counts[sel])


def test_r2t_first_record_owns_shared_kmer(oracle):
    shared = "ACGTTGCAAGCTTAGCATCGATCGGATCCAGT"
    b = (">s_7\n" + shared + "X" + "T" * 30 + "\n>s_3\n" + "G" * 10 + shared + "\n").encode()
    r = (">q1\n" + shared + "\n").encode()
    rows = oracle.r2t(r, b, 25, False, 0).decode().split("\t")
    assert rows[0] == "7" and rows[1] == ">q1" and rows[2] == "100"


@pytest.mark.parametrize("fixture,append,flags", [
    ("prep.fa", -1, 0), ("prep.a1.fa", 1, 0), ("prep.rev.fa", -1, 1), ("prep.a2rev.fa", 2, 1)])
def test_fastq_to_fasta_matches_reference_script(oracle, golden, fixture, append, flags):
    """util/support_scripts/fastQ_to_fastA.pl output (no option, -a 1, --rev, -a 2 --rev)."""
    assert oracle.fastq_to_fasta((golden / "prep.fq").read_bytes(), append, flags) == (golden / fixture).read_bytes()


def test_fastq_to_fasta_dirty_records(oracle, golden):
    dirty = (golden / "prep_dirty.fq").read_bytes()
    assert oracle.fastq_to_fasta(dirty, -1, oracle.FA_IGNORE_DIRTY) == (golden / "prep_dirty.ignore.fa").read_bytes()
    with pytest.raises(ValueError) as e:
        oracle.fastq_to_fasta(dirty)
    assert e.value.args[0] == 2     # the script dies on the second record


# ---- normalization tail: the oracle against the reference scripts' own output

@pytest.mark.parametrize("args,fixture,counts", [
    ((5, 2, 1), "norm.pairs.c5.accs", (133, 49, 49, 14)),
    ((200, 1, 10000), "norm.pairs.c200.accs", (133, 99, 30, 4)),
])
def test_norm_pairs_matches_reference_scripts(oracle, golden, args, fixture, counts):
    """sort -k1,1 | nbkc_merge_left_right_stats.pl --sorted | nbkc_normalize.pl
    (insilico_read_normalization.pl:865-985); counts as the script's stderr
    summary printed them."""
    table, accs, cnt = oracle.norm((golden / "norm.left.stats").read_bytes(), (golden / "norm.right.stats").read_bytes(),
                                   *args)
    assert table == (golden / "norm.pairs.stats").read_bytes()
    assert accs == (golden / fixture).read_bytes()
    assert cnt == counts


def test_norm_single_matches_reference_script(oracle, golden):
    _, accs, cnt = oracle.norm((golden / "norm.left.stats").read_bytes(), None, 5, 2, 1)
    assert accs == (golden / "norm.left.c5.accs").read_bytes()
    assert cnt == (149, 55, 44, 29)


def test_norm_reproduces_earlier_pair_fixture(oracle, golden):
    table, accs, _ = oracle.norm((golden / "left.stats").read_bytes(), (golden / "right.stats").read_bytes(), 3, 1,
                                 10000)
    assert table == (golden / "pairs.stats").read_bytes()
    assert accs == (golden / "normalized.accs").read_bytes()


def test_norm_extract_matches_reference(oracle, golden):
    """make_normalized_reads_file with PerlLib/Fastq_reader.pm (insilico:470-584)."""
    fq = (golden / "norm.left.fq").read_bytes()
    assert oracle.norm_extract(fq, (golden / "norm.pairs.c5.accs").read_bytes()) == \
        (golden / "norm.left.c5.fq").read_bytes()
    # a selected name without a record: the script dies
    recs = fq.split(b"\n")
    drop = [i for i in range(0, len(recs) - 1, 4) if recs[i].startswith(b"@x/2")][0]
    short = b"\n".join(recs[:drop] + recs[drop + 4:])
    with pytest.raises(ValueError) as e:
        oracle.norm_extract(short, (golden / "norm.pairs.c5.accs").read_bytes())
    assert str(e.value) == "1"


def test_drand48_is_perls_rand(oracle):
    """srand(12345); rand(1) x3 as perl 5.38 printed them (%.17g)."""
    a, c, m = 0x5DEECE66D, 0xB, (1 << 48) - 1
    x = (12345 << 16) | 0x330E
    got = []
    for _ in range(3):
        x = (a * x + c) & m
        got.append(x / 2 ** 48)
    assert ["%.17g" % v for v in got] == ["0.22532851279629895", "0.91918306853355602", "0.20684125324818226"]


def test_norm_extract_fasta_matches_reference(oracle, golden):
    """make_normalized_reads_file for --seqType fa, records read by
    PerlLib/Fasta_reader.pm (control and high bytes deleted, sequence lines
    joined without whitespace, ">header\\nsequence\\n")."""
    fa = (golden / "norm.left.fa").read_bytes()
    assert oracle.norm_extract(fa, (golden / "norm.pairs.c5.fa.accs").read_bytes()) == \
        (golden / "norm.left.c5.fa").read_bytes()
    # z\xc3z cannot be carried by any FASTA record: the script dies on it
    with pytest.raises(ValueError) as e:
        oracle.norm_extract(fa, (golden / "norm.pairs.c5.accs").read_bytes())
    assert str(e.value) == "1"


def test_debruijn_text_is_what_the_partition_script_read(oracle, golden):
    """The oracle's FastaToDeBruijn text of the small bundle is the one the
    reference's partition_chrysalis_graphs_n_reads.pl was run on: per
    component it wrote, a graph file of the header plus one line per k-mer."""
    import gzip
    text = oracle.debruijn((golden / "r2t.bundle.fa").read_bytes(), 24, False)
    assert text == gzip.decompress((golden / "r2t.bundle.deBruijn.gz").read_bytes())
    lines = {}
    comp = None
    for line in text.split(b"\n")[:-1]:
        if line.startswith(b"Component"):
            comp = int(line.split()[1])
            lines[comp] = 0
        else:
            assert len(line.split(b"\t")) == 4
            lines[comp] += 1
    for row in (golden / "r2t.bundle.deBruijn.partitions").read_text().splitlines():
        c, g, _ = map(int, row.split("\t"))
        assert g == 1 + lines[c]


def test_debruijn_small_cases(oracle):
    # 'X' joins and non-ACGT bytes break windows; a record with no window is
    # left out; canonical nodes count both strands
    text = oracle.debruijn(b">s_5\nACGTACGTAAXCCC\n>s_6\nAC\n>x\nacgtNacgta\n", 4, False)
    assert text == (b"Component 5\n0\t-1\t3\tACGTA\n1\t0\t2\tCGTAC\n2\t0\t1\tCGTAA\n"
                    b"Component 2\n0\t-1\t1\tACGTA\n")
    ss = oracle.debruijn(b">s_5\nACGTACGTAAXCCC\n", 4, True)
    assert ss == b"Component 5\n0\t-1\t2\tACGTA\n1\t0\t1\tCGTAC\n2\t1\t1\tGTACG\n3\t2\t1\tTACGT\n4\t0\t1\tCGTAA\n"
    assert oracle.debruijn(b"", 24, False) == b""
