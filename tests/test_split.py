"""tk_split_records (host code, no GPU): record-aligned cuts of FASTA and
FASTQ texts, including FASTQ quality lines that begin with '@'."""
import pytest

from trinityrnaseq_gb300 import kmer, synth


def fastq_with_at_quality(seed, pairs):
    left, _ = synth.gene_pairs(seed=seed, n_genes=100, n_pairs=pairs, fastq=True)
    lines = left.tobytes().split(b"\n")
    for i in range(3, len(lines), 4):   # quality lines
        if i % 8 == 3 and lines[i]:
            lines[i] = b"@" + lines[i][1:]
    return b"\n".join(lines)


@pytest.mark.parametrize("n", [1, 2, 3, 7, 64])
def test_fastq_cuts_at_records(native_built, n):
    t = fastq_with_at_quality(5, 5000)
    cuts = kmer.split_records(t, n)
    assert len(cuts) == n + 1 and cuts[0] == 0 and cuts[-1] == len(t)
    assert all(a <= b for a, b in zip(cuts, cuts[1:]))
    for a, b in zip(cuts, cuts[1:]):
        if b > a:
            piece = t[a:b].split(b"\n")
            assert piece[0].startswith(b"@") and piece[2].startswith(b"+")
            assert len([x for x in piece if x]) % 4 == 0


def test_fasta_cuts_at_headers(native_built):
    fa = synth.gene_pairs(seed=6, n_genes=100, n_pairs=3000, fastq=False)[0].tobytes()
    for n in (2, 5, 1000):
        cuts = kmer.split_records(fa, n)
        for a, b in zip(cuts, cuts[1:]):
            if b > a:
                assert fa[a:a + 1] == b">"


def test_tiny_and_empty_texts(native_built):
    assert kmer.split_records(b"", 3) == [0, 0, 0, 0]
    t = b">a\nACGT\n"
    assert kmer.split_records(t, 4) == [0, len(t), len(t), len(t), len(t)]
