#!/usr/bin/env python3
"""Regenerates the golden fixtures of tests/golden/ from the reference's own
Perl code (run here, where the reference checkout and Perl are available; the
fixtures are committed so nothing at test time needs the reference).

    python tests/golden/make_golden.py /path/to/trinityrnaseq [--prep-only]

What each fixture pins:
  edge.fa / bulk.fa          inputs (edge cases: multi-line records, lower case,
                             N and IUPAC bases, CRLF, blank lines, short and
                             empty reads; bulk: 300 seeded 76-nt reads)
  *.fasta_reader.tsv         acc and sequence per record from PerlLib/Fasta_reader.pm
  *.print_kmers.txt.gz       every window in order from util/misc/print_kmers.pl
  *.kmer_counter.txt.gz      k-mer counts from util/misc/kmer_counter.pl in DS
                             mode (each window and its reverse complement)
  edge.fq / edge.fastQ_to_fastA.fa
                             FASTQ records through util/support_scripts/fastQ_to_fastA.pl
  prep.fq / prep*.fa         the FASTQ->FASTA prep through fastQ_to_fastA.pl with no
                             option, -a 1, --rev, -a 2 --rev (Casava comments, CR, IUPAC)
  prep_dirty.fq / prep_dirty.ignore.fa
                             poorly formed records, --ignore_dirty
  left.fa right.fa           200 seeded read pairs (2x100)
  left.stats right.stats     the oracle's fastaToKmerCoverageStats tables, sorted
                             as util/insilico_read_normalization.pl:865-892 does
  pairs.stats                util/support_scripts/nbkc_merge_left_right_stats.pl --sorted
  normalized.accs            util/support_scripts/nbkc_normalize.pl --max_cov 3
                             --min_cov 1 --max_CV 10000 on pairs.stats
  r2t.bundle.fa r2t.reads.fa small bundle and reads
  r2t.out.sort               the oracle's readsToComponents rows through
                             `sort -k1,1n -k3,3nr -k2,2` under LC_ALL=C (Trinity:2258)
"""
import gzip
import os
import random
import subprocess
import sys
from pathlib import Path

HERE = Path(__file__).resolve().parent
ROOT = HERE.parent.parent
sys.path.insert(0, str(ROOT))

from oracle import oracle as O  # noqa: E402
from trinityrnaseq_gb300 import synth  # noqa: E402


def edge_fasta() -> bytes:
    rnd = random.Random(20240601)

    def s(n, alphabet="ACGT"):
        return "".join(rnd.choice(alphabet) for _ in range(n))

    recs = []
    recs.append("\n\n")                                       # leading blank lines
    recs.append(">plain1 some comment\n" + s(76) + "\n")
    recs.append(">multi2\n" + s(40) + "\n" + s(40) + "\n" + s(13) + "\n")   # k-mers across line breaks
    recs.append(">lower3\n" + s(30).lower() + s(30) + "\n")
    recs.append(">withN4\n" + s(20) + "N" + s(30) + "NN" + s(28) + "\n")
    recs.append(">iupac5\n" + s(35) + "R" + s(35) + "\n")
    recs.append(">short6\n" + s(24) + "\n")                    # shorter than k
    recs.append(">exact7\n" + s(25) + "\n")                    # exactly one window
    recs.append(">empty8\n\n")                                 # empty sequence
    recs.append(">crlf9\r\n" + s(50) + "\r\n" + s(20) + "\r\n")
    recs.append(">spaces10\n" + s(30) + " " + s(30) + "\t" + s(10) + "\n")
    recs.append(">allN11\n" + "N" * 60 + "\n")
    recs.append(">dup12\n" + "ACGT" * 20 + "\n")                # periodic, many repeats
    recs.append(">homopolymer13\n" + "A" * 80 + "\n")
    recs.append(">palin14\n" + "ACGTACGTACGTACGTACGTACGTACGT" + "\n")
    recs.append(">tab\tsep15\n" + s(60) + "\n")
    for i in range(16, 40):
        recs.append(f">r{i}\n" + s(rnd.randint(20, 150)) + "\n")
    recs.append(">last_no_newline\n" + s(55))
    return "".join(recs).encode()


def edge_fastq() -> bytes:
    rnd = random.Random(7)
    out = []
    for i in range(30):
        L = rnd.randint(10, 120)
        seq = "".join(rnd.choice("ACGTN" if i % 7 == 0 else "ACGT") for _ in range(L))
        hdr = f"@read{i} {1 + (i & 1)}:N:0:ACGT" if i % 3 == 0 else f"@read{i}"
        out.append(f"{hdr}\n{seq}\n+\n{'I' * L}\n")
    return "".join(out).encode()


def prep_fastq() -> bytes:
    """FASTQ for the FASTQ->FASTA prep: Casava comments (1:/2: appended, 3: not,
    names already ending in /1 left alone), tab and multiple separators, lower
    case, N and IUPAC letters, CRLF line ends and a CR inside a line."""
    rnd = random.Random(17)
    heads = ["r0 1:N:0:ACGT", "r1 2:Y:18:ATCACG", "r2/1 2:N:0:ACGT", "r3 3:N:0:ACGT", "r4\t1:N:0:ACGT", "r5",
             "r6  2:N:0", "r7/2", "r8 x 1:N", "r9 1:N:0:ACGT extra words"]
    out = []
    for i in range(40):
        L = rnd.randint(1, 90)
        alpha = "ACGT" if i % 4 else "ACGTNacgtnyrkmYRKMUu"
        seq = "".join(rnd.choice(alpha) for _ in range(L))
        hdr = heads[i % len(heads)].replace("r", "r%d_" % i, 1)
        qual = "".join(rnd.choice("!#5?I@") for _ in range(L))
        if i % 9 == 4:
            out.append(f"@{hdr}\r\n{seq}\r\n+\r\n{qual}\r\n")
        elif i % 13 == 6:
            cut = L // 2
            out.append(f"@{hdr}\n{seq[:cut]}\r{seq[cut:]}\n+{hdr}\n{qual[:cut]}\r{qual[cut:]}\n")
        else:
            out.append(f"@{hdr}\n{seq}\n+\n{qual}\n")
    return "".join(out).encode()


def prep_dirty_fastq() -> bytes:
    """Records fastQ_to_fastA.pl calls poorly formed: quality shorter or longer
    than the sequence, a blank quality line."""
    recs = ["@ok1\nACGTACGT\n+\nIIIIIIII\n", "@short 1:N\nACGTACGT\n+\nIIII\n", "@ok2 2:N\nGGGCCC\n+\nIIIIII\n",
            "@long\nACG\n+\nIIIII\n", "@blank\nACGT\n+\n\n", "@ok3\nTTTT\n+\nIIII\n"]
    return "".join(recs).encode()


def perl(ref: Path, script: str, *args, stdin=None) -> bytes:
    env = dict(os.environ, LC_ALL="C")
    return subprocess.run(["perl", str(ref / script), *map(str, args)], check=True, stdout=subprocess.PIPE,
                          input=stdin, env=env).stdout


def fasta_reader_dump(ref: Path, path: Path) -> bytes:
    code = ("use lib '%s/PerlLib'; use Fasta_reader; my $r = new Fasta_reader($ARGV[0]);"
            " while (my $s = $r->next()) { print $s->get_accession() . \"\\t\" . $s->get_sequence() . \"\\n\"; }"
            % ref)
    return subprocess.run(["perl", "-e", code, str(path)], check=True, stdout=subprocess.PIPE).stdout


def sorted_stats(text: bytes) -> bytes:
    lines = text.split(b"\n")
    head, body = lines[0], [l for l in lines[1:] if l]
    body.sort(key=lambda l: l.split(b"\t", 1)[0])            # sort -k1,1 under LC_ALL=C
    return head + b"\n" + b"".join(l + b"\n" for l in body)


def make_prep(ref: Path) -> None:
    """The FASTQ->FASTA prep fixtures (util/support_scripts/fastQ_to_fastA.pl)."""
    fq = HERE / "prep.fq"
    fq.write_bytes(prep_fastq())
    script = "util/support_scripts/fastQ_to_fastA.pl"
    (HERE / "prep.fa").write_bytes(perl(ref, script, "-I", fq))
    (HERE / "prep.a1.fa").write_bytes(perl(ref, script, "-I", fq, "-a", 1))
    (HERE / "prep.rev.fa").write_bytes(perl(ref, script, "-I", fq, "--rev"))
    (HERE / "prep.a2rev.fa").write_bytes(perl(ref, script, "-I", fq, "-a", 2, "--rev"))
    dq = HERE / "prep_dirty.fq"
    dq.write_bytes(prep_dirty_fastq())
    (HERE / "prep_dirty.ignore.fa").write_bytes(perl(ref, script, "-I", dq, "--ignore_dirty"))


def main() -> None:
    ref = Path(sys.argv[1] if len(sys.argv) > 1 else "/root/reference")
    HERE.mkdir(exist_ok=True)
    if len(sys.argv) > 2 and sys.argv[2] == "--prep-only":
        make_prep(ref)
        return
    make_prep(ref)
    edge = edge_fasta()
    (HERE / "edge.fa").write_bytes(edge)
    bulk = synth.transcriptome_reads(seed=11, n_transcripts=50, n_reads=300, read_len=76).tobytes()
    (HERE / "bulk.fa").write_bytes(bulk)
    for name in ("edge", "bulk"):
        fa = HERE / f"{name}.fa"
        (HERE / f"{name}.fasta_reader.tsv").write_bytes(fasta_reader_dump(ref, fa))
        pk = perl(ref, "util/misc/print_kmers.pl", fa, 25)
        (HERE / f"{name}.print_kmers.txt.gz").write_bytes(gzip.compress(pk, mtime=0))
        kc = perl(ref, "util/misc/kmer_counter.pl", fa, 25, 1)
        kc = b"".join(sorted(l + b"\n" for l in kc.split(b"\n") if l))
        (HERE / f"{name}.kmer_counter.txt.gz").write_bytes(gzip.compress(kc, mtime=0))
    fq = edge_fastq()
    (HERE / "edge.fq").write_bytes(fq)
    (HERE / "edge.fastQ_to_fastA.fa").write_bytes(perl(ref, "util/support_scripts/fastQ_to_fastA.pl", "-I",
                                                       HERE / "edge.fq"))
    # coverage stats through the live Perl consumers
    left, right = synth.gene_pairs(seed=5, n_genes=30, n_pairs=200, fastq=False)
    left, right = left.tobytes(), right.tobytes()
    (HERE / "left.fa").write_bytes(left)
    (HERE / "right.fa").write_bytes(right)
    keys, counts = O.count(left + right, 25, True)
    for side, txt in (("left", left), ("right", right)):
        st = O.cov_stats(txt, keys, counts, 25, True)
        (HERE / f"{side}.stats").write_bytes(sorted_stats(st))
    pairs = perl(ref, "util/support_scripts/nbkc_merge_left_right_stats.pl", "--left", HERE / "left.stats",
                 "--right", HERE / "right.stats", "--sorted")
    (HERE / "pairs.stats").write_bytes(pairs)
    norm = perl(ref, "util/support_scripts/nbkc_normalize.pl", "--stats_file", HERE / "pairs.stats", "--max_cov", 3,
                "--min_cov", 1, "--max_CV", 10000)
    (HERE / "normalized.accs").write_bytes(norm)
    # readsToComponents sort order
    b, r = synth.bundle_reads(seed=6, n_contigs=60, n_components=20, max_per_component=5, n_pairs=150)
    b, r = b.tobytes(), r.tobytes()
    (HERE / "r2t.bundle.fa").write_bytes(b)
    (HERE / "r2t.reads.fa").write_bytes(r)
    rows = O.r2t(r, b, 25, False, 0)
    srt = subprocess.run(["sort", "-k1,1n", "-k3,3nr", "-k2,2"], input=rows, stdout=subprocess.PIPE, check=True,
                         env=dict(os.environ, LC_ALL="C")).stdout
    (HERE / "r2t.out.sort").write_bytes(srt)
    print("fixtures written to", HERE)


if __name__ == "__main__":
    main()
