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
  norm.left.stats norm.right.stats
                             coverage-stats tables for the normalization tail
                             (duplicates, unpaired reads, odd names, every
                             branch of nbkc_normalize.pl)
  norm.pairs.stats           both sorted by insilico_read_normalization.pl:880's
                             `sort -k1,1`, then nbkc_merge_left_right_stats.pl --sorted
  norm.pairs.c5.accs norm.pairs.c200.accs
                             nbkc_normalize.pl on it (--max_cov 5 --min_cov 2
                             --max_CV 1; --max_cov 200 --min_cov 1 --max_CV 10000)
  norm.left.c5.accs          nbkc_normalize.pl on the sorted left table alone
  norm.left.fq / norm.left.c5.fq
                             FASTQ reads and the records make_normalized_reads_file
                             keeps for norm.pairs.c5.accs, read by
                             PerlLib/Fastq_reader.pm
  norm.left.fa / norm.left.c5.fa
                             the same for FASTA input, read by PerlLib/Fasta_reader.pm,
                             for norm.pairs.c5.fa.accs (without the one name with a
                             byte Fasta_reader deletes)
  r2t.bundle.fa r2t.reads.fa small bundle and reads
  r2t.out.sort               the oracle's readsToComponents rows through
                             `sort -k1,1n -k3,3nr -k2,2` under LC_ALL=C (Trinity:2258)
  r2t.bundle.deBruijn.gz     the oracle's FastaToDeBruijn --graph_per_record -K 24
                             text of r2t.bundle.fa (decision D8)
  r2t.bundle.deBruijn.partitions
                             what util/support_scripts/partition_chrysalis_graphs_n_reads.pl
                             (-N 1000 -L 100) makes of that text and r2t.out.sort:
                             per listed component, its id and the line counts of
                             the graph and reads files it wrote
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


def norm_tables():
    """Two coverage-stats tables (as fastaToKmerCoverageStats prints them,
    unsorted) for the normalization tail: mates named <core>/1 and <core>/2,
    unpaired reads on either side, a left name twice, names whose core ends
    in /1, /3 endings, no ending, an empty name, "_forward"/"_reverse" names,
    punctuation and a high byte around '/', and values that reach every
    branch of nbkc_normalize.pl (median 0, mean 0, stdev/mean > 1, "%.1f"
    ties, exponent forms of "%g").  Every value has at most 6 significant
    digits, so float32 carries it exactly to "%g"."""
    rnd = random.Random(4242)

    def val(kind):
        if kind == 0:
            return "0"
        if kind == 1:
            return "%g" % (rnd.randint(1, 400) / 4)                 # quarter steps: "%.1f" ties
        if kind == 2:
            return "%g" % float("%.6g" % rnd.uniform(0.001, 60))
        if kind == 3:
            return "%g" % float("%.6g" % rnd.uniform(1e5, 5e7))     # 1.23457e+06 forms
        return "%g" % float("%.6g" % rnd.uniform(1e-6, 1e-4))        # 1.5e-05 forms

    def row(name):
        med = rnd.choice([0, 1, 2, 2, 3, 4, 5, 7, 9, 12, 40, 300])
        mean = val(rnd.choice([0, 1, 1, 2, 2, 2, 3, 4]) if rnd.random() < 0.15 else rnd.choice([1, 2]))
        sd = val(rnd.choice([0, 1, 2, 2, 3, 4]))
        return f"{name}\t{med}\t{mean}\t{sd}\n"

    cores = [f"r{i:04d}" for i in range(150)]
    cores += ["a.b", "a", "a-x", "a0", "x/1", "y/1/2", "r_forward", "s_reverse", "t_forward_x_reverse", "z\xc3z",
              "P", "p", "u/3", "v/a", "w_"]
    left, right = [], []
    for c in cores:
        p = rnd.random()
        if c in ("x/1", "y/1/2"):
            left.append(c + "/1"); right.append(c + "/2")
        elif c == "u/3":
            left.append("u/3"); right.append("u/3")
        elif p < 0.75:
            left.append(c + "/1"); right.append(c + "/2")
        elif p < 0.83:
            left.append(c + "/1")
        elif p < 0.91:
            right.append(c + "/2")
        else:
            left.append(c); right.append(c + "/" + rnd.choice("123"))
    left.append("r0007/1")            # a name twice
    left.append(""); right.append("")  # empty names
    rnd.shuffle(left)
    rnd.shuffle(right)
    head = "acc\tmedian_cov\tmean_cov\tstdev\n"
    lt = (head + "".join(row(n) for n in left)).encode("latin-1")
    rt = (head + "".join(row(n) for n in right)).encode("latin-1")
    return lt, rt


def norm_fastq(names, seed):
    """FASTQ records for the extraction: each name once (headers as Trinity's
    inputs carry them: "@core/1", "@core 1:N:0:ACGT", "@core_forward/1"),
    and some reads no selection names."""
    rnd = random.Random(seed)
    out = []
    for i, n in enumerate(names):
        L = rnd.randint(5, 40)
        seq = "".join(rnd.choice("ACGT") for _ in range(L))
        qual = "".join(rnd.choice("!#5?I") for _ in range(L))
        out.append(f"@{n}\n{seq}\n+\n{qual}\n")
    return "".join(out).encode("latin-1")


def norm_fasta(names, seed):
    """FASTA records for the extraction from FASTA input: comments after a
    space or tab, CRLF records, a control byte in a comment, multi-line and
    lower-case sequences with a space and a tab inside, a blank line first."""
    rnd = random.Random(seed)
    out = ["\n"]
    for i, n in enumerate(names):
        L = rnd.randint(5, 70)
        seq = "".join(rnd.choice("ACGTacgtN") for _ in range(L))
        lines = [seq[j:j + 25] for j in range(0, L, 25)]
        if i % 6 == 5:
            lines[0] = lines[0][:3] + " " + lines[0][3:] + "\t"
        kind = i % 4
        if kind == 0:
            out.append(f">{n} some comment\tmore\n" + "".join(l + "\n" for l in lines))
        elif kind == 1:
            out.append(f">{n}\r\n" + "".join(l + "\r\n" for l in lines))
        elif kind == 2:
            out.append(f">{n}\n" + "".join(l + "\n" for l in lines))
        else:
            out.append(f">{n} \x01ctl\n" + "".join(l + "\n" for l in lines))
    return "".join(out).encode("latin-1")


def sort_stats_file(path: Path, out: Path) -> None:
    """insilico_read_normalization.pl:880's command, run as it runs it."""
    subprocess.run(f"head -n1 '{path}' > '{out}' && tail -n +2 '{path}' | sort -k1,1 >> '{out}'", shell=True,
                   check=True, env=dict(os.environ, LC_ALL="C"))


def extract_perl(ref: Path, fq: Path, accs: Path) -> bytes:
    """make_normalized_reads_file (insilico:452-466, 505-545) on one FASTQ:
    the records are read by the reference's PerlLib/Fastq_reader.pm."""
    code = (r"use lib '%s/PerlLib'; use Fastq_reader; my %%idx;"
            r" open(my $f, $ARGV[1]) or die; while (my $l = <$f>) { chomp $l; next unless $l =~ /\S/;"
            r" $l =~ s|/\w$||; $idx{$l} = 0; } close $f;"
            r" my $r = new Fastq_reader($ARGV[0]); while (my $s = $r->next()) { my $a = $s->get_core_read_name();"
            r" $a =~ s/_forward//; $a =~ s/_reverse//; if (exists $idx{$a}) { $idx{$a}++;"
            r" print $s->get_fastq_record(); } }"
            r' my @m = grep { !$idx{$_} } keys %%idx; die "missing @m" if @m;' % ref)
    return subprocess.run(["perl", "-e", code, str(fq), str(accs)], check=True, stdout=subprocess.PIPE).stdout


def extract_perl_fasta(ref: Path, fa: Path, accs: Path) -> bytes:
    """make_normalized_reads_file for --seqType fa (insilico:518-545): records
    read by the reference's PerlLib/Fasta_reader.pm."""
    code = (r"use lib '%s/PerlLib'; use Fasta_reader; my %%idx;"
            r" open(my $f, $ARGV[1]) or die; while (my $l = <$f>) { chomp $l; next unless $l =~ /\S/;"
            r" $l =~ s|/\w$||; $idx{$l} = 0; } close $f;"
            r" my $r = new Fasta_reader($ARGV[0]); while (my $s = $r->next()) { my $a = $s->get_accession();"
            r" $a =~ s|/[12]\s*$||; if (exists $idx{$a}) { $idx{$a}++;"
            r" print $s->get_FASTA_format(fasta_line_len => -1); } }"
            r' my @m = grep { !$idx{$_} } keys %%idx; die "missing @m" if @m;' % ref)
    return subprocess.run(["perl", "-e", code, str(fa), str(accs)], check=True, stdout=subprocess.PIPE).stdout


def make_norm(ref: Path) -> None:
    """The normalization-tail fixtures (insilico_read_normalization.pl:865-985,
    470-584) from the reference's own scripts."""
    lt, rt = norm_tables()
    lp, rp = HERE / "norm.left.stats", HERE / "norm.right.stats"
    lp.write_bytes(lt)
    rp.write_bytes(rt)
    ls, rs = HERE / "_norm.left.sort", HERE / "_norm.right.sort"
    sort_stats_file(lp, ls)
    sort_stats_file(rp, rs)
    pairs = perl(ref, "util/support_scripts/nbkc_merge_left_right_stats.pl", "--left", ls, "--right", rs, "--sorted")
    (HERE / "norm.pairs.stats").write_bytes(pairs)
    pp = HERE / "norm.pairs.stats"
    for tag, args in (("c5", (5, 2, 1)), ("c200", (200, 1, 10000))):
        acc = perl(ref, "util/support_scripts/nbkc_normalize.pl", "--stats_file", pp, "--max_cov", args[0],
                   "--min_cov", args[1], "--max_CV", args[2])
        (HERE / f"norm.pairs.{tag}.accs").write_bytes(acc)
    single = perl(ref, "util/support_scripts/nbkc_normalize.pl", "--stats_file", ls, "--max_cov", 5, "--min_cov", 2,
                  "--max_CV", 1)
    (HERE / "norm.left.c5.accs").write_bytes(single)
    # extraction: FASTQ headers for every left read (named as the reads were
    # before the FASTQ->FASTA prep added /1), plus reads nothing selects
    lnames = [l.split(b"\t", 1)[0].decode("latin-1") for l in lt.split(b"\n")[1:] if l]
    heads = []
    for i, n in enumerate(sorted(set(lnames))):
        core = n[:-2] if len(n) >= 3 and n[-2] == "/" and n[-1] in "12" else n
        if not core or core != core.strip():
            continue
        if i % 5 == 1 and not core.endswith(("/1", "/2")):
            heads.append(f"{core} 1:N:0:ACGT")
        else:
            heads.append(f"{core}/1")
    # reads nothing selects; and "x", "y" (the accs of x/1/1 and y/1/2/1,
    # whose own records have the core names x/1 and y/1/2) carried by reads of
    # their own, without which the script dies ("not all specified records
    # have been retrieved")
    heads += ["extra1/1", "extra2/1 1:N:0", "x/2", "y 2:N:0"]
    fq = HERE / "norm.left.fq"
    fq.write_bytes(norm_fastq(heads, 99))
    (HERE / "norm.left.c5.fq").write_bytes(extract_perl(ref, fq, HERE / "norm.pairs.c5.accs"))
    # the same from FASTA input (names as the stats carry them, "x" and "y"
    # again from reads of their own)
    fnames = [n for n in sorted(set(lnames)) if n] + ["extra9/1", "x/2", "y"]
    fa = HERE / "norm.left.fa"
    fa.write_bytes(norm_fasta(fnames, 98))
    # Fasta_reader deletes bytes 0x7F-0xFF, so no FASTA record can carry the
    # name z\xc3z (the script dies on it): the FASTA case selects the rest
    sel = HERE / "norm.pairs.c5.fa.accs"
    sel.write_bytes(b"".join(l + b"\n" for l in (HERE / "norm.pairs.c5.accs").read_bytes().split(b"\n")
                             if l and l != b"z\xc3z"))
    (HERE / "norm.left.c5.fa").write_bytes(extract_perl_fasta(ref, fa, sel))
    ls.unlink()
    rs.unlink()


def make_debruijn(ref: Path) -> None:
    """The de Bruijn text of the small bundle, and the reference's partition
    script run on it (Trinity:2319-2323)."""
    import shutil
    import tempfile
    text = O.debruijn((HERE / "r2t.bundle.fa").read_bytes(), 24, False)
    (HERE / "r2t.bundle.deBruijn.gz").write_bytes(gzip.compress(text, mtime=0))
    with tempfile.TemporaryDirectory() as tmp:
        t = Path(tmp)
        (t / "bundle.deBruijn").write_bytes(text)
        shutil.copy(HERE / "r2t.out.sort", t / "readsToComponents.out.sort")
        perl(ref, "util/support_scripts/partition_chrysalis_graphs_n_reads.pl", "--deBruijns",
             t / "bundle.deBruijn", "--componentReads", t / "readsToComponents.out.sort", "-N", 1000, "-L", 100)
        rows = []
        for line in (t / "component_base_listing.txt").read_text().splitlines():
            comp, base = line.split("\t")
            g = Path(base + ".graph.tmp").read_bytes().count(b"\n")
            r = Path(base + ".reads.tmp").read_bytes().count(b"\n")
            rows.append(f"{comp}\t{g}\t{r}\n")
        (HERE / "r2t.bundle.deBruijn.partitions").write_text("".join(rows))


def main() -> None:
    if len(sys.argv) < 2:
        sys.exit(__doc__)
    ref = Path(sys.argv[1])
    HERE.mkdir(exist_ok=True)
    if len(sys.argv) > 2 and sys.argv[2] == "--debruijn-only":
        make_debruijn(ref)
        return
    if len(sys.argv) > 2 and sys.argv[2] == "--prep-only":
        make_prep(ref)
        return
    if len(sys.argv) > 2 and sys.argv[2] == "--norm-only":
        make_norm(ref)
        return
    make_prep(ref)
    make_norm(ref)
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
    make_debruijn(ref)
    print("fixtures written to", HERE)


if __name__ == "__main__":
    main()
