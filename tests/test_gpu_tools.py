"""The drop-in executables, run with the command lines Trinity uses, produce
the files the reference's consumers read: the jellyfish dump/histo of
Trinity:2612-2638 and util/insilico_read_normalization.pl:617-643, the
coverage-stats table of util/insilico_read_normalization.pl:837-846 and the
readsToComponents file of Trinity:2237-2251."""
import os
import subprocess

import numpy as np
import pytest

from trinityrnaseq_gb300.build import BIN
from trinityrnaseq_gb300.kmer import format_histo
from tests.helpers import sort_stats, trinity_r2t_sort

pytestmark = pytest.mark.gpu


def run(args, cwd, stdout=None):
    r = subprocess.run([str(a) for a in args], cwd=cwd, stdout=stdout or subprocess.PIPE, stderr=subprocess.PIPE)
    assert r.returncode == 0, r.stderr.decode()
    return r.stdout


def sorted_records(dump: bytes):
    lines = dump.split(b"\n")
    recs = list(zip(lines[0::2], lines[1::2]))
    return sorted(r for r in recs if r[0])


def test_jellyfish_version(native_built):
    out = run([BIN / "jellyfish", "--version"], cwd=None)
    assert out.split()[1].startswith(b"2.")


def test_jellyfish_count_histo_dump(native_built, oracle, golden, tmp_path):
    both = tmp_path / "both.fa"
    both.write_bytes((golden / "left.fa").read_bytes() + (golden / "right.fa").read_bytes() +
                     (golden / "bulk.fa").read_bytes())
    jf = BIN / "jellyfish"
    run([jf, "count", "-t", 4, "-m", 25, "-s", 100000000, "--canonical", both], cwd=tmp_path)
    assert (tmp_path / "mer_counts.jf").exists()
    run([jf, "histo", "-t", 4, "-o", "kmers.histo", "mer_counts.jf"], cwd=tmp_path)
    with open(tmp_path / "kmers.fa", "wb") as fh:
        run([jf, "dump", "-L", 2, "mer_counts.jf"], cwd=tmp_path, stdout=fh)
    keys, counts = oracle.count(both.read_bytes(), 25, True)
    want_dump = oracle.dump(keys, counts, 25, 2)
    got = (tmp_path / "kmers.fa").read_bytes()
    assert sorted_records(got) == sorted_records(want_dump)
    assert got == want_dump          # both are in key order
    assert (tmp_path / "kmers.histo").read_bytes() == format_histo(oracle.histo(counts, 1, 10000), 1, 10000)
    # -o names the database; a second count with a custom path
    run([jf, "count", "-m", 25, "-s", "1G", "-C", "-o", "db2.jf", both], cwd=tmp_path)
    with open(tmp_path / "all.fa", "wb") as fh:
        run([jf, "dump", "-L", 1, "db2.jf"], cwd=tmp_path, stdout=fh)
    assert (tmp_path / "all.fa").read_bytes() == oracle.dump(keys, counts, 25, 1)
    # several input files (and an empty one) are counted as their concatenation
    parts = [golden / "left.fa", golden / "right.fa", tmp_path / "empty.fa", golden / "bulk.fa"]
    (tmp_path / "empty.fa").write_bytes(b"")
    run([jf, "count", "-m", 25, "-s", "1G", "-C", "-o", "db3.jf", *parts], cwd=tmp_path)
    with open(tmp_path / "multi.fa", "wb") as fh:
        run([jf, "dump", "-L", 1, "db3.jf"], cwd=tmp_path, stdout=fh)
    assert (tmp_path / "multi.fa").read_bytes() == oracle.dump(keys, counts, 25, 1)


def test_fastaToKmerCoverageStats(native_built, oracle, golden, tmp_path):
    left = (golden / "left.fa").read_bytes()
    right = (golden / "right.fa").read_bytes()
    keys, counts = oracle.count(left + right, 25, True)
    (tmp_path / "kmers.fa").write_bytes(oracle.dump(keys, counts, 25, 2))   # the -L 2 catalogue
    for side in ("left", "right"):
        (tmp_path / f"{side}.fa").write_bytes((golden / f"{side}.fa").read_bytes())
        with open(tmp_path / f"{side}.stats", "wb") as fh:
            run([BIN / "fastaToKmerCoverageStats", "--reads", f"{side}.fa", "--kmers", "kmers.fa", "--kmer_size", 25,
                 "--num_threads", 2, "--DS"], cwd=tmp_path, stdout=fh)
        got = (tmp_path / f"{side}.stats").read_bytes()
        assert sort_stats(got) == (golden / f"{side}.stats").read_bytes()


def test_fastaToKmerCoverageStats_kmers_from_reads(native_built, oracle, golden, tmp_path):
    (tmp_path / "r.fa").write_bytes((golden / "bulk.fa").read_bytes())
    out = run([BIN / "fastaToKmerCoverageStats", "--kmers_from_reads", "r.fa", "--reads", "r.fa", "--num_threads", 1],
              cwd=tmp_path)
    text = (golden / "bulk.fa").read_bytes()
    keys, counts = oracle.count(text, 25, False)
    assert out == oracle.cov_stats(text, keys, counts, 25, False)


@pytest.mark.parametrize("chunk", [50000000, 37])
def test_ReadsToTranscripts(native_built, oracle, golden, tmp_path, chunk):
    (tmp_path / "bundle.fa").write_bytes((golden / "r2t.bundle.fa").read_bytes())
    (tmp_path / "both.fa").write_bytes((golden / "r2t.reads.fa").read_bytes())
    run([BIN / "ReadsToTranscripts", "-i", "both.fa", "-f", "bundle.fa", "-o", "readsToComponents.out", "-t", 4,
         "-max_mem_reads", chunk], cwd=tmp_path)
    got = (tmp_path / "readsToComponents.out").read_bytes()
    assert trinity_r2t_sort(got) == (golden / "r2t.out.sort").read_bytes()
    assert not [p for p in os.listdir(tmp_path) if ".tmp." in p]
    run([BIN / "ReadsToTranscripts", "-i", "both.fa", "-f", "bundle.fa", "-o", "p50.out", "-p", 50, "-strand"],
        cwd=tmp_path)
    b = (golden / "r2t.bundle.fa").read_bytes()
    r = (golden / "r2t.reads.fa").read_bytes()
    assert (tmp_path / "p50.out").read_bytes() == oracle.r2t(r, b, 25, True, 50)


def test_tools_fail_loudly_on_bad_input(native_built, tmp_path):
    (tmp_path / "bad.fq").write_bytes(b"@r1\nACGT\n+\nIIII\n@r2\nACGT\n")
    r = subprocess.run([str(BIN / "jellyfish"), "count", "-m", "25", "-s", "1M", "bad.fq"], cwd=tmp_path,
                       stdout=subprocess.PIPE, stderr=subprocess.PIPE)
    assert r.returncode != 0 and b"Error" in r.stderr
    assert not (tmp_path / "mer_counts.jf").exists()


def _shuffled(text: bytes, seed: int, drop: float) -> bytes:
    import random
    recs = text.split(b"\n")
    recs = [b"\n".join(recs[i:i + 4]) + b"\n" for i in range(0, len(recs) - 1, 4)]
    rnd = random.Random(seed)
    rnd.shuffle(recs)
    return b"".join(r for r in recs if rnd.random() >= drop)


def _oracle_normalize(oracle, sides, ss, pairs_together, max_cov, min_cov, max_cv, fasta=False):
    """The script's own sequence of steps, each through the oracle:
    seqtk-trinity (FASTQ), jellyfish count (+ dump -L 2),
    fastaToKmerCoverageStats, sort / merge / nbkc_normalize.pl,
    make_normalized_reads_file."""
    fas = []
    for i, (tag, fq) in enumerate(sides):
        letter = ss[i] if i < len(ss) else ""
        flags = oracle.FA_IF_MISSING | (oracle.FA_REV if letter == "R" else 0)
        fas.append(fq if fasta else oracle.fastq_to_fasta(fq, 2 if tag == "right" else 1, flags))
    canonical = not ss
    keys, counts = oracle.count(b"".join(fas), 25, canonical)
    d2 = oracle.dump(keys, counts, 25, 2)
    k2, c2 = oracle.load_dump(d2, 25, canonical)
    stats = [oracle.cov_stats(fa, k2, c2, 25, canonical) for fa in fas]
    if pairs_together:
        _, accs, _ = oracle.norm(stats[0], stats[1], max_cov, min_cov, max_cv)
        return [oracle.norm_extract(fq, accs) for _, fq in sides]
    out = []
    for (tag, fq), st in zip(sides, stats):
        _, accs, _ = oracle.norm(st, None, max_cov, min_cov, max_cv)
        out.append(oracle.norm_extract(fq, accs))
    return out


@pytest.mark.parametrize("ss,pairs_together,single", [("", True, False), ("RF", True, False), ("", False, False),
                                                      ("", False, True)])
def test_insilico_read_normalization(native_built, oracle, tmp_path, ss, pairs_together, single):
    """bin/insilico_read_normalization with Trinity's command line
    (Trinity:3426-3448) writes the normalized FASTQ the script's steps write."""
    from trinityrnaseq_gb300 import synth
    left, right = synth.gene_pairs(seed=71, n_genes=60, n_pairs=6000, fastq=True)
    lfq, rfq = _shuffled(left.tobytes(), 1, 0.03), _shuffled(right.tobytes(), 2, 0.03)
    (tmp_path / "reads_2.fq").write_bytes(rfq)
    # the left reads in two files, cut at a record boundary
    recs = lfq.split(b"\n")
    cut = (len(recs) // 8) * 4
    (tmp_path / "reads_1.fq").write_bytes(b"\n".join(recs[:cut]) + b"\n")
    (tmp_path / "reads_1b.fq").write_bytes(b"\n".join(recs[cut:]))
    out = tmp_path / "norm"
    args = [BIN / "insilico_read_normalization", "--seqType", "fq", "--JM", "4G", "--max_cov", 30, "--min_cov", 1,
            "--CPU", 4, "--output", out, "--max_CV", 10000]
    if ss:
        args += ["--SS_lib_type", ss]
    if single:
        args += ["--single", "reads_1.fq,reads_1b.fq"]
        sides = [("single", lfq)]
    else:
        args += ["--left", "reads_1.fq,reads_1b.fq", "--right", "reads_2.fq"]
        if pairs_together:
            args += ["--pairs_together", "--PARALLEL_STATS"]
        sides = [("left", lfq), ("right", rfq)]
    r = subprocess.run([str(a) for a in args], cwd=tmp_path, stdout=subprocess.PIPE, stderr=subprocess.PIPE)
    assert r.returncode == 0, r.stderr.decode()
    assert b"reads selected during normalization" in r.stderr
    want = _oracle_normalize(oracle, sides, ss, pairs_together, 30, 1, 10000)
    for (tag, _), w in zip(sides, want):
        got = (out / f"{tag}.norm.fq").read_bytes()
        assert got == w, tag
        assert os.path.islink(out / f"{tag}.norm.fq")
    assert (out / "reads_1.fq_ext_all_reads.normalized_K25_maxC30_minC1_maxCV10000.fq").exists()


def _shuffled_fasta(text: bytes, seed: int, drop: float) -> bytes:
    import random
    recs = [b">" + r for r in text.split(b">")[1:]]
    rnd = random.Random(seed)
    rnd.shuffle(recs)
    return b"".join(r for r in recs if rnd.random() >= drop)


@pytest.mark.parametrize("pairs_together", [True, False])
def test_insilico_read_normalization_fasta(native_built, oracle, tmp_path, pairs_together):
    """--seqType fa: FASTA counted as it is, records extracted with
    PerlLib/Fasta_reader.pm's rules; outputs left.norm.fa / right.norm.fa."""
    from trinityrnaseq_gb300 import synth
    left, right = synth.gene_pairs(seed=72, n_genes=60, n_pairs=6000, fastq=False)
    lfa, rfa = _shuffled_fasta(left.tobytes(), 3, 0.03), _shuffled_fasta(right.tobytes(), 4, 0.03)
    (tmp_path / "l.fa").write_bytes(lfa)
    (tmp_path / "r.fa").write_bytes(rfa)
    out = tmp_path / "norm"
    args = [BIN / "insilico_read_normalization", "--seqType", "fa", "--JM", "4G", "--max_cov", 30, "--min_cov", 1,
            "--CPU", 4, "--output", out, "--max_CV", 10000, "--left", "l.fa", "--right", "r.fa"]
    if pairs_together:
        args.append("--pairs_together")
    r = subprocess.run([str(a) for a in args], cwd=tmp_path, stdout=subprocess.PIPE, stderr=subprocess.PIPE)
    assert r.returncode == 0, r.stderr.decode()
    sides = [("left", lfa), ("right", rfa)]
    want = _oracle_normalize(oracle, sides, "", pairs_together, 30, 1, 10000, fasta=True)
    for (tag, _), w in zip(sides, want):
        assert (out / f"{tag}.norm.fa").read_bytes() == w, tag
    assert (out / "l.fa.normalized_K25_maxC30_minC1_maxCV10000.fa").exists()


def test_trinkmer_bins_writes_each_bins_catalogue(native_built, oracle, tmp_path):
    """Phase 2's per-bin k-mer catalogues (what `inchworm --reads ...
    --minKmerCount 2 --DS` builds in each bin's Trinity run) from one batched
    pass over the reads list file that write_partitioned_trinity_cmds.pl reads
    (the last field of each line is a bin's reads file)."""
    from trinityrnaseq_gb300 import synth
    text, off, _ = synth.power_law_bins(seed=9, n_bins=25, alpha=1.8, min_reads=50, max_reads=3000)
    t = text.tobytes()
    paths = []
    for b in range(25):
        p = tmp_path / f"c{b}.trinity.reads.fa"
        p.write_bytes(t[int(off[b]):int(off[b + 1])])
        paths.append(p)
    (tmp_path / "partitioned_reads.files.list").write_text(
        "".join(f"bin{b}\t{p}\n" if b % 2 else f"{p}\n" for b, p in enumerate(paths)))
    run([BIN / "trinkmer_bins", "--reads_list_file", tmp_path / "partitioned_reads.files.list", "-K", 25,
         "--min_kmer_cov", 2, "--histo", "--max_batch_gb", 0.0001], cwd=tmp_path)
    for p in paths:
        keys, counts = oracle.count(p.read_bytes(), 25, True)
        assert (tmp_path / (p.name + ".K25.kmers.fa")).read_bytes() == oracle.dump(keys, counts, 25, 2)
        h = oracle.histo(counts, 1, 10000)
        want = "".join(f"{c} {h[c]}\n" for c in range(1, 10002) if h[c])
        assert (tmp_path / (p.name + ".K25.histo")).read_text() == want


def test_unchanged_perl_normalization_over_the_drop_ins(native_built, tmp_path):
    """util/insilico_read_normalization.pl as shipped, with bin/jellyfish and
    bin/seqtk-trinity found first on PATH and bin/fastaToKmerCoverageStats as
    $TRINITY_HOME/Inchworm/bin/fastaToKmerCoverageStats, selects the same
    reads as bin/insilico_read_normalization.  Needs a reference checkout
    (TRINITY_REFERENCE_HOME) and Perl with DB_File; skipped otherwise.  The
    script is copied into a scratch tree under tmp_path whose PerlLib and
    util/support_scripts point at the reference's, so that its
    $FindBin::RealBin/.. is the scratch tree holding the drop-ins."""
    import shutil
    from pathlib import Path
    from trinityrnaseq_gb300 import synth
    ref = os.environ.get("TRINITY_REFERENCE_HOME")
    if not ref or not Path(ref, "util", "insilico_read_normalization.pl").exists():
        pytest.skip("no reference checkout named by TRINITY_REFERENCE_HOME")
    if not shutil.which("perl") or subprocess.run(["perl", "-MDB_File", "-Mthreads", "-e", "1"]).returncode:
        pytest.skip("perl with DB_File and threads is required")
    home = tmp_path / "trinity"
    (home / "util").mkdir(parents=True)
    (home / "Inchworm" / "bin").mkdir(parents=True)
    (home / "trinity-plugins" / "BIN").mkdir(parents=True)
    shutil.copy(Path(ref, "util", "insilico_read_normalization.pl"), home / "util")
    os.symlink(Path(ref, "util", "support_scripts"), home / "util" / "support_scripts")
    os.symlink(Path(ref, "PerlLib"), home / "PerlLib")
    os.symlink(BIN / "fastaToKmerCoverageStats", home / "Inchworm" / "bin" / "fastaToKmerCoverageStats")
    os.symlink(BIN / "seqtk-trinity", home / "trinity-plugins" / "BIN" / "seqtk-trinity")
    left, right = synth.gene_pairs(seed=73, n_genes=80, n_pairs=8000, fastq=True)
    (tmp_path / "l.fq").write_bytes(left.tobytes())
    (tmp_path / "r.fq").write_bytes(right.tobytes())
    common = ["--seqType", "fq", "--JM", "2G", "--max_cov", 30, "--min_cov", 1, "--max_CV", 10000, "--CPU", 4,
              "--left", "l.fq", "--right", "r.fq", "--pairs_together", "--PARALLEL_STATS"]
    env = dict(os.environ, PATH=f"{BIN}:{os.environ.get('PATH', '')}")
    r = subprocess.run(["perl", str(home / "util" / "insilico_read_normalization.pl"), *map(str, common),
                        "--output", "perl_out"], cwd=tmp_path, env=env, stdout=subprocess.PIPE, stderr=subprocess.PIPE)
    assert r.returncode == 0, r.stderr.decode()[-2000:]
    run([BIN / "insilico_read_normalization", *common, "--output", "gpu_out"], cwd=tmp_path)
    for tag in ("left", "right"):
        assert (tmp_path / "perl_out" / f"{tag}.norm.fq").read_bytes() == \
            (tmp_path / "gpu_out" / f"{tag}.norm.fq").read_bytes(), tag
