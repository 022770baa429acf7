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
