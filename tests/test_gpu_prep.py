"""FASTQ -> FASTA read prep on the GPU (tk_reads_to_fasta, bin/seqtk-trinity)
against util/support_scripts/fastQ_to_fastA.pl's own output (golden fixtures)
and the oracle's restatement of it, byte for byte."""
import subprocess

import pytest

from trinityrnaseq_gb300 import ReadSet, native, synth
from trinityrnaseq_gb300.build import BIN

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("fixture,append,rev", [
    ("prep.fa", -1, False), ("prep.a1.fa", 1, False), ("prep.rev.fa", -1, True), ("prep.a2rev.fa", 2, True)])
def test_prep_matches_reference_script(ctx, golden, fixture, append, rev):
    rs = ReadSet(ctx, (golden / "prep.fq").read_bytes())
    assert rs.to_fasta(append, revcomp=rev) == (golden / fixture).read_bytes()


def test_prep_edge_fastq(ctx, golden):
    rs = ReadSet(ctx, (golden / "edge.fq").read_bytes())
    assert rs.to_fasta() == (golden / "edge.fastQ_to_fastA.fa").read_bytes()


def test_prep_dirty_records(ctx, golden):
    rs = ReadSet(ctx, (golden / "prep_dirty.fq").read_bytes())
    assert rs.to_fasta(ignore_dirty=True) == (golden / "prep_dirty.ignore.fa").read_bytes()
    with pytest.raises(native.TrinkmerError) as e:
        rs.to_fasta()
    assert e.value.status == native.TK_E_PARSE


@pytest.mark.parametrize("append,rev,if_missing", [(1, False, True), (2, True, True), (-1, True, False), (7, False, False)])
def test_prep_parity_200k_pairs(ctx, oracle, append, rev, if_missing):
    left, _ = synth.gene_pairs(seed=51, n_genes=500, n_pairs=200000, fastq=True)
    text = left.tobytes()
    flags = (oracle.FA_REV if rev else 0) | (oracle.FA_IF_MISSING if if_missing else 0)
    want = oracle.fastq_to_fasta(text, append, flags)
    assert ReadSet(ctx, text).to_fasta(append, revcomp=rev, if_missing=if_missing) == want


def test_prep_rejects_fasta_input(ctx, golden):
    rs = ReadSet(ctx, (golden / "edge.fa").read_bytes())
    with pytest.raises(native.TrinkmerError) as e:
        rs.to_fasta()
    assert e.value.status == native.TK_E_INVAL


def test_seqtk_trinity_cli(native_built, oracle, golden, tmp_path):
    """The command line Trinity runs: `cat f.fq | seqtk-trinity seq -A -R 2 [-r] -`."""
    fq = (golden / "prep.fq").read_bytes()
    for args, flags in ((["-R", "2"], oracle.FA_IF_MISSING), (["-R", "1", "-r"], oracle.FA_IF_MISSING | oracle.FA_REV)):
        p = subprocess.run([str(BIN / "seqtk-trinity"), "seq", "-A", *args, "-"], input=fq, capture_output=True,
                           timeout=300)
        assert p.returncode == 0, p.stderr
        assert p.stdout == oracle.fastq_to_fasta(fq, int(args[1]), flags)
    bad = subprocess.run([str(BIN / "seqtk-trinity"), "seq", "-A", str(golden / "prep_dirty.fq")], capture_output=True,
                         timeout=300)
    assert bad.returncode != 0 and b"improperly formatted" in bad.stderr
