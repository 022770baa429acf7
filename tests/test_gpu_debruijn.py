"""GPU parity of the per-record de Bruijn graphs (Inchworm FastaToDeBruijn
--graph_per_record, Trinity:2298-2302) with the oracle's restatement, byte
for byte, through the C ABI and the drop-in executable."""
import gzip
import subprocess

import numpy as np
import pytest

from trinityrnaseq_gb300 import DeBruijnGraphs, synth

pytestmark = pytest.mark.gpu


def gpu_text(ctx, bundle, K=24, ss=False):
    g = DeBruijnGraphs(ctx, bundle, K, ss)
    t = g.text()
    assert t.count(b"Component ") == g.n_components
    assert t.count(b"\n") == g.n_components + g.n_nodes
    g.free()
    return t


@pytest.mark.parametrize("ss", [False, True])
def test_golden_bundle(ctx, oracle, golden, ss):
    b = (golden / "r2t.bundle.fa").read_bytes()
    got = gpu_text(ctx, b, 24, ss)
    assert got == oracle.debruijn(b, 24, ss)
    if not ss:
        assert got == gzip.decompress((golden / "r2t.bundle.deBruijn.gz").read_bytes())


@pytest.mark.parametrize("K", [1, 4, 15, 16, 24, 30])
def test_every_k(ctx, oracle, K):
    b, _ = synth.bundle_reads(seed=40 + K, n_contigs=300, n_components=90, max_per_component=6, n_pairs=10)
    b = b.tobytes()
    for ss in (False, True):
        assert gpu_text(ctx, b, K, ss) == oracle.debruijn(b, K, ss)


def test_edge_records(ctx, oracle, golden):
    """'X' joins, N and other bytes, lower case, records without a window
    (left out), repeats inside a record, palindromic windows (even K+1),
    multi-line records, headers without s_."""
    rnd = np.random.default_rng(3)
    rep = rnd.choice(np.frombuffer(b"ACGT", dtype=np.uint8), 40).tobytes()
    recs = [b">s_9\nACGTACGTAAXCCC\n", b">s_10\nAC\n", b">noid\nacgtNacgtaGGGGGGG\n",
            b">s_3\n" + rep + b"X" + rep + b"X" + rep[::-1] + b"\n", b">s_4\nACGTACGTACGTACGT\nAACCGGTT\n",
            b">s_77 extra words\n" + b"N" * 30 + b"\n", b">s_12\n" + b"A" * 60 + b"\n"]
    b = b"".join(recs) + (golden / "edge.fa").read_bytes()
    for K in (3, 7, 24):
        for ss in (False, True):
            assert gpu_text(ctx, b, K, ss) == oracle.debruijn(b, K, ss), (K, ss)


def test_empty_inputs(ctx, oracle):
    for b in (b"", b">s_1\n\n", b">s_1\nACGT\n>s_2\nNNNNNNNNNNNNNNNNNNNNNNNNNNNNNN\n"):
        assert gpu_text(ctx, b, 24) == oracle.debruijn(b, 24, False) == b""


def test_large_bundle(ctx, oracle):
    """30,000 components (more records than fit in the bits a packed
    record+k-mer key would leave)."""
    b, _ = synth.bundle_reads(seed=77, n_contigs=40000, n_components=30000, max_per_component=4, n_pairs=10)
    b = b.tobytes()
    assert gpu_text(ctx, b, 24) == oracle.debruijn(b, 24, False)


def test_tool_writes_the_graphs(native_built, oracle, golden, tmp_path):
    exe = native_built["tools"]["FastaToDeBruijn"]
    b = golden / "r2t.bundle.fa"
    out = subprocess.run([str(exe), "--fasta", str(b), "-K", "24", "--graph_per_record", "--threads", "4"],
                         stdout=subprocess.PIPE, check=True).stdout
    assert out == oracle.debruijn(b.read_bytes(), 24, False)
    ss = subprocess.run([str(exe), "--fasta", str(b), "-K", "24", "--graph_per_record", "--SS"],
                        stdout=subprocess.PIPE, check=True).stdout
    assert ss == oracle.debruijn(b.read_bytes(), 24, True)
    bad = subprocess.run([str(exe), "--fasta", str(b), "-K", "24"], stdout=subprocess.PIPE, stderr=subprocess.PIPE)
    assert bad.returncode != 0
