"""The normalization tail on the GPU (tk_norm_*): each side's stats sorted by
read name, nbkc_merge_left_right_stats.pl --sorted, nbkc_normalize.pl, and
make_normalized_reads_file -- against the reference scripts' own output
(golden fixtures) and the oracle's restatement of them, byte for byte."""
import random

import numpy as np
import pytest

from trinityrnaseq_gb300 import KmerTable, Normalization, ReadSet, coverage_stats, format_stats, native, synth

pytestmark = pytest.mark.gpu


def table_inputs(ctx, stats: bytes):
    """A read set named as the table's rows, and the rows' values."""
    rows = [l.split(b"\t") for l in stats.split(b"\n")[1:] if l]
    fasta = b"".join(b">" + r[0] + b"\nACGT\n" for r in rows)
    med = np.array([int(r[1]) for r in rows], dtype=np.uint32)
    mean = np.array([float(r[2]) for r in rows], dtype=np.float32)
    sd = np.array([float(r[3]) for r in rows], dtype=np.float32)
    rs = ReadSet(ctx, fasta)
    assert rs.n_reads == len(rows)
    return rs, (med, mean, sd)


@pytest.mark.parametrize("args,fixture,counts", [
    ((5, 2, 1), "norm.pairs.c5.accs", (133, 49, 49, 14)),
    ((200, 1, 10000), "norm.pairs.c200.accs", (133, 99, 30, 4)),
])
def test_pairs_match_reference_scripts(ctx, golden, args, fixture, counts):
    lrs, ls = table_inputs(ctx, (golden / "norm.left.stats").read_bytes())
    rrs, rs = table_inputs(ctx, (golden / "norm.right.stats").read_bytes())
    nm = Normalization(ctx, lrs, ls, rrs, rs, *args)
    assert nm.table() == (golden / "norm.pairs.stats").read_bytes()
    assert nm.accs() == (golden / fixture).read_bytes()
    c = nm.counts
    assert (c["rows"], c["selected"], c["aberrant"], c["below_min"]) == counts


def test_single_side_matches_reference_script(ctx, golden, oracle):
    stats = (golden / "norm.left.stats").read_bytes()
    lrs, ls = table_inputs(ctx, stats)
    nm = Normalization(ctx, lrs, ls, None, None, 5, 2, 1)
    assert nm.accs() == (golden / "norm.left.c5.accs").read_bytes()
    table, _, cnt = oracle.norm(stats, None, 5, 2, 1)
    assert nm.table() == table
    assert nm.counts["selected"] == cnt[1]


def test_extract_matches_reference(ctx, golden):
    lrs, ls = table_inputs(ctx, (golden / "norm.left.stats").read_bytes())
    rrs, rs = table_inputs(ctx, (golden / "norm.right.stats").read_bytes())
    nm = Normalization(ctx, lrs, ls, rrs, rs, 5, 2, 1)
    fq = ReadSet(ctx, (golden / "norm.left.fq").read_bytes())
    assert nm.extract(fq) == (golden / "norm.left.c5.fq").read_bytes()
    # without the record of a selected name: the script dies, so does this
    recs = (golden / "norm.left.fq").read_bytes().split(b"\n")
    drop = [i for i in range(0, len(recs) - 1, 4) if recs[i].startswith(b"@x/2")][0]
    short = ReadSet(ctx, b"\n".join(recs[:drop] + recs[drop + 4:]))
    with pytest.raises(native.TrinkmerError) as e:
        nm.extract(short)
    assert e.value.status == native.TK_E_PARSE


def test_extract_fasta(ctx, golden, oracle):
    """FASTA input: the name z\xc3z loses its high byte in Fasta_reader, so
    the full selection dies as the script does; without that pair the records
    are those the oracle (pinned to Fasta_reader's output) extracts."""
    lt, rt = (golden / "norm.left.stats").read_bytes(), (golden / "norm.right.stats").read_bytes()
    fa_text = (golden / "norm.left.fa").read_bytes()
    fa = ReadSet(ctx, fa_text)
    lrs, ls = table_inputs(ctx, lt)
    rrs, rs = table_inputs(ctx, rt)
    nm = Normalization(ctx, lrs, ls, rrs, rs, 5, 2, 1)
    with pytest.raises(native.TrinkmerError) as e:
        nm.extract(fa)
    assert e.value.status == native.TK_E_PARSE

    def drop(t):
        return b"".join(l + b"\n" for l in t.split(b"\n") if l and not l.startswith(b"z\xc3z"))
    lrs2, ls2 = table_inputs(ctx, drop(lt))
    rrs2, rs2 = table_inputs(ctx, drop(rt))
    nm2 = Normalization(ctx, lrs2, ls2, rrs2, rs2, 5, 2, 1)
    got = nm2.extract(fa)
    assert got == oracle.norm_extract(fa_text, nm2.accs())
    assert got.count(b">") == len(nm2.accs().splitlines())


def test_earlier_pair_fixture(ctx, golden):
    lrs, ls = table_inputs(ctx, (golden / "left.stats").read_bytes())
    rrs, rs = table_inputs(ctx, (golden / "right.stats").read_bytes())
    nm = Normalization(ctx, lrs, ls, rrs, rs, 3, 1, 10000)
    assert nm.table() == (golden / "pairs.stats").read_bytes()
    assert nm.accs() == (golden / "normalized.accs").read_bytes()


def shuffled_fastq(text: bytes, seed: int, drop: float = 0.0) -> bytes:
    recs = text.split(b"\n")
    recs = [b"\n".join(recs[i:i + 4]) + b"\n" for i in range(0, len(recs) - 1, 4)]
    rnd = random.Random(seed)
    rnd.shuffle(recs)
    if drop:
        recs = [r for r in recs if rnd.random() >= drop]
    return b"".join(recs)


@pytest.mark.parametrize("seed,max_cov,drop", [(61, 5, 0.0), (62, 30, 0.02), (63, 200, 0.1)])
def test_pipeline_parity_100k_pairs(ctx, oracle, seed, max_cov, drop):
    """FASTQ -> prep -> count -> stats -> sort/merge/select -> extract, mates in
    shuffled orders with unpaired reads on both sides, against the oracle on
    the stats tables fastaToKmerCoverageStats would print."""
    left, right = synth.gene_pairs(seed=seed, n_genes=400, n_pairs=100000, fastq=True)
    lfq, rfq = shuffled_fastq(left.tobytes(), seed, drop), shuffled_fastq(right.tobytes(), seed + 1, drop)
    lq, rq = ReadSet(ctx, lfq), ReadSet(ctx, rfq)
    lfa, rfa = ReadSet(ctx, lq.to_fasta(1, if_missing=True)), ReadSet(ctx, rq.to_fasta(2, if_missing=True))
    t = KmerTable(ctx, 25, True)
    t.add(lfa)
    t.add(rfa)
    ls, rs = coverage_stats(t, lfa), coverage_stats(t, rfa)
    nm = Normalization(ctx, lfa, ls, rfa, rs, max_cov, 1, 10000)
    lt = format_stats(lfa.accessions(), *ls)
    rt = format_stats(rfa.accessions(), *rs)
    table, accs, cnt = oracle.norm(lt, rt, max_cov, 1, 10000)
    assert nm.accs() == accs
    assert nm.table() == table
    c = nm.counts
    assert (c["rows"], c["selected"], c["aberrant"], c["below_min"]) == cnt
    assert nm.extract(lq) == oracle.norm_extract(lfq, accs)
    assert nm.extract(rq) == oracle.norm_extract(rfq, accs)


def test_odd_names_take_the_repair_walk(ctx, oracle):
    """Names whose sorted orders disagree with their pairing (punctuation
    around '/', /3 endings, duplicates) make speculative merge chunks miss
    their successors; the walk is redone sequentially and must agree."""
    rnd = random.Random(7)
    alpha = "ab/.01-_"
    cores = sorted({"r" + "".join(rnd.choice(alpha) for _ in range(rnd.randint(0, 6))) for _ in range(20000)})
    left, right = [], []
    for cname in cores:
        p = rnd.random()
        if p < 0.6:
            left.append(cname + "/1"); right.append(cname + "/2")
        elif p < 0.75:
            left.append(cname + "/1")
        elif p < 0.9:
            right.append(cname + "/2")
        else:
            left.append(cname); right.append(cname + "/" + rnd.choice("123"))
    left += rnd.sample(left, 50)   # duplicate names
    rnd.shuffle(left)
    rnd.shuffle(right)

    def side(names):
        med = np.array([rnd.randint(0, 20) for _ in names], dtype=np.uint32)
        mean = np.array([rnd.choice([0.0, 1.5, 2.25, 7.0, 13.37, 100.5]) for _ in names], dtype=np.float32)
        sd = np.array([rnd.choice([0.0, 0.5, 1.25, 3.3, 40.0]) for _ in names], dtype=np.float32)
        fa = "".join(f">{n}\nACGT\n" for n in names).encode()
        return ReadSet(ctx, fa), (med, mean, sd), format_stats([n.encode() for n in names], med, mean, sd)

    lrs, ls, lt = side(left)
    rrs, rs, rt = side(right)
    nm = Normalization(ctx, lrs, ls, rrs, rs, 4, 1, 2)
    table, accs, cnt = oracle.norm(lt, rt, 4, 1, 2)
    assert nm.table() == table
    assert nm.accs() == accs
    single = Normalization(ctx, lrs, ls, None, None, 4, 1, 2)
    t1, a1, _ = oracle.norm(lt, None, 4, 1, 2)
    assert single.table() == t1
    assert single.accs() == a1


def test_empty_and_device_inputs(ctx, oracle):
    import torch
    empty = ReadSet(ctx, b"")
    nm = Normalization(ctx, empty, (np.zeros(0, np.uint32), np.zeros(0, np.float32), np.zeros(0, np.float32)))
    assert nm.accs() == b"" and nm.counts["rows"] == 0
    assert nm.table() == b"acc\tmedian_cov\tmean_cov\tstdev\n"
    # statistics already on the device
    names = [f"q{i}/1" for i in range(1000)]
    rs = ReadSet(ctx, "".join(f">{n}\nACGT\n" for n in names).encode())
    med = torch.arange(1000, dtype=torch.int32, device="cuda") % 9
    mean = torch.linspace(0.5, 50, 1000, device="cuda")
    sd = torch.linspace(0, 5, 1000, device="cuda")
    torch.cuda.synchronize()
    nm = Normalization(ctx, rs, (med.data_ptr(), mean.data_ptr(), sd.data_ptr()), max_cov=3, device=True)
    host = (med.cpu().numpy().astype(np.uint32), mean.cpu().numpy(), sd.cpu().numpy())
    _, accs, _ = oracle.norm(format_stats([n.encode() for n in names], *host), None, 3, 1, 10000)
    assert nm.accs() == accs


def test_out_of_range_statistics_are_rejected(ctx):
    rs = ReadSet(ctx, b">a/1\nACGT\n>b/1\nACGT\n")
    bad = (np.array([1, 1], np.uint32), np.array([1.0, np.inf], np.float32), np.array([0, 0], np.float32))
    with pytest.raises(native.TrinkmerError) as e:
        Normalization(ctx, rs, bad)
    assert e.value.status == native.TK_E_INVAL
    # min_cov 0 with a median of 0 selected: Perl dies dividing by it
    zero = (np.array([0, 1], np.uint32), np.array([1.0, 1.0], np.float32), np.array([0, 0], np.float32))
    with pytest.raises(native.TrinkmerError):
        Normalization(ctx, rs, zero, min_cov=0)


def test_sides_in_pieces_select_like_whole_sides(ctx, oracle):
    """tk_norm_select_multi: a side split into record-aligned pieces (each its
    own read set, statistics concatenated in order) selects what the whole
    side selects, and the pieces' extractions concatenate to the whole one."""
    from trinityrnaseq_gb300.kmer import split_records
    left, right = synth.gene_pairs(seed=64, n_genes=300, n_pairs=60000, fastq=True)
    lfq, rfq = shuffled_fastq(left.tobytes(), 5, 0.01), shuffled_fastq(right.tobytes(), 6, 0.01)
    whole = [ReadSet(ctx, lfq), ReadSet(ctx, rfq)]
    t = KmerTable(ctx, 25, True)
    t.add_many(whole)
    stats = [coverage_stats(t, r) for r in whole]
    nm = Normalization(ctx, whole[0], stats[0], whole[1], stats[1], 20, 1, 10000)
    pieces = []
    for text in (lfq, rfq):
        cuts = split_records(text, 3)
        pieces.append([ReadSet(ctx, text[cuts[i]:cuts[i + 1]]) for i in range(3)])
    nm2 = Normalization(ctx, pieces[0], stats[0], pieces[1], stats[1], 20, 1, 10000)
    assert nm2.accs() == nm.accs()
    assert nm2.table() == nm.table()
    for side in range(2):
        assert nm2.extract(pieces[side]) == nm.extract(whole[side])
    # one piece alone lacks records of selected names: an error, as for a short file
    with pytest.raises(native.TrinkmerError):
        nm2.extract(pieces[0][0])


def test_extract_copy_async_overlaps_the_next_extraction(ctx):
    """tk_norm_extract_copy_async: one side's records go down on the copy
    stream while the other side's are extracted; both land intact."""
    torch = pytest.importorskip("torch")
    left, right = synth.gene_pairs(seed=33, n_genes=300, n_pairs=30000, fastq=True)
    sides = [ReadSet(ctx, x.tobytes()) for x in (left, right)]
    fas = [ReadSet(ctx, r.to_fasta(a, if_missing=True)) for r, a in zip(sides, (1, 2))]
    t = KmerTable(ctx, 25, True)
    t.add_many(fas)
    st = [coverage_stats(t, r) for r in fas]
    nm = Normalization(ctx, fas[0], st[0], fas[1], st[1], 20, 1, 10000)
    want = [nm.extract(r) for r in sides]
    assert all(len(w) > 0 for w in want)
    bufs = [torch.zeros(len(w) + 16, dtype=torch.uint8).pin_memory() for w in want]
    lens = [nm.extract_into(r, b.data_ptr(), b.numel(), overlap=True) for r, b in zip(sides, bufs)]
    ctx.synchronize()
    for b, n, w in zip(bufs, lens, want):
        assert b.numpy()[:n].tobytes() == w
    # several extractions in flight at once (each earlier text kept until its
    # copy ends), then the handle freed before anything is waited for
    more = [torch.zeros(len(want[i % 2]) + 16, dtype=torch.uint8).pin_memory() for i in range(5)]
    lens = [nm.extract_into(sides[i % 2], b.data_ptr(), b.numel(), overlap=True) for i, b in enumerate(more)]
    nm.free()
    ctx.synchronize()
    for i, (b, n) in enumerate(zip(more, lens)):
        assert b.numpy()[:n].tobytes() == want[i % 2]
