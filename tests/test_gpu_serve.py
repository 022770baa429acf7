"""The job server: a mix of counting, normalization and assignment jobs of
different sizes, submitted together, runs concurrently and every result is
bit-identical to the same job run alone through the plain calls."""
import numpy as np
import pytest

from trinityrnaseq_gb300 import native as N
from trinityrnaseq_gb300 import synth
from trinityrnaseq_gb300.serve import Server, plain_run

pytestmark = pytest.mark.gpu


def same(a, b):
    if isinstance(a, (bytes, bytearray)):
        return a == b
    if isinstance(a, tuple):
        return all(same(x, y) for x, y in zip(a, b))
    a, b = np.asarray(a), np.asarray(b)
    return a.shape == b.shape and np.array_equal(a.view(np.uint8), b.view(np.uint8))


def job_mix():
    jobs = []
    for i, n in enumerate((2000, 40000, 5000, 120000)):
        jobs.append((N.TK_JOB_COUNT, synth.transcriptome_reads(seed=100 + i, n_reads=n).tobytes(), b"", 1 + (i % 2)))
    for i, n in enumerate((3000, 30000)):
        l, r = synth.gene_pairs(seed=200 + i, n_genes=300, n_pairs=n, fastq=bool(i % 2))
        jobs.append((N.TK_JOB_NORMALIZE, l.tobytes(), r.tobytes(), 1))
    b, r = synth.bundle_reads(seed=300, n_contigs=800, n_components=250, max_per_component=10, n_pairs=20000)
    jobs.append((N.TK_JOB_R2T, r.tobytes(), b.tobytes(), 1))
    return jobs


def submit(srv, kind, t1, t2, mc):
    if kind == N.TK_JOB_COUNT:
        return srv.submit_count(t1, min_count=mc)
    if kind == N.TK_JOB_NORMALIZE:
        return srv.submit_normalize(t1, t2)
    return srv.submit_r2t(t1, t2)


@pytest.mark.parametrize("slots,budget", [(4, 0), (3, 64 << 20)])
def test_served_equals_alone(ctx, slots, budget):
    jobs = job_mix()
    alone = [plain_run(ctx, k, t1, t2, min_count=mc) for k, t1, t2, mc in jobs]
    with Server(ctx.device, slots=slots, hbm_budget=budget) as srv:
        ids = [submit(srv, *j) for j in jobs]
        for jid, (kind, *_), want in zip(ids, jobs, alone):
            st, lat, q = srv.wait(jid)
            assert st == 0, srv.error(jid)
            assert lat >= q >= 0
            assert same(srv.result(jid, kind), want)
            srv.release(jid)
        bud, in_use, maxc = srv.stats()
        assert in_use == 0
        if budget == 0:
            assert maxc > 1          # jobs overlapped on the GPU
        else:
            assert maxc >= 1         # a tight budget admits jobs as memory frees up


def test_queued_count_jobs_are_batched(ctx):
    """Count jobs queued behind a running one run as bins of one batched pass,
    with per-job minimum counts and histograms equal to their solo runs."""
    jobs = []
    for i in range(12):
        txt = synth.transcriptome_reads(seed=500 + i, n_reads=1500 + 700 * i, fastq=bool(i % 3 == 0)).tobytes()
        if i == 4:
            txt = txt[:-1]          # no trailing newline
        jobs.append((txt, 1 + (i % 3)))
    alone = [plain_run(ctx, N.TK_JOB_COUNT, t, min_count=mc) for t, mc in jobs]
    with Server(ctx.device, slots=1) as srv:
        ids = [srv.submit_count(t, min_count=mc) for t, mc in jobs]
        for jid, want in zip(ids, alone):
            st, _, _ = srv.wait(jid)
            assert st == 0, srv.error(jid)
            assert same(srv.result(jid, N.TK_JOB_COUNT), want)
        assert srv.batched_jobs() > 0


def test_bad_job_fails_alone(ctx):
    with Server(ctx.device, slots=2) as srv:
        bad = srv.submit_count(b"@r\nACGT\n+\nII\n@x\n")   # truncated FASTQ
        good = srv.submit_count(synth.transcriptome_reads(seed=7, n_reads=1000).tobytes())
        st, _, _ = srv.wait(bad)
        assert st == N.TK_E_PARSE
        st2, _, _ = srv.wait(good)
        assert st2 == 0


def test_served_normalization_selects_like_plain_calls(ctx):
    """A normalize job with max_cov selects and extracts what tk_norm does
    alone, FASTA and FASTQ mates, while other jobs share the GPU."""
    jobs = []
    for i, fq in enumerate((False, True)):
        l, r = synth.gene_pairs(seed=400 + i, n_genes=200, n_pairs=20000, fastq=fq)
        jobs.append((l.tobytes(), r.tobytes(), (5 + 20 * i, 1, 10000)))
    want = [plain_run(ctx, "normalize_select", l, r, norm=nm) for l, r, nm in jobs]
    with Server(ctx.device, slots=3) as srv:
        ids = [srv.submit_normalize(l, r, max_cov=nm[0], min_cov=nm[1], max_cv=nm[2]) for l, r, nm in jobs]
        extra = srv.submit_count(jobs[0][0])
        for jid, w in zip(ids, want):
            st, _, _ = srv.wait(jid)
            assert st == 0, srv.error(jid)
            got = srv.result(jid, "normalize_select")
            assert got[0] == w[0] and got[1] == w[1] and got[2] == w[2] and got[3] == w[3]
            assert got[1][1] == len(got[0].splitlines()) > 0
            srv.release(jid)
        assert srv.wait(extra)[0] == 0
        srv.release(extra)


def test_admission_waits_for_free_device_memory(ctx):
    """With most of the GPU's memory held outside the server (here by
    PyTorch), jobs that fit the budget but not the free memory are held back
    and run one at a time; every result still equals the job run alone."""
    torch = pytest.importorskip("torch")
    dev = torch.device(f"cuda:{ctx.device}")
    jobs = [(N.TK_JOB_COUNT, synth.transcriptome_reads(seed=500 + i, n_reads=400000).tobytes(), b"", 1)
            for i in range(3)]
    alone = [plain_run(ctx, k, t1, t2, min_count=mc) for k, t1, t2, mc in jobs]
    ctx.trim()
    torch.cuda.synchronize(dev)
    free, total = torch.cuda.mem_get_info(dev)
    # leave about 3 GB free: less than the 1/64 margin plus a job's estimate
    # (32 x its ~31 MB text), more than a job of this size really allocates
    hog = torch.empty(max(0, free - (3 << 30)), dtype=torch.uint8, device=dev)
    try:
        with Server(ctx.device, slots=3, hbm_budget=1 << 40) as srv:
            ids = [submit(srv, *j) for j in jobs]
            for jid, (kind, *_), want in zip(ids, jobs, alone):
                st, _, _ = srv.wait(jid)
                assert st == 0, srv.error(jid)
                assert same(srv.result(jid, kind), want)
                srv.release(jid)
            assert srv.held_by_free_memory() > 0
            assert srv.stats()[2] == 1       # never two at once
    finally:
        del hog
        torch.cuda.empty_cache()
