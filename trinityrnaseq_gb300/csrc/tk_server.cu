// tk_server.cu -- continuous-batching job server for the k-mer path (host code).
//
// The reference's only job-level concurrency is ParaFly running independent
// processes (trinity-plugins/ParaFly, Trinity:3652) and Perl threads running
// two fastaToKmerCoverageStats at once (util/insilico_read_normalization.pl:
// 853-854).  Here one resident process keeps a set of worker slots, each with
// its own CUDA context stream, and admits queued jobs whenever a slot is free,
// the job's HBM estimate fits the remaining budget and the GPU has that much
// memory free (first queued job that fits, so small jobs flow around a large
// one that waits for memory).  Jobs in
// different slots run concurrently on the GPU.  Every job computes exactly
// what the plain single-job calls compute, so a result does not depend on
// what else was running.
#include "tk_internal.cuh"

#include <algorithm>
#include <chrono>
#include <condition_variable>
#include <cstring>
#include <new>
#include <deque>
#include <map>
#include <memory>
#include <mutex>
#include <thread>

namespace {

using clk = std::chrono::steady_clock;

struct Job {
    uint64_t id = 0;
    tk_job_spec spec{};
    uint64_t est = 0;
    int status = 1;                          // 1 = pending / running
    clk::time_point t_submit, t_start, t_done;
    std::vector<std::vector<char>> out;      // per-kind outputs (see tk_job_output)
    std::string error;
};

}  // namespace

struct tk_server {
    int device = 0;
    uint64_t budget = 0;
    uint64_t in_use = 0;
    bool stop = false;
    uint64_t next_id = 1;
    std::mutex mu;
    std::condition_variable cv_work, cv_done;
    std::deque<Job *> queue;
    std::map<uint64_t, std::unique_ptr<Job>> jobs;
    std::vector<std::thread> workers;
    int slots = 0;
    int running = 0;
    int max_running = 0;
    uint64_t batched_jobs = 0;               // jobs that ran inside a batched pass
    uint64_t held_by_free = 0;               // admissions put off because the GPU had too little free memory
};

namespace {

// device bytes a job may hold at its peak: text copies, packed reads, line
// arrays, bucketed k-mers and a table at <= 0.6 load (distinct <= windows)
uint64_t job_estimate(const tk_job_spec &s) {
    uint64_t a = s.len, b = s.len2;
    switch (s.kind) {
    case TK_JOB_COUNT: return 32 * a + (64ULL << 20);
    case TK_JOB_NORMALIZE: return (s.max_cov >= 2 ? 40 : 32) * (a + b) + (64ULL << 20);
    case TK_JOB_R2T: return 6 * a + 48 * b + (64ULL << 20);
    default: return 64ULL << 20;
    }
}

template <typename T>
std::vector<char> as_bytes(const std::vector<T> &v) {
    std::vector<char> o(v.size() * sizeof(T));
    if (!o.empty()) std::memcpy(o.data(), v.data(), o.size());
    return o;
}

int run_count(tk_ctx *c, Job &j) {
    const tk_job_spec &s = j.spec;
    tk_table *t = nullptr;
    tk_reads *r = nullptr;
    int e = tk_table_create(c, s.k, s.canonical, 0, &t);
    if (!e) e = tk_reads_parse(c, s.text, s.len, TK_HOST, &r);
    if (!e) e = tk_table_add_reads(t, r);
    std::vector<uint64_t> hist(10002);   // below 1, 1..10000, above 10000
    if (!e) e = tk_table_histo(t, 1, 10000, hist.data());
    uint64_t len = 0;
    if (!e) e = tk_table_dump_fasta(t, s.min_count ? s.min_count : 1, TK_HOST, nullptr, 0, &len);
    std::vector<char> dump(len);
    if (!e && len) e = tk_table_dump_fasta(t, s.min_count ? s.min_count : 1, TK_HOST, dump.data(), len, &len);
    if (r) tk_reads_free(r);
    if (t) tk_table_free(t);
    if (!e) {
        j.out.push_back(std::move(dump));
        j.out.push_back(as_bytes(hist));
    }
    return e;
}

// first non-whitespace byte of a job's text ('>' FASTA, '@' FASTQ)
char text_format(const tk_job_spec &s) {
    for (uint64_t i = 0; i < s.len; i++) {
        char ch = s.text[i];
        if (ch != ' ' && ch != '\t' && ch != '\n' && ch != '\r') return ch;
    }
    return 0;
}

// Several count jobs as the bins of one batched pass (tk_count_bins_ex): one
// parse, one persistent counting launch, one dump formatting for all of them.
// The texts are copied straight into one device buffer, a newline between
// jobs whose text does not end with one.
int run_count_batch(tk_ctx *c, std::vector<Job *> &batch) {
    const uint32_t n = (uint32_t)batch.size();
    std::vector<uint64_t> off(n + 1);
    std::vector<uint32_t> minc(n);
    uint64_t total = 0;
    for (uint32_t i = 0; i < n; i++) {
        const tk_job_spec &s = batch[i]->spec;
        off[i] = total;
        total += s.len + ((s.len && s.text[s.len - 1] != '\n') ? 1 : 0);
        minc[i] = s.min_count ? s.min_count : 1;
    }
    off[n] = total;
    char *d_text = nullptr;
    int e = tk::dmalloc(c, (void **)&d_text, total + 64, "batched count text");
    static const char nl = '\n';
    for (uint32_t i = 0; !e && i < n; i++) {
        const tk_job_spec &s = batch[i]->spec;
        if (s.len) e = tk::cuda_check(c, cudaMemcpyAsync(d_text + off[i], s.text, s.len, cudaMemcpyHostToDevice, c->stream), "batch h2d");
        if (!e && off[i] + s.len < off[i + 1])
            e = tk::cuda_check(c, cudaMemcpyAsync(d_text + off[i] + s.len, &nl, 1, cudaMemcpyHostToDevice, c->stream), "batch sep");
    }
    std::vector<uint64_t> histos((size_t)n * 10002);
    tk_bins *bins = nullptr;
    if (!e) e = tk_count_bins_ex(c, d_text, total, TK_DEVICE, off.data(), n, batch[0]->spec.k, batch[0]->spec.canonical,
                                 minc.data(), histos.data(), &bins);
    uint64_t tlen = 0;
    std::vector<uint64_t> toff(n + 1);
    std::vector<char> text;
    if (!e) e = tk_bins_info(bins, &tlen, nullptr);
    if (!e) e = tk_bins_dump_offsets(bins, toff.data());
    if (!e) {
        text.resize(tlen);
        e = tk_bins_dump_text(bins, text.data(), tlen);
    }
    if (bins) tk_bins_free(bins);
    if (d_text) tk::dfree(c, d_text);
    if (e) return e;
    for (uint32_t i = 0; i < n; i++) {
        Job &j = *batch[i];
        j.out.clear();
        j.out.emplace_back(text.begin() + (long)toff[i], text.begin() + (long)toff[i + 1]);
        std::vector<char> h(10002 * 8);
        std::memcpy(h.data(), histos.data() + (size_t)i * 10002, h.size());
        j.out.push_back(std::move(h));
    }
    return TK_OK;
}

int run_normalize(tk_ctx *c, Job &j) {
    const tk_job_spec &s = j.spec;
    tk_table *t = nullptr;
    tk_reads *rl = nullptr, *rr = nullptr;
    int e = tk_table_create(c, s.k, s.canonical, 0, &t);
    if (!e) e = tk_reads_parse(c, s.text, s.len, TK_HOST, &rl);
    if (!e) e = tk_reads_parse(c, s.text2, s.len2, TK_HOST, &rr);
    if (!e) {
        const tk_reads *sets[2] = {rl, rr};
        e = tk_table_add_reads_multi(t, sets, 2);
    }
    std::vector<std::vector<char>> names;
    for (tk_reads *r : {rl, rr}) {
        if (e || !r) break;
        uint64_t n = 0;
        tk_reads_info(r, &n, nullptr, nullptr, nullptr);
        std::vector<uint32_t> med(n), nlen(n);
        std::vector<float> mean(n), sd(n);
        std::vector<uint64_t> noff(n);
        if (n) e = tk_coverage_stats(t, r, TK_HOST, med.data(), mean.data(), sd.data());
        if (!e && n) e = tk_reads_names(r, noff.data(), nlen.data());
        j.out.push_back(as_bytes(med));
        j.out.push_back(as_bytes(mean));
        j.out.push_back(as_bytes(sd));
        names.push_back(as_bytes(noff));
        names.push_back(as_bytes(nlen));
    }
    for (auto &v : names) j.out.push_back(std::move(v));
    if (!e && s.max_cov >= 2) {
        // the insilico selection and extraction over the statistics just computed
        auto ptr = [&](int which) { return (const void *)j.out[which].data(); };
        tk_norm *nm = nullptr;
        e = tk_norm_select(c, rl, (const uint32_t *)ptr(0), (const float *)ptr(1), (const float *)ptr(2), rr,
                           (const uint32_t *)ptr(3), (const float *)ptr(4), (const float *)ptr(5), TK_HOST,
                           s.max_cov, s.min_cov, s.max_cv, &nm);
        tk_norm_counts cnt{};
        uint64_t alen = 0;
        if (!e) e = tk_norm_info(nm, &cnt, &alen);
        std::vector<char> accs(alen);
        if (!e && alen) e = tk_norm_accs(nm, TK_HOST, accs.data(), alen);
        std::vector<std::vector<char>> recs;
        for (tk_reads *r : {rl, rr}) {
            uint64_t n = 0;
            if (!e) e = tk_norm_extract(nm, r, &n);
            std::vector<char> t(n);
            if (!e && n) e = tk_norm_extract_copy(nm, TK_HOST, t.data(), n);
            recs.push_back(std::move(t));
        }
        if (nm) tk_norm_free(nm);
        if (!e) {
            const uint64_t cv[4] = {cnt.rows, cnt.selected, cnt.aberrant, cnt.below_min};
            j.out.push_back(std::move(accs));
            j.out.push_back(as_bytes(std::vector<uint64_t>(cv, cv + 4)));
            for (auto &t : recs) j.out.push_back(std::move(t));
        }
    }
    if (rl) tk_reads_free(rl);
    if (rr) tk_reads_free(rr);
    if (t) tk_table_free(t);
    return e;
}

int run_r2t(tk_ctx *c, Job &j) {
    const tk_job_spec &s = j.spec;
    tk_r2t *z = nullptr;
    tk_reads *r = nullptr;
    int e = tk_r2t_create(c, s.text2, s.len2, TK_HOST, s.k, s.strand, &z);
    if (!e) e = tk_reads_parse(c, s.text, s.len, TK_HOST, &r);
    uint64_t n = 0;
    if (!e) tk_reads_info(r, &n, nullptr, nullptr, nullptr);
    std::vector<int32_t> rec(n);
    std::vector<uint32_t> hits(n), nwin(n), nlen(n);
    std::vector<uint64_t> noff(n), roff(n + 1), comp;
    if (!e && n) e = tk_r2t_assign(z, r, TK_HOST, rec.data(), hits.data(), nwin.data());
    if (!e && n) e = tk_reads_names(r, noff.data(), nlen.data());
    if (!e) e = tk_reads_offsets(r, roff.data());
    std::vector<char> seq(roff[n]);
    if (!e && roff[n]) e = tk_reads_copy_seq(r, seq.data(), roff[n]);
    uint64_t nrec = 0;
    if (!e) e = tk_r2t_info(z, &nrec, nullptr);
    comp.resize(nrec);
    if (!e && nrec) e = tk_r2t_component_ids(z, comp.data());
    if (r) tk_reads_free(r);
    if (z) tk_r2t_free(z);
    if (!e) {
        j.out.push_back(as_bytes(rec));
        j.out.push_back(as_bytes(hits));
        j.out.push_back(as_bytes(nwin));
        j.out.push_back(as_bytes(noff));
        j.out.push_back(as_bytes(nlen));
        j.out.push_back(as_bytes(roff));
        j.out.push_back(std::move(seq));
        j.out.push_back(as_bytes(comp));
    }
    return e;
}

constexpr size_t BATCH_JOBS = 64;
constexpr uint64_t BATCH_BYTES = 256ULL << 20;

// Device memory a job starting on slot context c can get now: what the GPU
// reports free plus the blocks c keeps cached for reuse, less a margin for
// the CUDA runtime's own needs.  Memory the other slots' running jobs have not
// allocated yet is covered by the budget check; this check catches memory
// held outside the budget (other processes, other slots' caches).
uint64_t free_for(tk_ctx *c) {
    size_t f = 0, t = 0;
    if (!c || cudaMemGetInfo(&f, &t) != cudaSuccess) {
        cudaGetLastError();
        return ~0ULL;   // unknown: leave admission to the budget
    }
    const uint64_t avail = (uint64_t)f + tk::ctx_cached_bytes(c), margin = (uint64_t)t / 64;
    return avail > margin ? avail - margin : 0;
}

void worker_loop(tk_server *s) {
    tk_ctx *c = nullptr;
    int ce = tk_ctx_create(s->device, &c);
    for (;;) {
        std::vector<Job *> batch;
        {
            std::unique_lock<std::mutex> lk(s->mu);
            for (;;) {
                if (s->stop) {
                    if (c) tk_ctx_destroy(c);
                    return;
                }
                // first queued job that fits both the remaining budget and the
                // memory the GPU has free for this slot (its estimate is an
                // upper bound of what it allocates); a job larger than either
                // runs when nothing else is running
                const uint64_t avail = s->queue.empty() ? 0 : free_for(c);
                bool held = false;
                for (auto it = s->queue.begin(); it != s->queue.end(); ++it) {
                    uint64_t need = std::min((*it)->est, s->budget);
                    const bool fits_budget = s->in_use + need <= s->budget;
                    const bool fits_free = need <= avail || s->running == 0;
                    if (fits_budget && !fits_free) held = true;
                    if (fits_budget && fits_free) {
                        Job *j = *it;
                        s->queue.erase(it);
                        s->in_use += need;
                        j->est = need;
                        batch.push_back(j);
                        break;
                    }
                }
                if (held) s->held_by_free++;
                if (!batch.empty()) break;
                s->cv_work.wait(lk);
            }
            // continuous batching: later count jobs of the same kind of input
            // join this one in a single batched pass while memory allows
            Job *head = batch[0];
            const uint64_t fb = free_for(c);
            const uint64_t avail_batch = fb == ~0ULL ? ~0ULL : s->in_use - head->est + fb;
            if (head->spec.kind == TK_JOB_COUNT && head->spec.len < BATCH_BYTES) {
                uint64_t bytes = head->spec.len;
                const char fmt = text_format(head->spec);
                for (auto it = s->queue.begin(); it != s->queue.end() && batch.size() < BATCH_JOBS;) {
                    Job *j = *it;
                    const tk_job_spec &q = j->spec;
                    uint64_t need = std::min(j->est, s->budget);
                    if (q.kind == TK_JOB_COUNT && q.k == head->spec.k && q.canonical == head->spec.canonical &&
                        bytes + q.len <= BATCH_BYTES && text_format(q) == fmt && s->in_use + need <= s->budget &&
                        s->in_use + need <= avail_batch) {
                        it = s->queue.erase(it);
                        s->in_use += need;
                        j->est = need;
                        bytes += q.len;
                        batch.push_back(j);
                    } else {
                        ++it;
                    }
                }
            }
            s->running++;
            s->max_running = std::max(s->max_running, s->running);
        }
        const auto t_start = clk::now();
        for (Job *j : batch) j->t_start = t_start;
        std::vector<int> st(batch.size(), ce);
        if (!ce) {
            int be = batch.size() > 1 ? run_count_batch(c, batch) : -1;
            for (size_t i = 0; i < batch.size(); i++) {
                if (be == TK_OK) { st[i] = TK_OK; continue; }
                Job &j = *batch[i];        // alone, or the batch failed: one by one
                j.out.clear();
                switch (j.spec.kind) {
                case TK_JOB_COUNT: st[i] = run_count(c, j); break;
                case TK_JOB_NORMALIZE: st[i] = run_normalize(c, j); break;
                case TK_JOB_R2T: st[i] = run_r2t(c, j); break;
                default: st[i] = TK_E_INVAL;
                }
                if (st[i]) j.error = tk_ctx_last_error(c);
            }
        }
        // keep this slot's cache of freed blocks within its share of the budget
        if (c && tk::ctx_cached_bytes(c) > s->budget / (uint64_t)s->slots) tk_ctx_trim(c);
        {
            std::lock_guard<std::mutex> lk(s->mu);
            const auto t_done = clk::now();
            for (size_t i = 0; i < batch.size(); i++) {
                Job *j = batch[i];
                j->t_done = t_done;
                j->status = st[i];
                if (st[i] && j->error.empty()) j->error = c ? tk_ctx_last_error(c) : "no CUDA context";
                s->in_use -= j->est;
            }
            s->running--;
            s->batched_jobs += batch.size() > 1 ? batch.size() : 0;
        }
        s->cv_done.notify_all();
        s->cv_work.notify_all();
    }
}

}  // namespace

extern "C" {

int tk_server_create(int device, int slots, uint64_t hbm_budget, tk_server **out) {
    if (!out || slots < 1 || slots > 64) return TK_E_INVAL;
    *out = nullptr;
    int n = 0;
    if (cudaGetDeviceCount(&n) != cudaSuccess || n <= 0) {
        cudaGetLastError();
        return TK_E_NODEV;
    }
    if (device < 0 || device >= n) return TK_E_INVAL;
    tk_server *s = new (std::nothrow) tk_server();
    if (!s) return TK_E_OOM;
    s->device = device;
    s->slots = slots;
    if (!hbm_budget) {
        size_t f = 0, t = 0;
        cudaSetDevice(device);
        cudaMemGetInfo(&f, &t);
        hbm_budget = (uint64_t)(f * 0.8);
    }
    s->budget = hbm_budget;
    for (int i = 0; i < slots; i++) s->workers.emplace_back(worker_loop, s);
    *out = s;
    return TK_OK;
}

int tk_server_submit(tk_server *s, const tk_job_spec *spec, uint64_t *job_id) {
    if (!s || !spec || !job_id) return TK_E_INVAL;
    if (spec->kind < TK_JOB_COUNT || spec->kind > TK_JOB_R2T) return TK_E_INVAL;
    if (spec->k < 1 || spec->k > tk::MAX_K) return TK_E_INVAL;
    auto j = std::make_unique<Job>();
    j->spec = *spec;
    j->est = job_estimate(*spec);
    j->t_submit = clk::now();
    {
        std::lock_guard<std::mutex> lk(s->mu);
        j->id = s->next_id++;
        *job_id = j->id;
        s->queue.push_back(j.get());
        s->jobs[j->id] = std::move(j);
    }
    s->cv_work.notify_all();
    return TK_OK;
}

int tk_server_wait(tk_server *s, uint64_t id, int *status, uint64_t *latency_ns, uint64_t *queued_ns) {
    if (!s) return TK_E_INVAL;
    std::unique_lock<std::mutex> lk(s->mu);
    auto it = s->jobs.find(id);
    if (it == s->jobs.end()) return TK_E_INVAL;
    Job *j = it->second.get();
    s->cv_done.wait(lk, [&] { return j->status != 1; });
    if (status) *status = j->status;
    if (latency_ns) *latency_ns = (uint64_t)std::chrono::duration_cast<std::chrono::nanoseconds>(j->t_done - j->t_submit).count();
    if (queued_ns) *queued_ns = (uint64_t)std::chrono::duration_cast<std::chrono::nanoseconds>(j->t_start - j->t_submit).count();
    return TK_OK;
}

int tk_job_output(tk_server *s, uint64_t id, int which, const void **data, uint64_t *bytes) {
    if (!s || !data || !bytes) return TK_E_INVAL;
    std::lock_guard<std::mutex> lk(s->mu);
    auto it = s->jobs.find(id);
    if (it == s->jobs.end()) return TK_E_INVAL;
    Job *j = it->second.get();
    if (j->status != TK_OK || which < 0 || which >= (int)j->out.size()) return TK_E_INVAL;
    *data = j->out[(size_t)which].data();
    *bytes = j->out[(size_t)which].size();
    return TK_OK;
}

const char *tk_job_error(tk_server *s, uint64_t id) {
    if (!s) return "no server";
    std::lock_guard<std::mutex> lk(s->mu);
    auto it = s->jobs.find(id);
    return it == s->jobs.end() ? "no such job" : it->second->error.c_str();
}

int tk_job_release(tk_server *s, uint64_t id) {
    if (!s) return TK_E_INVAL;
    std::lock_guard<std::mutex> lk(s->mu);
    auto it = s->jobs.find(id);
    if (it == s->jobs.end() || it->second->status == 1) return TK_E_INVAL;
    s->jobs.erase(it);
    return TK_OK;
}

int tk_server_stats(tk_server *s, uint64_t *budget, uint64_t *in_use, int *max_concurrent) {
    if (!s) return TK_E_INVAL;
    std::lock_guard<std::mutex> lk(s->mu);
    if (budget) *budget = s->budget;
    if (in_use) *in_use = s->in_use;
    if (max_concurrent) *max_concurrent = s->max_running;
    return TK_OK;
}

int tk_server_held_by_free_memory(tk_server *s, uint64_t *admissions) {
    if (!s || !admissions) return TK_E_INVAL;
    std::lock_guard<std::mutex> lk(s->mu);
    *admissions = s->held_by_free;
    return TK_OK;
}

int tk_server_batched_jobs(tk_server *s, uint64_t *jobs) {
    if (!s || !jobs) return TK_E_INVAL;
    std::lock_guard<std::mutex> lk(s->mu);
    *jobs = s->batched_jobs;
    return TK_OK;
}

void tk_server_destroy(tk_server *s) {
    if (!s) return;
    {
        std::unique_lock<std::mutex> lk(s->mu);
        // let queued and running jobs finish
        s->cv_done.wait(lk, [&] { return s->queue.empty() && s->running == 0; });
        s->stop = true;
    }
    s->cv_work.notify_all();
    for (auto &t : s->workers) t.join();
    delete s;
}

}  // extern "C"
