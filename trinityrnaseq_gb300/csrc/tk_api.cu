// tk_api.cu -- the extern "C" boundary of libtrinkmer_cuda.so (include/trinkmer.h).
//
// Host plumbing only: argument checks, stream-ordered device allocation,
// host<->device staging for TK_HOST buffers, CUDA-event profiling and error
// text.  All compute is in the tk_*.cu kernels; there is no CPU fallback --
// without a usable GPU every entry point returns TK_E_NODEV or TK_E_CUDA.
#include "tk_internal.cuh"

#include <algorithm>
#include <cctype>
#include <cstdlib>
#include <cstring>
#include <new>

namespace tk {
int parse_reads(tk_ctx *c, tk_reads *r);
int table_info(tk_table *t, uint64_t *distinct, uint64_t *total, uint64_t *capacity);
int table_histo(tk_table *t, uint64_t low, uint64_t high, uint64_t *hist);
int table_sorted_pairs(tk_table *t, uint32_t min_count, uint64_t **keys, uint32_t **cnt, uint64_t *n);
int table_insert_pairs(tk_table *t, const uint64_t *d_keys, const uint32_t *d_cnt, uint64_t n);
int table_load_dump_reads(tk_table *t, const tk_reads *r);
int coverage_stats(tk_table *t, const tk_reads *rd, uint32_t *d_median, float *d_mean, float *d_stdev);
int r2t_build(tk_r2t *z, const tk_reads *b);
int r2t_assign(tk_r2t *z, const tk_reads *rd, int32_t *d_rec, uint32_t *d_hits, uint32_t *d_nwin);

int set_err(tk_ctx *c, int code, const std::string &msg) {
    if (c) c->last_error = msg;
    return code;
}

int cuda_check(tk_ctx *c, cudaError_t e, const char *what) {
    if (e == cudaSuccess) return TK_OK;
    std::string m = std::string(what) + ": " + cudaGetErrorString(e);
    if (e == cudaErrorMemoryAllocation) return set_err(c, TK_E_OOM, m);
    return set_err(c, TK_E_CUDA, m);
}

int check_launch(tk_ctx *c, const char *what) { return cuda_check(c, cudaGetLastError(), what); }

// Large blocks (tables, bucketed k-mers, texts, dump buffers) come from
// cudaMalloc and, once freed, stay with the context for the next request of
// about the same size.  Carving them out of the stream-ordered pool instead
// left the pool's mapping fragmented after a few rounds of differently sized
// requests, and the random-access kernels on a table placed in it ran 10%
// slower (insert) to 45% slower (histogram and dump) from then on.  A request
// takes the smallest cached block at most 1/8 larger.  A freed block may still
// be in use by work queued on the context's stream; it is only handed out
// again to work queued on that same stream, after it.  Blocks cached by all
// contexts of the process are capped at BIG_CACHE_MAX; past it a context
// frees its least recently freed blocks first.
constexpr size_t BIG_BLOCK = 256ull << 20;
static std::atomic<size_t> g_big_cached{0};

// 128 GB, or TRINKMER_BLOCK_CACHE_GB (several processes sharing one GPU, such
// as two coverage-statistics runs side by side, each keep their own cache)
static size_t big_cache_max() {
    static const size_t v = [] {
        const char *e = getenv("TRINKMER_BLOCK_CACHE_GB");
        return e ? (size_t)(strtod(e, nullptr) * (double)(1ull << 30)) : (size_t)(128ull << 30);
    }();
    return v;
}
#define BIG_CACHE_MAX big_cache_max()

uint64_t ctx_cached_bytes(const tk_ctx *c) {
    uint64_t n = 0;
    for (auto &b : c->big_free) n += b.second;
    return n;
}

static void big_release(tk_ctx *c) {
    if (c->big_free.empty()) return;
    cudaStreamSynchronize(c->stream);
    if (c->copy_stream) cudaStreamSynchronize(c->copy_stream);
    for (auto &b : c->big_free) {
        cudaFree(b.first);
        g_big_cached -= b.second;
    }
    c->big_free.clear();
}

static int alloc_error(tk_ctx *c, cudaError_t e, size_t bytes, const char *what) {
    cudaGetLastError();
    return set_err(c, e == cudaErrorMemoryAllocation ? TK_E_OOM : TK_E_CUDA,
                   std::string("device allocation of ") + std::to_string(bytes) + " bytes for " + what + ": " +
                       cudaGetErrorString(e));
}

int dmalloc(tk_ctx *c, void **p, size_t bytes, const char *what) {
    *p = nullptr;
    if (bytes >= BIG_BLOCK) {
        int best = -1;
        for (size_t i = 0; i < c->big_free.size(); i++) {
            const size_t sz = c->big_free[i].second;
            if (sz >= bytes && sz - bytes <= bytes / 8 && (best < 0 || sz < c->big_free[best].second)) best = (int)i;
        }
        if (best >= 0) {
            *p = c->big_free[best].first;
            const size_t sz = c->big_free[best].second;
            c->big_free.erase(c->big_free.begin() + best);
            g_big_cached -= sz;
            c->big_used[*p] = sz;
            return TK_OK;
        }
        cudaError_t e = cudaMalloc(p, bytes);
        if (e == cudaErrorMemoryAllocation) {
            // give back what this context caches and what the pool holds, then retry
            cudaGetLastError();
            big_release(c);
            cudaStreamSynchronize(c->stream);
            cudaMemPool_t pool;
            if (cudaDeviceGetDefaultMemPool(&pool, c->device) == cudaSuccess) cudaMemPoolTrimTo(pool, 0);
            e = cudaMalloc(p, bytes);
        }
        if (e != cudaSuccess) {
            *p = nullptr;
            return alloc_error(c, e, bytes, what);
        }
        c->big_used[*p] = bytes;
        return TK_OK;
    }
    cudaError_t e = cudaMallocAsync(p, bytes ? bytes : 16, c->stream);
    if (e != cudaSuccess) {
        *p = nullptr;
        return alloc_error(c, e, bytes, what);
    }
    return TK_OK;
}

void dfree(tk_ctx *c, void *p) {
    if (!p) return;
    auto it = c->big_used.find(p);
    if (it == c->big_used.end()) {
        cudaFreeAsync(p, c->stream);
        return;
    }
    const size_t sz = it->second;
    c->big_used.erase(it);
    if (sz > BIG_CACHE_MAX || g_big_cached + sz > BIG_CACHE_MAX) {
        // over the cap: give back this context's least recently freed blocks
        // (or this one, if it alone is too big) once the queued work is done
        cudaStreamSynchronize(c->stream);
        if (c->copy_stream) cudaStreamSynchronize(c->copy_stream);
        if (sz > BIG_CACHE_MAX) {
            cudaFree(p);
            return;
        }
        size_t drop = 0;
        while (drop < c->big_free.size() && g_big_cached + sz > BIG_CACHE_MAX) {
            cudaFree(c->big_free[drop].first);
            g_big_cached -= c->big_free[drop].second;
            drop++;
        }
        c->big_free.erase(c->big_free.begin(), c->big_free.begin() + drop);
        if (g_big_cached + sz > BIG_CACHE_MAX) {   // the rest is cached by other contexts
            cudaFree(p);
            return;
        }
    }
    g_big_cached += sz;
    c->big_free.push_back({p, sz});
}

static cudaEvent_t take_event(tk_ctx *c) {
    if (!c->free_events.empty()) {
        cudaEvent_t e = c->free_events.back();
        c->free_events.pop_back();
        return e;
    }
    cudaEvent_t e = nullptr;
    cudaEventCreate(&e);
    return e;
}

void prof_begin(tk_ctx *c, int kid, cudaEvent_t *ev) {
    *ev = nullptr;
    if (!c->prof) return;
    *ev = take_event(c);
    cudaEventRecord(*ev, c->stream);
    if (kid >= 0 && kid < TK_KID_NUM) c->prof_open[kid] = c->launches;
}

void prof_end(tk_ctx *c, int kid, cudaEvent_t ev, uint64_t units) {
    if (!c->prof || !ev) return;
    cudaEvent_t b = take_event(c);
    cudaEventRecord(b, c->stream);
    const uint64_t n = (kid >= 0 && kid < TK_KID_NUM) ? c->launches - c->prof_open[kid] : 0;
    c->pending.push_back({ev, b, kid, units, n});
}

void prof_add_units(tk_ctx *c, int kid, uint64_t units) {
    if (c->prof && kid >= 0 && kid < TK_KID_NUM) c->prof_units[kid] += units;
}

static int prof_fold(tk_ctx *c) {
    if (c->pending.empty()) return TK_OK;
    TK_CUDA(c, cudaStreamSynchronize(c->stream));
    for (auto &p : c->pending) {
        float ms = 0;
        cudaEventElapsedTime(&ms, p.a, p.b);
        c->prof_ms[p.kid] += ms;
        c->prof_launches[p.kid] += p.launches;
        c->prof_units[p.kid] += p.units;
        c->free_events.push_back(p.a);
        c->free_events.push_back(p.b);
    }
    c->pending.clear();
    return TK_OK;
}

// copies a caller buffer to a fresh device allocation (or aliases a device one)
static int stage_in(tk_ctx *c, const void *src, uint64_t bytes, int where, void **dst, bool *owned) {
    if (where == TK_DEVICE) {
        *dst = const_cast<void *>(src);
        *owned = false;
        return TK_OK;
    }
    TK_TRY(dmalloc(c, dst, bytes + 64, "staged input"));
    *owned = true;
    if (bytes) TK_CUDA(c, cudaMemcpyAsync(*dst, src, bytes, cudaMemcpyHostToDevice, c->stream));
    return TK_OK;
}

// Random-access ceiling probe: independent random 8-byte accesses to the key
// words of a table of 16-byte slots (loads, or CAS + red.add as the count
// insert does), four in flight per thread.  Every index is masked into the
// table, so the probe stays in bounds for any size.
__global__ void k_random_probe(unsigned long long *tab, uint64_t mask, uint64_t n_access, int atomics,
                               unsigned long long *sink) {
    const uint64_t tid = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x, nth = (uint64_t)gridDim.x * blockDim.x;
    uint64_t acc = 0;
    for (uint64_t i = tid * 4; i < n_access; i += nth * 4) {
        unsigned long long v[4];
#pragma unroll
        for (int j = 0; j < 4; j++) {
            unsigned long long *p = tab + 2 * (mix64(i + j) & mask);
            if (atomics) {
                v[j] = atomicCAS(p, 0xFFFFFFFFFFFFFFFEULL, 0ULL);
                atomicAdd(reinterpret_cast<unsigned int *>(p + 1), 1u);
            } else {
                v[j] = __ldcg(p);
            }
        }
#pragma unroll
        for (int j = 0; j < 4; j++) acc += v[j];
    }
    if (acc == 0x123456789ULL) sink[0] = acc;
}

// drops the cached dump text once the table's contents change
// the context's copy stream, created on first use
static cudaStream_t copy_stream(tk_ctx *c) {
    if (!c->copy_stream && cudaStreamCreateWithFlags(&c->copy_stream, cudaStreamNonBlocking) != cudaSuccess) {
        c->copy_stream = nullptr;
        cudaGetLastError();
    }
    return c->copy_stream;
}

static void dump_invalidate(tk_table *t) {
    if (t->dump_copy_done) {
        // the device text is freed in stream order after its host copy ends
        cudaStreamWaitEvent(t->ctx->stream, t->dump_copy_done, 0);
        cudaEventDestroy(t->dump_copy_done);
        t->dump_copy_done = nullptr;
    }
    if (t->d_dump) dfree(t->ctx, t->d_dump);
    t->d_dump = nullptr;
    t->dump_len = 0;
    t->dump_valid = false;
}

// the table's contents change: its dump text and coverage cache are stale
static void table_changed(tk_table *t) {
    dump_invalidate(t);
    t->hot_valid = false;
}

}  // namespace tk

using namespace tk;

#define CHECK_CTX(c) do { if (!(c)) return TK_E_INVAL; if (cudaSetDevice((c)->device) != cudaSuccess) return set_err((c), TK_E_CUDA, "cudaSetDevice"); } while (0)

extern "C" {

const char *tk_version(void) { return "trinkmer-gb300 0.1 (sm_103a)"; }

const char *tk_status_string(int s) {
    switch (s) {
    case TK_OK: return "ok";
    case TK_E_INVAL: return "invalid argument";
    case TK_E_CUDA: return "CUDA error";
    case TK_E_OOM: return "out of memory";
    case TK_E_PARSE: return "malformed input";
    case TK_E_TABLE_FULL: return "hash table full";
    case TK_E_BUDGET: return "over the HBM admission budget";
    case TK_E_NODEV: return "no CUDA device";
    case TK_E_RANGE: return "buffer too small";
    default: return "unknown status";
    }
}

int tk_ctx_create(int device, tk_ctx **out) {
    if (!out) return TK_E_INVAL;
    *out = nullptr;
    int n = 0;
    if (cudaGetDeviceCount(&n) != cudaSuccess || n <= 0) {
        cudaGetLastError();
        return TK_E_NODEV;
    }
    if (device < 0 || device >= n) return TK_E_INVAL;
    if (cudaSetDevice(device) != cudaSuccess) return TK_E_CUDA;
    tk_ctx *c = new (std::nothrow) tk_ctx();
    if (!c) return TK_E_OOM;
    c->device = device;
    cudaDeviceGetAttribute(&c->sm_count, cudaDevAttrMultiProcessorCount, device);
    if (cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking) != cudaSuccess) {
        delete c;
        return TK_E_CUDA;
    }
    c->own_stream = true;
    // keep freed blocks in the stream-ordered pool: the hot path allocates per call
    cudaMemPool_t pool;
    if (cudaDeviceGetDefaultMemPool(&pool, device) == cudaSuccess) {
        uint64_t thr = UINT64_MAX;
        cudaMemPoolSetAttribute(pool, cudaMemPoolAttrReleaseThreshold, &thr);
    }
    if (cudaMalloc(&c->d_err, DE_COUNT * sizeof(uint32_t)) != cudaSuccess) {
        cudaStreamDestroy(c->stream);
        delete c;
        return TK_E_OOM;
    }
    cudaMemset(c->d_err, 0, DE_COUNT * sizeof(uint32_t));
    *out = c;
    return TK_OK;
}

static void ctx_release_now(tk_ctx *c);

// a child handle (read set, table, bundle) starts / stops using the context
static void ctx_acquire(tk_ctx *c) { c->live.fetch_add(1); }
static void ctx_release(tk_ctx *c) {
    if (c->live.fetch_sub(1) == 1 && c->closing.load()) ctx_release_now(c);
}

void tk_ctx_destroy(tk_ctx *c) {
    if (!c) return;
    c->closing.store(true);
    if (c->live.load() == 0) ctx_release_now(c);
}

static void ctx_release_now(tk_ctx *c) {
    cudaSetDevice(c->device);
    cudaStreamSynchronize(c->stream);
    big_release(c);
    for (auto &b : c->big_used) cudaFree(b.first);   // none once every handle is freed
    c->big_used.clear();
    if (c->copy_stream) {
        cudaStreamSynchronize(c->copy_stream);
        cudaStreamDestroy(c->copy_stream);
    }
    for (auto &p : c->pending) { cudaEventDestroy(p.a); cudaEventDestroy(p.b); }
    for (auto e : c->free_events) cudaEventDestroy(e);
    if (c->bins_exec) cudaGraphExecDestroy(c->bins_exec);
    cudaFree(c->d_err);
    if (c->own_stream) cudaStreamDestroy(c->stream);
    cudaMemPool_t pool;
    if (cudaDeviceGetDefaultMemPool(&pool, c->device) == cudaSuccess) cudaMemPoolTrimTo(pool, 0);
    delete c;
}

const char *tk_ctx_last_error(const tk_ctx *c) { return c ? c->last_error.c_str() : "no context"; }

void *tk_ctx_stream(tk_ctx *c) { return c ? (void *)c->stream : nullptr; }

int tk_ctx_synchronize(tk_ctx *c) {
    CHECK_CTX(c);
    if (c->copy_stream) TK_CUDA(c, cudaStreamSynchronize(c->copy_stream));
    return cuda_check(c, cudaStreamSynchronize(c->stream), "synchronize");
}

int tk_ctx_set_profiling(tk_ctx *c, int on) {
    CHECK_CTX(c);
    TK_TRY(prof_fold(c));
    c->prof = on != 0;
    return TK_OK;
}

int tk_ctx_profile(tk_ctx *c, int kid, double *ms, uint64_t *launches, uint64_t *units) {
    CHECK_CTX(c);
    if (kid < 0 || kid >= TK_KID_NUM) return TK_E_INVAL;
    TK_TRY(prof_fold(c));
    if (ms) *ms = c->prof_ms[kid];
    if (launches) *launches = c->prof_launches[kid];
    if (units) *units = c->prof_units[kid];
    return TK_OK;
}

int tk_ctx_reset_profile(tk_ctx *c) {
    CHECK_CTX(c);
    TK_TRY(prof_fold(c));
    for (int i = 0; i < TK_KID_NUM; i++) { c->prof_ms[i] = 0; c->prof_launches[i] = 0; c->prof_units[i] = 0; }
    return TK_OK;
}

uint64_t tk_ctx_kernel_launches(const tk_ctx *c) { return c ? c->launches : 0; }

int tk_ctx_set_reprobes(tk_ctx *c, int max_probes) {
    CHECK_CTX(c);
    if (max_probes < 1) return TK_E_INVAL;
    c->max_probes = max_probes;
    return TK_OK;
}

int tk_ctx_random_access_rate(tk_ctx *c, uint64_t table_bytes, int atomics, double *accesses_per_s) {
    CHECK_CTX(c);
    if (!accesses_per_s || table_bytes < 4096) return TK_E_INVAL;
    uint64_t slots = 1;
    while (slots * 2 * 16 <= table_bytes) slots <<= 1;
    unsigned long long *tab = nullptr, *sink = nullptr;
    TK_TRY(dmalloc(c, (void **)&tab, slots * 16, "probe table"));
    int e = dmalloc(c, (void **)&sink, 8, "probe sink");
    const uint64_t n = 1ULL << 27;
    const unsigned grid = (unsigned)c->sm_count * 8;
    cudaEvent_t a = nullptr, b = nullptr;
    if (!e) {
        cudaMemsetAsync(tab, 0, slots * 16, c->stream);
        cudaEventCreate(&a);
        cudaEventCreate(&b);
        k_random_probe<<<grid, 256, 0, c->stream>>>(tab, slots - 1, n, atomics, sink);   // warm-up
        cudaEventRecord(a, c->stream);
        for (int r = 0; r < 3; r++) k_random_probe<<<grid, 256, 0, c->stream>>>(tab, slots - 1, n, atomics, sink);
        cudaEventRecord(b, c->stream);
        c->launches += 4;
        e = cuda_check(c, cudaEventSynchronize(b), "probe sync");
    }
    if (!e) {
        float ms = 0;
        cudaEventElapsedTime(&ms, a, b);
        *accesses_per_s = 3.0 * (double)n / (ms / 1e3);
    }
    if (a) cudaEventDestroy(a);
    if (b) cudaEventDestroy(b);
    dfree(c, tab);
    if (sink) dfree(c, sink);
    return e;
}

int tk_ctx_trim(tk_ctx *c) {
    CHECK_CTX(c);
    big_release(c);
    cudaMemPool_t pool;
    if (cudaDeviceGetDefaultMemPool(&pool, c->device) == cudaSuccess) {
        TK_CUDA(c, cudaStreamSynchronize(c->stream));
        cudaMemPoolTrimTo(pool, 0);
    }
    return TK_OK;
}

int tk_ctx_mem_info(tk_ctx *c, uint64_t *free_bytes, uint64_t *total_bytes) {
    CHECK_CTX(c);
    size_t f = 0, t = 0;
    TK_CUDA(c, cudaMemGetInfo(&f, &t));
    if (free_bytes) *free_bytes = f;
    if (total_bytes) *total_bytes = t;
    return TK_OK;
}

// ------------------------------------------------------------------ reads

int tk_reads_parse(tk_ctx *c, const char *text, uint64_t len, int where, tk_reads **out) {
    CHECK_CTX(c);
    if (!out || (!text && len)) return set_err(c, TK_E_INVAL, "tk_reads_parse: null text");
    *out = nullptr;
    tk_reads *r = new (std::nothrow) tk_reads();
    if (!r) return TK_E_OOM;
    r->ctx = c;
    ctx_acquire(c);
    r->text_len = len;
    void *d = nullptr;
    bool owned = false;
    int e = stage_in(c, text, len, where, &d, &owned);
    r->d_text = (char *)d;
    r->own_text = owned;
    if (!e) e = parse_reads(c, r);
    if (e) {
        tk_reads_free(r);
        return e;
    }
    *out = r;
    return TK_OK;
}

}  // extern "C"

// Parses n texts; `after(i, reads)` runs on each read set as soon as it is
// parsed, while the later host texts are still uploading.
template <typename After>
static int parse_many_then(tk_ctx *c, const char *const *texts, const uint64_t *lens, uint32_t n, int where,
                           tk_reads **out, After &&after) {
    cudaStream_t cs = where == TK_HOST ? copy_stream(c) : nullptr;
    if (!cs) {
        // device texts (or no copy stream): one after another
        for (uint32_t i = 0; i < n; i++) {
            int e = tk_reads_parse(c, texts[i], lens[i], where, &out[i]);
            if (!e) e = after(i, out[i]);
            if (e) {
                for (uint32_t j = 0; j <= i; j++) { tk_reads_free(out[j]); out[j] = nullptr; }
                return e;
            }
        }
        return TK_OK;
    }
    // every upload is queued on the copy stream up front; text i is parsed on
    // the main stream as soon as its own upload has landed, while the later
    // ones are still in flight
    std::vector<char *> dev(n, nullptr);
    std::vector<cudaEvent_t> landed(n, nullptr);
    int e = TK_OK;
    for (uint32_t i = 0; i < n && !e; i++) e = dmalloc(c, (void **)&dev[i], lens[i] + 64, "staged input");
    cudaEvent_t allocated = nullptr;
    if (!e) e = cuda_check(c, cudaEventCreateWithFlags(&allocated, cudaEventDisableTiming), "event");
    if (!e) e = cuda_check(c, cudaEventRecord(allocated, c->stream), "event record");
    if (!e) e = cuda_check(c, cudaStreamWaitEvent(cs, allocated, 0), "copy stream wait");
    for (uint32_t i = 0; i < n && !e; i++) {
        e = cuda_check(c, cudaEventCreateWithFlags(&landed[i], cudaEventDisableTiming), "event");
        if (!e && lens[i]) e = cuda_check(c, cudaMemcpyAsync(dev[i], texts[i], lens[i], cudaMemcpyHostToDevice, cs), "h2d");
        if (!e) e = cuda_check(c, cudaEventRecord(landed[i], cs), "event record");
    }
    uint32_t made = 0;
    for (uint32_t i = 0; i < n && !e; i++) {
        e = cuda_check(c, cudaStreamWaitEvent(c->stream, landed[i], 0), "parse wait");
        if (e) break;
        tk_reads *r = new (std::nothrow) tk_reads();
        if (!r) {
            e = TK_E_OOM;
            break;
        }
        r->ctx = c;
        ctx_acquire(c);
        r->text_len = lens[i];
        r->d_text = dev[i];
        r->own_text = true;
        dev[i] = nullptr;
        out[i] = r;
        made = i + 1;
        e = parse_reads(c, r);
        if (!e) e = after(i, r);
    }
    if (e) {
        cudaStreamSynchronize(cs);
        for (uint32_t j = 0; j < made; j++) { tk_reads_free(out[j]); out[j] = nullptr; }
    }
    for (uint32_t i = 0; i < n; i++) {
        if (dev[i]) {
            if (landed[i] || allocated) cudaStreamWaitEvent(c->stream, landed[i] ? landed[i] : allocated, 0);
            dfree(c, dev[i]);
        }
        if (landed[i]) cudaEventDestroy(landed[i]);
    }
    if (allocated) cudaEventDestroy(allocated);
    return e;
}

extern "C" {

int tk_reads_parse_many(tk_ctx *c, const char *const *texts, const uint64_t *lens, uint32_t n, int where,
                        tk_reads **out) {
    CHECK_CTX(c);
    if (!out || (!texts && n) || (!lens && n)) return set_err(c, TK_E_INVAL, "tk_reads_parse_many: null argument");
    for (uint32_t i = 0; i < n; i++) {
        out[i] = nullptr;
        if (!texts[i] && lens[i]) return set_err(c, TK_E_INVAL, "tk_reads_parse_many: null text");
    }
    return parse_many_then(c, texts, lens, n, where, out, [](uint32_t, tk_reads *) { return TK_OK; });
}

int tk_table_count_texts(tk_table *t, const char *const *texts, const uint64_t *lens, uint32_t n, int where,
                         tk_reads **out) {
    if (!t) return TK_E_INVAL;
    tk_ctx *c = t->ctx;
    CHECK_CTX(c);
    if (!out || (!texts && n) || (!lens && n)) return set_err(c, TK_E_INVAL, "tk_table_count_texts: null argument");
    for (uint32_t i = 0; i < n; i++) {
        out[i] = nullptr;
        if (!texts[i] && lens[i]) return set_err(c, TK_E_INVAL, "tk_table_count_texts: null text");
    }
    if (n > COUNT_MAX_SETS) {
        // more texts than one counting pass takes: parse, then count in groups
        TK_TRY(tk_reads_parse_many(c, texts, lens, n, where, out));
        int e = tk_table_add_reads_multi(t, out, n);
        if (e)
            for (uint32_t i = 0; i < n; i++) { tk_reads_free(out[i]); out[i] = nullptr; }
        return e;
    }
    table_changed(t);
    TK_TRY(table_count_begin(t));
    std::vector<BucketKeys> bk(n);
    int e = parse_many_then(c, texts, lens, n, where, out,
                            [&](uint32_t i, tk_reads *r) { return table_bucket_pass(t, r, &bk[i]); });
    if (!e) e = table_count_buckets(t, bk);
    if (e) {
        for (BucketKeys &b : bk) table_bucket_free(t, &b);
        for (uint32_t i = 0; i < n; i++) { tk_reads_free(out[i]); out[i] = nullptr; }
    }
    return e;
}

// ---- record-aligned split of a host text (host code only)

// true when a FASTQ record starts at p (p is a line start holding '@'): the
// line after its sequence line starts with '+'.  A quality line that starts
// with '@' is followed by a header and a sequence line, so it fails the test.
static bool fastq_record_at(const char *t, uint64_t len, uint64_t p) {
    const void *e1 = std::memchr(t + p, '\n', len - p);
    if (!e1) return false;
    const uint64_t s2 = (uint64_t)((const char *)e1 - t) + 1;
    if (s2 >= len) return false;
    const void *e2 = std::memchr(t + s2, '\n', len - s2);
    if (!e2) return false;
    const uint64_t s3 = (uint64_t)((const char *)e2 - t) + 1;
    return s3 < len && t[s3] == '+';
}

int tk_split_records(const char *text, uint64_t len, uint32_t n_chunks, uint64_t *cuts) {
    if (!cuts || n_chunks == 0 || (!text && len)) return TK_E_INVAL;
    uint64_t first = 0;
    while (first < len && std::isspace((unsigned char)text[first])) first++;
    const char mark = first < len && text[first] == '@' ? '@' : '>';
    cuts[0] = 0;
    uint64_t prev = 0;
    for (uint32_t i = 1; i < n_chunks; i++) {
        uint64_t p = std::max<uint64_t>(prev, len / n_chunks * i);
        uint64_t cut = len;
        while (p < len) {
            // the next line start at or after p
            if (p > 0 && text[p - 1] != '\n') {
                const void *nl = std::memchr(text + p, '\n', len - p);
                if (!nl) break;
                p = (uint64_t)((const char *)nl - text) + 1;
                continue;
            }
            if (p > first && text[p] == mark && (mark == '>' || fastq_record_at(text, len, p))) {
                cut = p;
                break;
            }
            const void *nl = std::memchr(text + p, '\n', len - p);
            if (!nl) break;
            p = (uint64_t)((const char *)nl - text) + 1;
        }
        cuts[i] = prev = cut;
    }
    cuts[n_chunks] = len;
    return TK_OK;
}

int tk_reads_to_fasta(tk_reads *r, int append, int flags, int where, char *out, uint64_t cap, uint64_t *len_out) {
    if (!r || !len_out) return TK_E_INVAL;
    tk_ctx *c = r->ctx;
    CHECK_CTX(c);
    if (r->format != TK_FMT_FASTQ && r->n_reads)
        return set_err(c, TK_E_INVAL, "tk_reads_to_fasta: the read set was not parsed from FASTQ");
    if (flags & ~(TK_FA_REVCOMP | TK_FA_IGNORE_DIRTY | TK_FA_IF_MISSING))
        return set_err(c, TK_E_INVAL, "tk_reads_to_fasta: unknown flag");
    if (append < -1) return set_err(c, TK_E_INVAL, "tk_reads_to_fasta: append must be -1 (none) or >= 0");
    if (!r->d_fasta || r->fasta_append != append || r->fasta_flags != flags) {
        if (r->d_fasta) dfree(c, r->d_fasta);
        r->d_fasta = nullptr;
        r->fasta_flags = -1;
        TK_TRY(reads_fasta(r, append, flags, &r->d_fasta, &r->fasta_len));
        r->fasta_append = append;
        r->fasta_flags = flags;
    }
    *len_out = r->fasta_len;
    if (!out) return TK_OK;
    if (cap < r->fasta_len) return set_err(c, TK_E_RANGE, "tk_reads_to_fasta: buffer smaller than the text");
    if (r->fasta_len)
        TK_CUDA(c, cudaMemcpyAsync(out, r->d_fasta, r->fasta_len,
                                   where == TK_DEVICE ? cudaMemcpyDeviceToDevice : cudaMemcpyDeviceToHost, c->stream));
    return cuda_check(c, cudaStreamSynchronize(c->stream), "fasta copy");
}

int tk_reads_info(const tk_reads *r, uint64_t *n_reads, uint64_t *n_bases, uint32_t *max_len, int *format) {
    if (!r) return TK_E_INVAL;
    if (n_reads) *n_reads = r->n_reads;
    if (n_bases) *n_bases = r->n_bases;
    if (max_len) *max_len = r->max_len;
    if (format) *format = r->format;
    return TK_OK;
}

int tk_reads_names(const tk_reads *r, uint64_t *name_off, uint32_t *name_len) {
    if (!r) return TK_E_INVAL;
    tk_ctx *c = r->ctx;
    CHECK_CTX(c);
    if (r->n_reads == 0) return TK_OK;
    if (name_off) TK_CUDA(c, cudaMemcpyAsync(name_off, r->d_name_off, r->n_reads * 8, cudaMemcpyDeviceToHost, c->stream));
    if (name_len) TK_CUDA(c, cudaMemcpyAsync(name_len, r->d_name_len, r->n_reads * 4, cudaMemcpyDeviceToHost, c->stream));
    return cuda_check(c, cudaStreamSynchronize(c->stream), "names sync");
}

int tk_reads_offsets(const tk_reads *r, uint64_t *rd_off) {
    if (!r || !rd_off) return TK_E_INVAL;
    tk_ctx *c = r->ctx;
    CHECK_CTX(c);
    TK_CUDA(c, cudaMemcpyAsync(rd_off, r->d_rd_off, (r->n_reads + 1) * 8, cudaMemcpyDeviceToHost, c->stream));
    return cuda_check(c, cudaStreamSynchronize(c->stream), "offsets sync");
}

int tk_reads_copy_seq(const tk_reads *r, char *dst, uint64_t cap) {
    if (!r || (!dst && r->seq_len)) return TK_E_INVAL;
    tk_ctx *c = r->ctx;
    CHECK_CTX(c);
    if (cap < r->seq_len) return set_err(c, TK_E_RANGE, "tk_reads_copy_seq: buffer smaller than the packed reads");
    if (r->seq_len) TK_CUDA(c, cudaMemcpyAsync(dst, r->d_seq, r->seq_len, cudaMemcpyDeviceToHost, c->stream));
    return cuda_check(c, cudaStreamSynchronize(c->stream), "seq sync");
}

void tk_reads_free(tk_reads *r) {
    if (!r) return;
    tk_ctx *c = r->ctx;
    cudaSetDevice(c->device);
    if (r->own_text) dfree(c, r->d_text);
    dfree(c, r->d_seq_alloc);
    if (r->d_pack_alloc) dfree(c, r->d_pack_alloc);
    if (r->d_fasta) dfree(c, r->d_fasta);
    dfree(c, r->d_rd_off);
    dfree(c, r->d_name_off);
    dfree(c, r->d_name_len);
    delete r;
    ctx_release(c);
}

// ------------------------------------------------------------------ table

static int table_new(tk_ctx *c, int k, int canonical, tk_table **out) {
    tk_table *t = new (std::nothrow) tk_table();
    if (!t) return TK_E_OOM;
    t->ctx = c;
    ctx_acquire(c);
    t->k = k;
    t->canonical = canonical ? 1 : 0;
    t->ovf_cap = 1 << 20;
    int e = dmalloc(c, (void **)&t->d_ovf, t->ovf_cap * 12, "overflow list");
    if (!e) e = dmalloc(c, (void **)&t->d_counters, 2 * sizeof(unsigned long long), "table counters");
    if (!e) e = dmalloc(c, (void **)&t->d_hll, 4096 * 4, "HLL registers");
    if (!e) {
        cudaMemsetAsync(t->d_counters, 0, 2 * sizeof(unsigned long long), c->stream);
        cudaMemsetAsync(t->d_hll, 0, 4096 * 4, c->stream);
    }
    if (e) {
        tk_table_free(t);
        return e;
    }
    *out = t;
    return TK_OK;
}

int tk_table_create(tk_ctx *c, int k, int canonical, uint64_t capacity_hint, tk_table **out) {
    CHECK_CTX(c);
    if (!out) return TK_E_INVAL;
    *out = nullptr;
    if (k < 1 || k > MAX_K) return set_err(c, TK_E_INVAL, "k must be in 1..31");
    tk_table *t = nullptr;
    TK_TRY(table_new(c, k, canonical, &t));
    if (capacity_hint) {
        uint64_t cap = 1024;
        while (cap < capacity_hint) cap <<= 1;
        int e = table_alloc(t, cap);
        if (e) {
            tk_table_free(t);
            return e;
        }
    }
    *out = t;
    return TK_OK;
}

int tk_table_add_reads(tk_table *t, const tk_reads *r) {
    if (!t || !r) return TK_E_INVAL;
    tk_ctx *c = t->ctx;
    CHECK_CTX(c);
    if (r->ctx != c) return set_err(c, TK_E_INVAL, "read set and table belong to different contexts");
    table_changed(t);
    return table_count_seq(t, r);
}

int tk_table_add_reads_multi(tk_table *t, const tk_reads *const *sets, uint32_t n_sets) {
    if (!t || (!sets && n_sets)) return TK_E_INVAL;
    tk_ctx *c = t->ctx;
    CHECK_CTX(c);
    for (uint32_t i = 0; i < n_sets; i++) {
        if (!sets[i]) return set_err(c, TK_E_INVAL, "tk_table_add_reads_multi: null read set");
        if (sets[i]->ctx != c) return set_err(c, TK_E_INVAL, "read set and table belong to different contexts");
    }
    table_changed(t);
    return table_count_many(t, sets, (int)n_sets);
}

int tk_table_count_text(tk_table *t, const char *text, uint64_t len, int where) {
    if (!t) return TK_E_INVAL;
    tk_reads *r = nullptr;
    TK_TRY(tk_reads_parse(t->ctx, text, len, where, &r));
    int e = tk_table_add_reads(t, r);
    tk_reads_free(r);
    return e;
}

int tk_table_info(tk_table *t, uint64_t *distinct, uint64_t *total, uint64_t *capacity) {
    if (!t) return TK_E_INVAL;
    CHECK_CTX(t->ctx);
    return table_info(t, distinct, total, capacity);
}

int tk_table_histo(tk_table *t, uint64_t low, uint64_t high, uint64_t *hist) {
    if (!t || !hist) return TK_E_INVAL;
    CHECK_CTX(t->ctx);
    return table_histo(t, low, high, hist);
}

int tk_table_dump(tk_table *t, uint32_t min_count, int where, uint64_t *keys, uint32_t *counts, uint64_t cap,
                  uint64_t *n_out) {
    if (!t || !n_out) return TK_E_INVAL;
    tk_ctx *c = t->ctx;
    CHECK_CTX(c);
    uint64_t *dk = nullptr;
    uint32_t *dc = nullptr;
    uint64_t n = 0;
    TK_TRY(table_sorted_pairs(t, min_count, &dk, &dc, &n));
    *n_out = n;
    int e = TK_OK;
    if (keys || counts) {
        if (cap < n) e = set_err(c, TK_E_RANGE, "tk_table_dump: capacity below the number of pairs");
        cudaMemcpyKind kind = where == TK_DEVICE ? cudaMemcpyDeviceToDevice : cudaMemcpyDeviceToHost;
        if (!e && keys && n) e = cuda_check(c, cudaMemcpyAsync(keys, dk, n * 8, kind, c->stream), "dump keys");
        if (!e && counts && n) e = cuda_check(c, cudaMemcpyAsync(counts, dc, n * 4, kind, c->stream), "dump counts");
    }
    dfree(c, dk);
    dfree(c, dc);
    if (!e) e = cuda_check(c, cudaStreamSynchronize(c->stream), "dump sync");
    return e;
}

// builds (or reuses) the device text of the dump at min_count
static int dump_build(tk_table *t, uint32_t min_count) {
    tk_ctx *c = t->ctx;
    if (!t->dump_valid || t->dump_min != min_count) {
        dump_invalidate(t);
        uint64_t *dk = nullptr;
        uint32_t *dc = nullptr;
        uint64_t n = 0;
        TK_TRY(table_sorted_pairs(t, min_count, &dk, &dc, &n));
        char *text = nullptr;
        uint64_t len = 0;
        int e = format_dump(c, dk, dc, n, t->k, &text, &len);
        dfree(c, dk);
        dfree(c, dc);
        if (e) return e;
        t->d_dump = text;
        t->dump_len = len;
        t->dump_min = min_count;
        t->dump_valid = true;
    }
    return TK_OK;
}

int tk_table_dump_fasta(tk_table *t, uint32_t min_count, int where, char *out, uint64_t cap, uint64_t *len_out) {
    if (!t || !len_out) return TK_E_INVAL;
    tk_ctx *c = t->ctx;
    CHECK_CTX(c);
    TK_TRY(dump_build(t, min_count));
    *len_out = t->dump_len;
    int e = TK_OK;
    if (out) {
        cudaMemcpyKind kind = where == TK_DEVICE ? cudaMemcpyDeviceToDevice : cudaMemcpyDeviceToHost;
        if (cap < t->dump_len) e = set_err(c, TK_E_RANGE, "tk_table_dump_fasta: buffer smaller than the dump");
        else if (t->dump_len)
            e = cuda_check(c, cudaMemcpyAsync(out, t->d_dump, t->dump_len, kind, c->stream), "dump text copy");
    }
    if (!e) e = cuda_check(c, cudaStreamSynchronize(c->stream), "dump text sync");
    return e;
}

int tk_table_dump_fasta_async(tk_table *t, uint32_t min_count, char *out, uint64_t cap, uint64_t *len_out) {
    if (!t || !len_out) return TK_E_INVAL;
    tk_ctx *c = t->ctx;
    CHECK_CTX(c);
    TK_TRY(dump_build(t, min_count));
    *len_out = t->dump_len;
    if (!out) return TK_OK;
    if (cap < t->dump_len) return set_err(c, TK_E_RANGE, "tk_table_dump_fasta_async: buffer smaller than the dump");
    if (!t->dump_len) return TK_OK;
    cudaStream_t cs = copy_stream(c);
    if (!cs) return tk_table_dump_fasta(t, min_count, TK_HOST, out, cap, len_out);
    cudaEvent_t built = nullptr;
    TK_CUDA(c, cudaEventCreateWithFlags(&built, cudaEventDisableTiming));
    int e = cuda_check(c, cudaEventRecord(built, c->stream), "event record");
    if (!e) e = cuda_check(c, cudaStreamWaitEvent(cs, built, 0), "copy stream wait");
    cudaEventDestroy(built);
    if (!e) e = cuda_check(c, cudaMemcpyAsync(out, t->d_dump, t->dump_len, cudaMemcpyDeviceToHost, cs), "dump d2h");
    if (!e && !t->dump_copy_done) e = cuda_check(c, cudaEventCreateWithFlags(&t->dump_copy_done, cudaEventDisableTiming), "event");
    if (!e) e = cuda_check(c, cudaEventRecord(t->dump_copy_done, cs), "event record");
    return e;
}

int tk_table_load_pairs(tk_table *t, const uint64_t *keys, const uint32_t *counts, uint64_t n, int where) {
    if (!t || (!keys && n)) return TK_E_INVAL;
    tk_ctx *c = t->ctx;
    CHECK_CTX(c);
    if (n == 0) return TK_OK;
    table_changed(t);
    void *dk = nullptr, *dc = nullptr;
    bool ok_k = false, ok_c = false;
    int e = stage_in(c, keys, n * 8, where, &dk, &ok_k);
    if (!e && counts) e = stage_in(c, counts, n * 4, where, &dc, &ok_c);
    if (!e) e = table_insert_pairs(t, (const uint64_t *)dk, (const uint32_t *)dc, n);
    if (ok_k) dfree(c, dk);
    if (ok_c) dfree(c, dc);
    return e;
}

int tk_table_load_dump_fasta(tk_table *t, const char *text, uint64_t len, int where) {
    if (!t) return TK_E_INVAL;
    tk_ctx *c = t->ctx;
    CHECK_CTX(c);
    tk_reads *r = nullptr;
    TK_TRY(tk_reads_parse(c, text, len, where, &r));
    int e = TK_OK;
    if (r->format == TK_FMT_FASTQ) e = set_err(c, TK_E_PARSE, "k-mer catalogue must be FASTA ('>COUNT' headers)");
    table_changed(t);
    if (!e) e = table_load_dump_reads(t, r);
    tk_reads_free(r);
    return e;
}

void tk_table_free(tk_table *t) {
    if (!t) return;
    tk_ctx *c = t->ctx;
    cudaSetDevice(c->device);
    dfree(c, t->t.slots);
    dfree(c, t->d_ovf);
    dfree(c, t->d_counters);
    dfree(c, t->d_hll);
    dfree(c, t->d_hot);
    dump_invalidate(t);
    delete t;
    ctx_release(c);
}

// ------------------------------------------------------------------ coverage

int tk_coverage_stats(tk_table *t, const tk_reads *r, int where, uint32_t *median, float *mean, float *stdev) {
    if (!t || !r || !median || !mean || !stdev) return TK_E_INVAL;
    tk_ctx *c = t->ctx;
    CHECK_CTX(c);
    if (r->ctx != c) return set_err(c, TK_E_INVAL, "read set and table belong to different contexts");
    const uint64_t n = r->n_reads;
    if (n == 0) return TK_OK;
    if (where == TK_DEVICE) {
        TK_TRY(coverage_stats(t, r, median, mean, stdev));
        return cuda_check(c, cudaStreamSynchronize(c->stream), "coverage sync");
    }
    uint32_t *dm = nullptr;
    float *da = nullptr, *ds = nullptr;
    int e = dmalloc(c, (void **)&dm, n * 4, "median");
    if (!e) e = dmalloc(c, (void **)&da, n * 4, "mean");
    if (!e) e = dmalloc(c, (void **)&ds, n * 4, "stdev");
    if (!e) e = coverage_stats(t, r, dm, da, ds);
    if (!e) e = cuda_check(c, cudaMemcpyAsync(median, dm, n * 4, cudaMemcpyDeviceToHost, c->stream), "median d2h");
    if (!e) e = cuda_check(c, cudaMemcpyAsync(mean, da, n * 4, cudaMemcpyDeviceToHost, c->stream), "mean d2h");
    if (!e) e = cuda_check(c, cudaMemcpyAsync(stdev, ds, n * 4, cudaMemcpyDeviceToHost, c->stream), "stdev d2h");
    dfree(c, dm);
    dfree(c, da);
    dfree(c, ds);
    if (!e) e = cuda_check(c, cudaStreamSynchronize(c->stream), "coverage sync");
    return e;
}

// ------------------------------------------------------------------ R2T

// Component id of every bundle record: the integer after "s_" in its
// accession, else the record ordinal.
static int bundle_component_ids(tk_ctx *c, const tk_reads *b, const char *bundle, uint64_t len, int where,
                                std::vector<uint64_t> *ids) {
    ids->assign(b->n_reads, 0);
    std::vector<uint64_t> off(b->n_reads);
    std::vector<uint32_t> nl(b->n_reads);
    TK_TRY(tk_reads_names(b, off.data(), nl.data()));
    std::vector<char> host_text;
    const char *ht = bundle;
    if (where == TK_DEVICE) {
        host_text.resize(len);
        TK_CUDA(c, cudaMemcpy(host_text.data(), bundle, len, cudaMemcpyDeviceToHost));
        ht = host_text.data();
    }
    for (uint64_t i = 0; i < b->n_reads; i++) {
        const char *h = ht + off[i];
        const uint32_t L = nl[i];
        uint64_t id = i;
        if (L > 2 && h[0] == 's' && h[1] == '_' && h[2] >= '0' && h[2] <= '9') {
            id = 0;
            for (uint32_t j = 2; j < L && h[j] >= '0' && h[j] <= '9'; j++) id = id * 10 + (uint64_t)(h[j] - '0');
        }
        (*ids)[i] = id;
    }
    return TK_OK;
}

int tk_r2t_create(tk_ctx *c, const char *bundle, uint64_t len, int where, int k, int strand, tk_r2t **out) {
    CHECK_CTX(c);
    if (!out) return TK_E_INVAL;
    *out = nullptr;
    if (k < 1 || k > MAX_K) return set_err(c, TK_E_INVAL, "k must be in 1..31");
    tk_r2t *z = new (std::nothrow) tk_r2t();
    if (!z) return TK_E_OOM;
    z->ctx = c;
    ctx_acquire(c);
    z->k = k;
    z->strand = strand ? 1 : 0;
    tk_reads *b = nullptr;
    int e = table_new(c, k, !strand, &z->table);
    if (!e) e = tk_reads_parse(c, bundle, len, where, &b);
    if (!e && b->format == TK_FMT_FASTQ) e = set_err(c, TK_E_PARSE, "bundle must be FASTA");
    if (!e) e = r2t_build(z, b);
    if (!e) {
        z->n_records = b->n_reads;
        e = bundle_component_ids(c, b, bundle, len, where, &z->comp_id);
    }
    if (b) tk_reads_free(b);
    if (e) {
        tk_r2t_free(z);
        return e;
    }
    *out = z;
    return TK_OK;
}

int tk_r2t_info(const tk_r2t *z, uint64_t *n_records, uint64_t *n_kmers) {
    if (!z) return TK_E_INVAL;
    if (n_records) *n_records = z->n_records;
    if (n_kmers) {
        uint64_t d = 0;
        TK_TRY(table_info(z->table, &d, nullptr, nullptr));
        *n_kmers = d;
    }
    return TK_OK;
}

int tk_r2t_component_ids(const tk_r2t *z, uint64_t *ids) {
    if (!z || !ids) return TK_E_INVAL;
    std::copy(z->comp_id.begin(), z->comp_id.end(), ids);
    return TK_OK;
}

int tk_r2t_assign(tk_r2t *z, const tk_reads *r, int where, int32_t *rec, uint32_t *hits, uint32_t *nwin) {
    if (!z || !r || !rec || !hits || !nwin) return TK_E_INVAL;
    tk_ctx *c = z->ctx;
    CHECK_CTX(c);
    if (r->ctx != c) return set_err(c, TK_E_INVAL, "read set and bundle belong to different contexts");
    const uint64_t n = r->n_reads;
    if (n == 0) return TK_OK;
    if (where == TK_DEVICE) {
        TK_TRY(r2t_assign(z, r, rec, hits, nwin));
        return cuda_check(c, cudaStreamSynchronize(c->stream), "assign sync");
    }
    int32_t *dr = nullptr;
    uint32_t *dh = nullptr, *dn = nullptr;
    int e = dmalloc(c, (void **)&dr, n * 4, "rec");
    if (!e) e = dmalloc(c, (void **)&dh, n * 4, "hits");
    if (!e) e = dmalloc(c, (void **)&dn, n * 4, "nwin");
    if (!e) e = r2t_assign(z, r, dr, dh, dn);
    if (!e) e = cuda_check(c, cudaMemcpyAsync(rec, dr, n * 4, cudaMemcpyDeviceToHost, c->stream), "rec d2h");
    if (!e) e = cuda_check(c, cudaMemcpyAsync(hits, dh, n * 4, cudaMemcpyDeviceToHost, c->stream), "hits d2h");
    if (!e) e = cuda_check(c, cudaMemcpyAsync(nwin, dn, n * 4, cudaMemcpyDeviceToHost, c->stream), "nwin d2h");
    dfree(c, dr);
    dfree(c, dh);
    dfree(c, dn);
    if (!e) e = cuda_check(c, cudaStreamSynchronize(c->stream), "assign sync");
    return e;
}

void tk_r2t_free(tk_r2t *z) {
    if (!z) return;
    tk_ctx *c = z->ctx;
    if (z->table) tk_table_free(z->table);
    delete z;
    ctx_release(c);
}

// ------------------------------------------------------------------ de Bruijn graphs

static int norm_copy_out(tk_ctx *c, const char *src, uint64_t len, int where, char *out, uint64_t cap,
                         const char *what);

int tk_dbg_create(tk_ctx *c, const char *bundle, uint64_t len, int where, int K, int strand, tk_dbg **out) {
    CHECK_CTX(c);
    if (!out) return TK_E_INVAL;
    *out = nullptr;
    if (K < 1 || K > MAX_K - 1) return set_err(c, TK_E_INVAL, "FastaToDeBruijn: K must be in 1..30");
    tk_dbg *g = new (std::nothrow) tk_dbg();
    if (!g) return TK_E_OOM;
    g->ctx = c;
    ctx_acquire(c);
    g->k = K;
    g->strand = strand ? 1 : 0;
    tk_reads *b = nullptr;
    int e = tk_reads_parse(c, bundle, len, where, &b);
    if (!e && b->format == TK_FMT_FASTQ) e = set_err(c, TK_E_PARSE, "bundle must be FASTA");
    std::vector<uint64_t> ids;
    if (!e) {
        g->n_records = b->n_reads;
        e = bundle_component_ids(c, b, bundle, len, where, &ids);
    }
    if (!e) e = dbg_build(g, b, ids);
    if (b) tk_reads_free(b);
    if (e) {
        tk_dbg_free(g);
        return e;
    }
    *out = g;
    return TK_OK;
}

int tk_dbg_info(const tk_dbg *g, uint64_t *n_components, uint64_t *n_nodes, uint64_t *text_len) {
    if (!g) return TK_E_INVAL;
    if (n_components) *n_components = g->n_components;
    if (n_nodes) *n_nodes = g->n_nodes;
    if (text_len) *text_len = g->text_len;
    return TK_OK;
}

int tk_dbg_text(const tk_dbg *g, int where, char *out, uint64_t cap) {
    if (!g) return TK_E_INVAL;
    tk_ctx *c = g->ctx;
    CHECK_CTX(c);
    return norm_copy_out(c, g->d_text, g->text_len, where, out, cap, "tk_dbg_text");
}

void tk_dbg_free(tk_dbg *g) {
    if (!g) return;
    tk_ctx *c = g->ctx;
    cudaSetDevice(c->device);
    dfree(c, g->d_text);
    delete g;
    ctx_release(c);
}

// ------------------------------------------------------------------ normalization

int tk_norm_select_multi(tk_ctx *c, const tk_reads *const *left, uint32_t n_left, const uint32_t *left_median,
                         const float *left_mean, const float *left_stdev, const tk_reads *const *right,
                         uint32_t n_right, const uint32_t *right_median, const float *right_mean,
                         const float *right_stdev, int where, int max_cov, int min_cov, int max_cv, tk_norm **out) {
    if (!out) return TK_E_INVAL;
    *out = nullptr;
    CHECK_CTX(c);
    if (!left || n_left == 0 || (right && n_right == 0))
        return set_err(c, TK_E_INVAL, "tk_norm_select: no read set on a side");
    if (where != TK_HOST && where != TK_DEVICE) return set_err(c, TK_E_INVAL, "tk_norm_select: where");
    uint64_t nl = 0, nr = 0;
    for (uint32_t i = 0; i < n_left; i++) {
        if (!left[i] || left[i]->ctx != c) return set_err(c, TK_E_INVAL, "tk_norm_select: read sets of another context");
        nl += left[i]->n_reads;
    }
    for (uint32_t i = 0; right && i < n_right; i++) {
        if (!right[i] || right[i]->ctx != c) return set_err(c, TK_E_INVAL, "tk_norm_select: read sets of another context");
        nr += right[i]->n_reads;
    }
    if (nl && (!left_median || !left_mean || !left_stdev))
        return set_err(c, TK_E_INVAL, "tk_norm_select: left statistics missing");
    if (right && nr && (!right_median || !right_mean || !right_stdev))
        return set_err(c, TK_E_INVAL, "tk_norm_select: right statistics missing");
    if (nl > 0xFFFFFFFFull || nr > 0xFFFFFFFFull)
        return set_err(c, TK_E_INVAL, "tk_norm_select: more than 2^32 reads on a side");
    tk_norm *nm = new (std::nothrow) tk_norm();
    if (!nm) return TK_E_OOM;
    nm->ctx = c;
    nm->pairs = right != nullptr;
    nm->max_cov = max_cov;
    nm->min_cov = min_cov;
    nm->max_cv = max_cv;
    ctx_acquire(c);
    const tk_reads *const *sets[2] = {left, right};
    const uint32_t nsets[2] = {n_left, right ? n_right : 0u};
    const uint32_t *med[2] = {left_median, right_median};
    const float *mean[2] = {left_mean, right_mean};
    const float *sd[2] = {left_stdev, right_stdev};
    int e = norm_select(nm, sets, nsets, med, mean, sd, where);
    if (e) {
        tk_norm_free(nm);
        return e;
    }
    *out = nm;
    return TK_OK;
}

int tk_norm_select(tk_ctx *c, const tk_reads *left, const uint32_t *left_median, const float *left_mean,
                   const float *left_stdev, const tk_reads *right, const uint32_t *right_median,
                   const float *right_mean, const float *right_stdev, int where, int max_cov, int min_cov,
                   int max_cv, tk_norm **out) {
    if (!left) {
        if (out) *out = nullptr;
        return c ? set_err(c, TK_E_INVAL, "tk_norm_select: no left read set") : TK_E_INVAL;
    }
    return tk_norm_select_multi(c, &left, 1, left_median, left_mean, left_stdev, right ? &right : nullptr,
                                right ? 1u : 0u, right_median, right_mean, right_stdev, where, max_cov, min_cov,
                                max_cv, out);
}

int tk_norm_info(const tk_norm *nm, tk_norm_counts *counts, uint64_t *accs_len) {
    if (!nm) return TK_E_INVAL;
    if (counts) *counts = nm->counts;
    if (accs_len) *accs_len = nm->accs_len;
    return TK_OK;
}

static int norm_copy_out(tk_ctx *c, const char *src, uint64_t len, int where, char *out, uint64_t cap,
                         const char *what) {
    if (!out && len) return set_err(c, TK_E_INVAL, std::string(what) + ": no buffer");
    if (cap < len) return set_err(c, TK_E_RANGE, std::string(what) + ": buffer smaller than the text");
    if (len)
        TK_CUDA(c, cudaMemcpyAsync(out, src, len, where == TK_DEVICE ? cudaMemcpyDeviceToDevice : cudaMemcpyDeviceToHost,
                                   c->stream));
    return cuda_check(c, cudaStreamSynchronize(c->stream), what);
}

int tk_norm_accs(const tk_norm *nm, int where, char *out, uint64_t cap) {
    if (!nm) return TK_E_INVAL;
    tk_ctx *c = nm->ctx;
    CHECK_CTX(c);
    return norm_copy_out(c, nm->d_accs, nm->accs_len, where, out, cap, "tk_norm_accs");
}

int tk_norm_table(tk_norm *nm, int where, char *out, uint64_t cap, uint64_t *len) {
    if (!nm) return TK_E_INVAL;
    tk_ctx *c = nm->ctx;
    CHECK_CTX(c);
    TK_TRY(norm_table(nm));
    if (len) *len = nm->table_len;
    if (!out) return TK_OK;
    return norm_copy_out(c, nm->d_table, nm->table_len, where, out, cap, "tk_norm_table");
}

int tk_norm_extract_multi(tk_norm *nm, const tk_reads *const *sets, uint32_t n_sets, uint64_t *len) {
    if (!nm || !sets || n_sets == 0) return TK_E_INVAL;
    tk_ctx *c = nm->ctx;
    CHECK_CTX(c);
    for (uint32_t i = 0; i < n_sets; i++)
        if (!sets[i] || sets[i]->ctx != c) return set_err(c, TK_E_INVAL, "tk_norm_extract: read set of another context");
    TK_TRY(norm_extract(nm, sets, n_sets));
    if (len) *len = nm->ext_len;
    return TK_OK;
}

int tk_norm_extract(tk_norm *nm, const tk_reads *fastq, uint64_t *len) {
    if (!nm || !fastq) return TK_E_INVAL;
    return tk_norm_extract_multi(nm, &fastq, 1, len);
}

int tk_norm_extract_copy(const tk_norm *nm, int where, char *out, uint64_t cap) {
    if (!nm) return TK_E_INVAL;
    tk_ctx *c = nm->ctx;
    CHECK_CTX(c);
    return norm_copy_out(c, nm->d_ext, nm->ext_len, where, out, cap, "tk_norm_extract_copy");
}

int tk_norm_extract_copy_async(tk_norm *nm, char *out, uint64_t cap) {
    if (!nm) return TK_E_INVAL;
    tk_ctx *c = nm->ctx;
    CHECK_CTX(c);
    if (!out && nm->ext_len) return set_err(c, TK_E_INVAL, "tk_norm_extract_copy_async: no buffer");
    if (cap < nm->ext_len) return set_err(c, TK_E_RANGE, "tk_norm_extract_copy_async: buffer smaller than the text");
    if (!nm->ext_len) return TK_OK;
    cudaStream_t cs = copy_stream(c);
    if (!cs) return norm_copy_out(c, nm->d_ext, nm->ext_len, TK_HOST, out, cap, "tk_norm_extract_copy_async");
    cudaEvent_t built = nullptr;
    TK_CUDA(c, cudaEventCreateWithFlags(&built, cudaEventDisableTiming));
    int e = cuda_check(c, cudaEventRecord(built, c->stream), "event record");
    if (!e) e = cuda_check(c, cudaStreamWaitEvent(cs, built, 0), "copy stream wait");
    cudaEventDestroy(built);
    if (!e) e = cuda_check(c, cudaMemcpyAsync(out, nm->d_ext, nm->ext_len, cudaMemcpyDeviceToHost, cs), "records d2h");
    if (!e && !nm->ext_copy_done)
        e = cuda_check(c, cudaEventCreateWithFlags(&nm->ext_copy_done, cudaEventDisableTiming), "event");
    if (!e) e = cuda_check(c, cudaEventRecord(nm->ext_copy_done, cs), "event record");
    return e;
}

void tk_norm_free(tk_norm *nm) {
    if (!nm) return;
    tk_ctx *c = nm->ctx;
    cudaSetDevice(c->device);
    norm_release(nm);
    delete nm;
    ctx_release(c);
}

}  // extern "C"
