// tk_cov.cu -- K5: per-read k-mer coverage statistics
// (Inchworm fastaToKmerCoverageStats, called at
// util/insilico_read_normalization.pl:837-846).
//
// For each read, every window of k A/C/G/T bases is looked up in the count
// table (canonical key with --DS); a k-mer absent from the table counts 1
// (the catalogue is dumped at -L 2, Changelog.txt:536-538).  Windows holding
// another character are skipped.  median = element n/2 of the sorted values;
// mean and stdev come from exact integer sums (see finish_stats).
//
// Reads with at most 256 windows: one warp per read, values in registers,
// warp bitonic sort (tk_warp.cuh).  Longer reads: one block per read, values
// in a global scratch slab, block bitonic sort.
//
// Coverage cache.  The reads whose coverage is asked for are, in Trinity's
// use, the reads that were counted (insilico_read_normalization.pl counts
// both mate files and then looks every window of each up again), so a k-mer
// is looked up about as often as its count.  Before the first pass over a
// large table, the k-mers with the highest counts are copied into a small
// table sized to stay in L2 (64 MB, TRINKMER_COV_CACHE_MB): 32-byte buckets of
// four 8-byte entries; bucket = the top bits of a bijective hash of the key
// on its 2k bits, entry = (the rest of the hash << cbits) | count, so one
// sector answers a lookup.  Each bucket keeps the four highest counts that
// hash to it (a key displaces the smallest entry when its count is larger).
// A lookup that misses the cache reads the table itself, so the statistics
// do not depend on what the cache holds.  Random lookups into HBM run at
// ~40 G/s on GB300 whatever the table size above 1 GB, and into an
// L2-resident table at ~300 G/s; at the plain path's scale the 6-7M k-mers
// the cache holds answer ~70% of the lookups.
#include "tk_warp.cuh"

#include <algorithm>
#include <cstdlib>
#include <mutex>
#include <string>

namespace tk {

constexpr int CV_THREADS = 256;
constexpr uint32_t CV_WARP_MAX = 256;   // windows handled by the warp path

// ------------------------------------------------------------------ coverage cache

struct CovCache {
    uint64_t *ent;     // 4 entries per bucket; nullptr = no cache
    int n;             // key bits (2k)
    int rbits;         // hash bits an entry keeps; the other 64 - rbits hold the count
};

// A bijection of [0, 2^n): xor-shifts and multiplications by odd constants,
// each invertible modulo 2^n, so (bucket, remainder) identifies the key.
__host__ __device__ __forceinline__ uint64_t kmix_n(uint64_t x, int n) {
    const uint64_t m = (1ULL << n) - 1;   // n <= 62
    const int s = (n + 1) >> 1;
    x ^= x >> s;
    x = (x * 0x9E3779B97F4A7C15ULL) & m;
    x ^= x >> s;
    x = (x * 0xD6E8FEB86659FD93ULL) & m;
    x ^= x >> s;
    return x;
}

__device__ __forceinline__ bool cache_get(const CovCache &cc, uint64_t key, uint32_t *val) {
    const uint64_t h = kmix_n(key, cc.n);
    const uint64_t *b = cc.ent + ((h >> cc.rbits) << 2);
    const uint64_t r = h & ((1ULL << cc.rbits) - 1);
    const int cbits = 64 - cc.rbits;
    uint64_t e0, e1, e2, e3, pol;
    // L2 evict-last: the cache's lines outlive the table lines streamed past them
    asm("createpolicy.fractional.L2::evict_last.b64 %0, 1.0;" : "=l"(pol));
    asm("ld.global.L2::cache_hint.v4.u64 {%0,%1,%2,%3}, [%4], %5;"
        : "=l"(e0), "=l"(e1), "=l"(e2), "=l"(e3)
        : "l"(b), "l"(pol));
    // an entry is never 0 (its count is >= 2), so an empty entry matches nothing
    uint64_t hit = 0;
    hit = (e0 && (e0 >> cbits) == r) ? e0 : hit;
    hit = (e1 && (e1 >> cbits) == r) ? e1 : hit;
    hit = (e2 && (e2 >> cbits) == r) ? e2 : hit;
    hit = (e3 && (e3 >> cbits) == r) ? e3 : hit;
    *val = (uint32_t)(hit & (~0ULL >> cc.rbits));
    return hit != 0;
}

// the count of `key` for the statistics: the cache, else the table (1 when absent)
__device__ __forceinline__ uint32_t cov_lookup(const CovCache &cc, DevTable t, uint64_t key) {
    uint32_t v;
    if (cc.ent && cache_get(cc, key, &v)) return v;
    return tbl_get(t, key, 1u);
}

// Offers one (key, count) to its bucket: into an empty entry, else in place
// of the smallest count when larger.  A CAS lost to another thread re-reads
// the bucket; after 32 rounds the key is left out (the cache stays valid).
__device__ __forceinline__ void cache_offer(const CovCache &cc, uint64_t key, uint64_t count) {
    const uint64_t h = kmix_n(key, cc.n);
    unsigned long long *b = reinterpret_cast<unsigned long long *>(cc.ent + ((h >> cc.rbits) << 2));
    const uint64_t cmask = ~0ULL >> cc.rbits;
    const unsigned long long mine = ((h & ((1ULL << cc.rbits) - 1)) << (64 - cc.rbits)) | count;
    for (int round = 0; round < 32; round++) {
        int at = 0;
        unsigned long long old = 0, least = ~0ULL;
#pragma unroll
        for (int j = 0; j < 4; j++) {
            const unsigned long long e = *reinterpret_cast<volatile unsigned long long *>(b + j);
            const unsigned long long c = e ? (e & cmask) : 0ULL;
            if (c < least) {
                least = c;
                at = j;
                old = e;
            }
        }
        if (count <= least) return;
        if (atomicCAS(b + at, old, mine) == old) return;
    }
}

__global__ void __launch_bounds__(256) k_cache_build(const Slot *__restrict__ slots, uint64_t cap, CovCache cc) {
    const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
    const uint64_t cmask = ~0ULL >> cc.rbits;
    for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < cap; i += stride) {
        const ulonglong2 s = __ldcs(reinterpret_cast<const ulonglong2 *>(slots + i));
        const uint64_t c = (uint32_t)s.y;
        if (s.x == EMPTY_KEY || c < 2 || c > cmask) continue;
        cache_offer(cc, s.x, c);
    }
}

static uint64_t cache_bytes_wanted() {
    uint64_t mb = 64;
    if (const char *v = getenv("TRINKMER_COV_CACHE_MB")) mb = strtoull(v, nullptr, 10);
    return mb << 20;
}

// The cache of table t (built when missing or stale); cc->ent == nullptr when
// the table is small enough for L2 to hold it whole, or k is too small.
static int cache_get_or_build(tk_table *t, CovCache *cc) {
    cc->ent = nullptr;
    tk_ctx *c = t->ctx;
    const uint64_t want = cache_bytes_wanted();
    if (want < 32 || t->capacity * sizeof(Slot) < 4 * want) return TK_OK;
    int hbits = 0;
    while ((32ULL << (hbits + 1)) <= want) hbits++;
    const int n = 2 * t->k;
    if (n - hbits < 1 || 64 - (n - hbits) < 2) return TK_OK;
    const uint64_t bytes = 32ULL << hbits;
    cc->n = n;
    cc->rbits = n - hbits;
    if (!t->hot_valid || t->hot_bytes != bytes) {
        if (t->d_hot && t->hot_bytes != bytes) {
            dfree(c, t->d_hot);
            t->d_hot = nullptr;
        }
        if (!t->d_hot) TK_TRY(dmalloc(c, (void **)&t->d_hot, bytes, "coverage cache"));
        t->hot_bytes = bytes;
        TK_CUDA(c, cudaMemsetAsync(t->d_hot, 0, bytes, c->stream));
        cc->ent = t->d_hot;
        cudaEvent_t ev;
        prof_begin(c, TK_KID_COV_CACHE, &ev);
        const uint64_t blocks = std::min<uint64_t>((t->capacity + 255) / 256, (uint64_t)c->sm_count * 16);
        k_cache_build<<<(unsigned)std::max<uint64_t>(blocks, 1), 256, 0, c->stream>>>(t->t.slots, t->capacity, *cc);
        c->launches++;
        prof_end(c, TK_KID_COV_CACHE, ev, t->capacity);
        TK_TRY(check_launch(c, "coverage cache"));
        t->hot_valid = true;
    }
    cc->ent = t->d_hot;
    return TK_OK;
}

// Integer statistics of one read, uniform over the warp.
struct ReadSums {
    uint32_t cnt, med;
    uint64_t sum, hi, lo;
};
constexpr uint32_t LONG_READ = 0xFFFFFFFFu;   // cnt of a read left to the long-read pass

template <int S, bool CANON>
__device__ __forceinline__ ReadSums cov_warp_read(const CovCache &cc, DevTable t, const uint64_t *__restrict__ codes,
                                                  const uint32_t *__restrict__ inv, uint64_t start, uint32_t nwin,
                                                  int k) {
    const uint32_t span = (nwin + 31) / 32;
    uint32_t v[S];
    uint32_t vm = 0;
    uint32_t cnt = 0;
    uint64_t sum = 0, hi = 0, lo = 0;
    lane_windows_codes<S, CANON>(codes, inv, start, nwin, span, k, [&](int j, bool valid, uint64_t key) {
        uint32_t c = 0;
        if (valid) {
            c = cov_lookup(cc, t, key);
            vm |= 1u << j;
            cnt++;
            sum += c;
            uint64_t sq = (uint64_t)c * c;   // < 2^64
            uint64_t nlo = lo + sq;
            hi += nlo < lo;
            lo = nlo;
        }
        v[j] = c;
    });
    ReadSums rs;
    rs.cnt = warp_sum(cnt);
    rs.sum = warp_sum(sum);
    warp_sum_u128(hi, lo);
    rs.hi = hi;
    rs.lo = lo;
    rs.med = rs.cnt ? warp_select<S>(v, vm, rs.cnt / 2) : 0u;
    return rs;
}

// One warp, 32 consecutive reads [r0, r0 + 32): the warp computes each read's
// sums in turn and lane i keeps read r0 + i's; then every lane finishes its own
// read.  The floating-point finish runs on the FP64 pipe, whose cost is per
// warp instruction whatever the number of active lanes, so finishing 32 reads
// in one pass costs what one read alone would.  Reads with more than
// CV_WARP_MAX windows are appended to long_list (or, with no list, left to a
// separate pass) and not written here.
template <bool CANON>
__device__ __forceinline__ void cov_warp_chunk(const CovCache &cc, DevTable t, const uint64_t *__restrict__ codes,
                                               const uint32_t *__restrict__ inv,
                                               const uint64_t *__restrict__ rd_off, uint64_t n_reads, int k, uint64_t r0,
                                               uint32_t *__restrict__ median, float *__restrict__ mean,
                                               float *__restrict__ stdev, uint32_t *__restrict__ long_list,
                                               unsigned long long *__restrict__ long_n, ReadSums *__restrict__ held) {
    const unsigned lane = lane_id();
    const uint32_t nr = n_reads - r0 < 32 ? (uint32_t)(n_reads - r0) : 32u;
    // lane i holds the start of read r0 + i; the end of the last is one more load
    const uint64_t my_start = rd_off[r0 + (lane < nr ? lane : nr)];
    const uint64_t last_end = __shfl_sync(0xffffffffu, my_start, (int)(nr < 32 ? nr : 31));
    const uint64_t end_nr = nr < 32 ? last_end : rd_off[r0 + 32];
    for (uint32_t i = 0; i < nr; i++) {
        const uint64_t r = r0 + i;
        const uint64_t start = __shfl_sync(0xffffffffu, my_start, (int)i);
        const uint64_t next = i + 1 < 32 ? __shfl_sync(0xffffffffu, my_start, (int)(i + 1) & 31) : end_nr;
        const uint64_t L = (i + 1 < nr ? next : end_nr) - start - 1;
        const uint32_t nwin = L >= (uint64_t)k ? (uint32_t)(L - k + 1) : 0u;
        ReadSums rs;
        bool is_long = false;
        if (nwin <= 32) rs = cov_warp_read<1, CANON>(cc, t, codes, inv, start, nwin, k);
        else if (nwin <= 64) rs = cov_warp_read<2, CANON>(cc, t, codes, inv, start, nwin, k);
        else if (nwin <= 128) rs = cov_warp_read<4, CANON>(cc, t, codes, inv, start, nwin, k);
        else if (nwin <= CV_WARP_MAX) rs = cov_warp_read<8, CANON>(cc, t, codes, inv, start, nwin, k);
        else {
            is_long = true;
            if (long_list && lane == 0) long_list[atomicAdd(long_n, 1ULL)] = (uint32_t)r;
        }
        if (lane == 0) {
            if (is_long) rs.cnt = LONG_READ;
            held[i] = rs;
        }
    }
    __syncwarp();
    const ReadSums mine = held[lane < nr ? lane : 0];
    __syncwarp();
    if (lane < nr && mine.cnt != LONG_READ) {
        float m, sd;
        finish_stats(mine.cnt, mine.sum, mine.hi, mine.lo, &m, &sd);
        median[r0 + lane] = mine.med;
        mean[r0 + lane] = m;
        stdev[r0 + lane] = sd;
    }
}

template <bool CANON>
__global__ void __launch_bounds__(CV_THREADS, 6) k_coverage(CovCache cc, DevTable t, const uint64_t *__restrict__ codes,
                                                        const uint32_t *__restrict__ inv,
                                                        const uint64_t *__restrict__ rd_off, uint64_t n_reads, int k,
                                                        uint32_t *__restrict__ median, float *__restrict__ mean,
                                                        float *__restrict__ stdev, uint32_t *__restrict__ long_list,
                                                        unsigned long long *__restrict__ long_n) {
    __shared__ ReadSums held[CV_THREADS];
    const uint64_t warps = (uint64_t)gridDim.x * (CV_THREADS / 32);
    const uint64_t chunks = (n_reads + 31) / 32;
    for (uint64_t ch = (uint64_t)blockIdx.x * (CV_THREADS / 32) + (threadIdx.x >> 5); ch < chunks; ch += warps)
        cov_warp_chunk<CANON>(cc, t, codes, inv, rd_off, n_reads, k, ch * 32, median, mean, stdev, long_list, long_n,
                              held + (threadIdx.x & ~31u));
}

// long reads: one block per read, `slab` = this block's scratch (n2max values)
template <bool CANON>
__global__ void __launch_bounds__(CV_THREADS) k_coverage_long(CovCache cc, DevTable t, const uint8_t *__restrict__ seq,
                                                             const uint64_t *__restrict__ rd_off,
                                                             const uint32_t *__restrict__ list, uint64_t n_long, int k,
                                                             uint32_t *__restrict__ scratch, uint64_t n2max,
                                                             uint32_t *__restrict__ median, float *__restrict__ mean,
                                                             float *__restrict__ stdev) {
    __shared__ uint32_t s_cnt[CV_THREADS / 32];
    __shared__ uint64_t s_sum[CV_THREADS / 32], s_hi[CV_THREADS / 32], s_lo[CV_THREADS / 32];
    uint32_t *slab = scratch + (uint64_t)blockIdx.x * n2max;
    for (uint64_t i = blockIdx.x; i < n_long; i += gridDim.x) {
        const uint32_t r = list[i];
        const uint64_t start = rd_off[r];
        const uint32_t nwin = (uint32_t)(rd_off[r + 1] - start - 1 - (k - 1));
        uint32_t n2 = 1;
        while (n2 < nwin) n2 <<= 1;
        block_window_values<CANON>(seq, start, nwin, n2, k, slab,
                                   [&](uint64_t key) { return cov_lookup(cc, t, key); });
        uint32_t cnt = 0;
        uint64_t sum = 0, hi = 0, lo = 0;
        for (uint32_t w = threadIdx.x; w < nwin; w += blockDim.x) {
            uint32_t c = slab[w];
            if (c == PAD_VAL) continue;
            cnt++;
            sum += c;
            uint64_t sq = (uint64_t)c * c, nlo = lo + sq;
            hi += nlo < lo;
            lo = nlo;
        }
        cnt = warp_sum(cnt);
        sum = warp_sum(sum);
        warp_sum_u128(hi, lo);
        if (lane_id() == 0) {
            s_cnt[threadIdx.x >> 5] = cnt;
            s_sum[threadIdx.x >> 5] = sum;
            s_hi[threadIdx.x >> 5] = hi;
            s_lo[threadIdx.x >> 5] = lo;
        }
        block_bitonic_sort(slab, n2);
        if (threadIdx.x == 0) {
            uint32_t tc = 0;
            uint64_t ts = 0, th = 0, tl = 0;
            for (int w = 0; w < CV_THREADS / 32; w++) {
                tc += s_cnt[w];
                ts += s_sum[w];
                uint64_t nl = tl + s_lo[w];
                th += s_hi[w] + (nl < tl);
                tl = nl;
            }
            float m, s;
            finish_stats(tc, ts, th, tl, &m, &s);
            median[r] = tc ? slab[tc / 2] : 0u;
            mean[r] = m;
            stdev[r] = s;
        }
        __syncthreads();
    }
}

int coverage_stats(tk_table *t, const tk_reads *rd, uint32_t *d_median, float *d_mean, float *d_stdev) {
    tk_ctx *c = t->ctx;
    const uint64_t n = rd->n_reads;
    if (n == 0) return TK_OK;
    const int k = t->k;
    const bool may_long = rd->max_len >= (uint32_t)k && rd->max_len - k + 1 > CV_WARP_MAX;
    uint32_t *long_list = nullptr;
    unsigned long long *long_n = nullptr;
    TK_TRY(dmalloc(c, (void **)&long_n, 8, "long-read count"));
    int e = TK_OK;
    if (may_long) e = dmalloc(c, (void **)&long_list, n * 4, "long-read list");
    if (!e) e = cuda_check(c, cudaMemsetAsync(long_n, 0, 8, c->stream), "long reset");
    DevTable dt = t->t;
    Slot *empty = nullptr;
    if (!e && t->capacity == 0) {
        // an empty catalogue: every k-mer counts 1; give the kernel a one-slot table
        e = dmalloc(c, (void **)&empty, sizeof(Slot) * 2, "empty table");
        if (!e) {
            cudaMemsetAsync(empty, 0xFF, sizeof(Slot) * 2, c->stream);
            dt = tbl_empty(empty);
        }
    }
    CovCache cc{};
    if (!e && t->capacity) e = cache_get_or_build(t, &cc);
    if (!e) {
        const uint64_t chunks = (n + 31) / 32;
        const unsigned grid = (unsigned)std::max<uint64_t>(
            1, std::min<uint64_t>((chunks + CV_THREADS / 32 - 1) / (CV_THREADS / 32), (uint64_t)c->sm_count * 16));
        cudaEvent_t ev;
        prof_begin(c, TK_KID_COVERAGE, &ev);
        if (t->canonical)
            k_coverage<true><<<grid, CV_THREADS, 0, c->stream>>>(cc, dt, rd->d_codes, rd->d_inv, rd->d_rd_off, n, k,
                                                                 d_median, d_mean, d_stdev, long_list, long_n);
        else
            k_coverage<false><<<grid, CV_THREADS, 0, c->stream>>>(cc, dt, rd->d_codes, rd->d_inv, rd->d_rd_off, n, k,
                                                                  d_median, d_mean, d_stdev, long_list, long_n);
        c->launches++;
        prof_end(c, TK_KID_COVERAGE, ev, rd->n_bases);
        e = check_launch(c, "coverage");
    }
    unsigned long long hl = 0;
    if (!e && may_long) {
        e = cuda_check(c, cudaMemcpyAsync(&hl, long_n, 8, cudaMemcpyDeviceToHost, c->stream), "long n");
        if (!e) e = cuda_check(c, cudaStreamSynchronize(c->stream), "long sync");
    }
    if (!e && hl) {
        uint64_t n2max = 1;
        while (n2max < (uint64_t)(rd->max_len - k + 1)) n2max <<= 1;
        uint64_t grid = std::min<uint64_t>(hl, (uint64_t)c->sm_count * 2);
        uint32_t *scratch = nullptr;
        e = dmalloc(c, (void **)&scratch, grid * n2max * 4, "long-read scratch");
        if (!e) {
            if (t->canonical)
                k_coverage_long<true><<<(unsigned)grid, CV_THREADS, 0, c->stream>>>(
                    cc, dt, rd->d_seq, rd->d_rd_off, long_list, hl, k, scratch, n2max, d_median, d_mean, d_stdev);
            else
                k_coverage_long<false><<<(unsigned)grid, CV_THREADS, 0, c->stream>>>(
                    cc, dt, rd->d_seq, rd->d_rd_off, long_list, hl, k, scratch, n2max, d_median, d_mean, d_stdev);
            c->launches++;
            e = check_launch(c, "coverage long");
            dfree(c, scratch);
        }
    }
    if (long_list) dfree(c, long_list);
    dfree(c, long_n);
    if (empty) dfree(c, empty);
    return e;
}

// ---------------------------------------------------------------------------
// Allocation-free variant (tk_coverage_stats_noalloc).
//
// Some callers cannot allocate device memory while they compute: a resident
// service that has already carved all of its HBM into job slots under an
// admission budget, or a pipeline that must not risk an allocation failure or
// the implicit device synchronisation cudaMalloc/cudaFree can bring in the
// middle of its work.  For them the long-read statistics use a fixed slab in
// this file-scope device array instead of cudaMalloc'd scratch.  A GPU holds
// the array (16 MiB) from the moment this file's device code is loaded on it
// until the process exits; under lazy module loading that is the first launch
// of one of its kernels or the first address lookup below, whichever comes
// first.  Host code must not pass `g_noalloc_scratch` itself to a kernel: in host code
// that name is a host-side stand-in, so its device address is fetched once per
// device with cudaGetSymbolAddress (see noalloc_scratch_ptr).

constexpr uint64_t NOALLOC_SCRATCH_BYTES = 16ULL << 20;
constexpr int NOALLOC_BLOCKS = 32;
constexpr uint64_t NOALLOC_SLAB = NOALLOC_SCRATCH_BYTES / 4 / NOALLOC_BLOCKS;   // 131,072 windows per block
constexpr int NOALLOC_MAX_DEVICES = 64;

static __device__ __align__(256) uint32_t g_noalloc_scratch[NOALLOC_SCRATCH_BYTES / 4];
static __device__ __align__(16) Slot g_noalloc_empty[2] = {{EMPTY_KEY, 0u, 0u}, {EMPTY_KEY, 0u, 0u}};

// short reads only (<= 256 windows); longer reads are left to k_coverage_long_slab
template <bool CANON>
__global__ void __launch_bounds__(CV_THREADS, 4) k_coverage_short(DevTable t, const uint64_t *__restrict__ codes,
                                                              const uint32_t *__restrict__ inv,
                                                              const uint64_t *__restrict__ rd_off, uint64_t n_reads, int k,
                                                              uint32_t *__restrict__ median, float *__restrict__ mean,
                                                              float *__restrict__ stdev) {
    __shared__ ReadSums held[CV_THREADS];
    const uint64_t warps = (uint64_t)gridDim.x * (CV_THREADS / 32);
    const uint64_t chunks = (n_reads + 31) / 32;
    const CovCache none{};
    for (uint64_t ch = (uint64_t)blockIdx.x * (CV_THREADS / 32) + (threadIdx.x >> 5); ch < chunks; ch += warps)
        cov_warp_chunk<CANON>(none, t, codes, inv, rd_off, n_reads, k, ch * 32, median, mean, stdev, nullptr, nullptr,
                              held + (threadIdx.x & ~31u));
}

// Reads with more than 256 windows, one block per read; block b works in
// slab b of the static array.  A block takes 256 reads at a time, one per
// thread, lists the long ones in shared memory and then works through the
// list, so finding the long reads costs one parallel pass over the reads.
template <bool CANON>
__global__ void __launch_bounds__(CV_THREADS) k_coverage_long_slab(DevTable t, const uint8_t *__restrict__ seq,
                                                                  const uint64_t *__restrict__ rd_off, uint64_t n_reads,
                                                                  int k, uint32_t *__restrict__ scratch,
                                                                  uint32_t *__restrict__ median, float *__restrict__ mean,
                                                                  float *__restrict__ stdev) {
    __shared__ uint32_t s_cnt[CV_THREADS / 32];
    __shared__ uint64_t s_sum[CV_THREADS / 32], s_hi[CV_THREADS / 32], s_lo[CV_THREADS / 32];
    __shared__ uint32_t s_list[CV_THREADS];
    __shared__ uint32_t s_nlong;
    uint32_t *slab = scratch + (uint64_t)blockIdx.x * NOALLOC_SLAB;
    for (uint64_t base = (uint64_t)blockIdx.x * CV_THREADS; base < n_reads; base += (uint64_t)gridDim.x * CV_THREADS) {
        if (threadIdx.x == 0) s_nlong = 0;
        __syncthreads();
        {
            const uint64_t r = base + threadIdx.x;
            if (r < n_reads) {
                const uint64_t L = rd_off[r + 1] - rd_off[r] - 1;
                if (L >= (uint64_t)k && L - k + 1 > CV_WARP_MAX) s_list[atomicAdd(&s_nlong, 1u)] = threadIdx.x;
            }
        }
        __syncthreads();
        const uint32_t n_long = s_nlong;
        for (uint32_t li = 0; li < n_long; li++) {
            const uint64_t r = base + s_list[li];
            const uint64_t start = rd_off[r];
            const uint64_t L = rd_off[r + 1] - start - 1;
            const uint32_t nwin = (uint32_t)(L - k + 1);
            uint32_t n2 = 1;
            while (n2 < nwin) n2 <<= 1;
            // every slab entry read below is written first: nothing carries over between reads or calls
            block_window_values<CANON>(seq, start, nwin, n2, k, slab, [&](uint64_t key) { return tbl_get(t, key, 1u); });
            uint32_t cnt = 0;
            uint64_t sum = 0, hi = 0, lo = 0;
            for (uint32_t w = threadIdx.x; w < nwin; w += blockDim.x) {
                uint32_t c = slab[w];
                if (c == PAD_VAL) continue;
                cnt++;
                sum += c;
                uint64_t sq = (uint64_t)c * c, nlo = lo + sq;
                hi += nlo < lo;
                lo = nlo;
            }
            cnt = warp_sum(cnt);
            sum = warp_sum(sum);
            warp_sum_u128(hi, lo);
            if (lane_id() == 0) {
                s_cnt[threadIdx.x >> 5] = cnt;
                s_sum[threadIdx.x >> 5] = sum;
                s_hi[threadIdx.x >> 5] = hi;
                s_lo[threadIdx.x >> 5] = lo;
            }
            block_bitonic_sort(slab, n2);
            if (threadIdx.x == 0) {
                uint32_t tc = 0;
                uint64_t ts = 0, th = 0, tl = 0;
                for (int w = 0; w < CV_THREADS / 32; w++) {
                    tc += s_cnt[w];
                    ts += s_sum[w];
                    uint64_t nl = tl + s_lo[w];
                    th += s_hi[w] + (nl < tl);
                    tl = nl;
                }
                float m, s;
                finish_stats(tc, ts, th, tl, &m, &s);
                median[r] = tc ? slab[tc / 2] : 0u;
                mean[r] = m;
                stdev[r] = s;
            }
            __syncthreads();
        }
        __syncthreads();
    }
}

static std::mutex g_noalloc_mu;
static void *g_noalloc_scratch_dev[NOALLOC_MAX_DEVICES];
static void *g_noalloc_empty_dev[NOALLOC_MAX_DEVICES];

// Set-up, once per device, with that device current: the device addresses of
// the static scratch array and of the empty two-slot table.
static int noalloc_scratch_ptr(tk_ctx *c, uint32_t **scratch, Slot **empty) {
    if (c->device < 0 || c->device >= NOALLOC_MAX_DEVICES) return set_err(c, TK_E_INVAL, "device ordinal too large");
    std::lock_guard<std::mutex> g(g_noalloc_mu);
    if (!g_noalloc_scratch_dev[c->device]) {
        void *p = nullptr, *q = nullptr;
        cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
        if (e != cudaSuccess) return cuda_check(c, e, "cudaGetSymbolAddress(no-allocation scratch)");
        e = cudaGetSymbolAddress(&q, g_noalloc_empty);
        if (e != cudaSuccess) return cuda_check(c, e, "cudaGetSymbolAddress(empty table)");
        g_noalloc_scratch_dev[c->device] = p;
        g_noalloc_empty_dev[c->device] = q;
    }
    *scratch = (uint32_t *)g_noalloc_scratch_dev[c->device];
    *empty = (Slot *)g_noalloc_empty_dev[c->device];
    return TK_OK;
}

int coverage_stats_noalloc(tk_table *t, const tk_reads *rd, uint32_t *d_median, float *d_mean, float *d_stdev) {
    tk_ctx *c = t->ctx;
    const uint64_t n = rd->n_reads;
    const int k = t->k;
    if (rd->max_len >= (uint32_t)k && (uint64_t)(rd->max_len - k + 1) > NOALLOC_SLAB)
        return set_err(c, TK_E_RANGE, "tk_coverage_stats_noalloc: a read has " + std::to_string(rd->max_len - k + 1) +
                                          " windows; the allocation-free path handles at most " +
                                          std::to_string(NOALLOC_SLAB) + " per read");
    uint32_t *scratch = nullptr;
    Slot *empty = nullptr;
    TK_TRY(noalloc_scratch_ptr(c, &scratch, &empty));
    if (n == 0) return TK_OK;
    DevTable dt = t->t;
    if (t->capacity == 0) dt = tbl_empty(empty);
    const uint64_t chunks = (n + 31) / 32;
    const unsigned grid = (unsigned)std::max<uint64_t>(
        1, std::min<uint64_t>((chunks + CV_THREADS / 32 - 1) / (CV_THREADS / 32), (uint64_t)c->sm_count * 16));
    if (t->canonical)
        k_coverage_short<true><<<grid, CV_THREADS, 0, c->stream>>>(dt, rd->d_codes, rd->d_inv, rd->d_rd_off, n, k,
                                                                   d_median, d_mean, d_stdev);
    else
        k_coverage_short<false><<<grid, CV_THREADS, 0, c->stream>>>(dt, rd->d_codes, rd->d_inv, rd->d_rd_off, n, k,
                                                                    d_median, d_mean, d_stdev);
    c->launches++;
    TK_TRY(check_launch(c, "coverage (no allocation)"));
    if (rd->max_len >= (uint32_t)k && rd->max_len - k + 1 > CV_WARP_MAX) {
        if (t->canonical)
            k_coverage_long_slab<true><<<NOALLOC_BLOCKS, CV_THREADS, 0, c->stream>>>(
                dt, rd->d_seq, rd->d_rd_off, n, k, scratch, d_median, d_mean, d_stdev);
        else
            k_coverage_long_slab<false><<<NOALLOC_BLOCKS, CV_THREADS, 0, c->stream>>>(
                dt, rd->d_seq, rd->d_rd_off, n, k, scratch, d_median, d_mean, d_stdev);
        c->launches++;
        TK_TRY(check_launch(c, "coverage long reads (no allocation)"));
    }
    return cuda_check(c, cudaStreamSynchronize(c->stream), "coverage (no allocation) sync");
}

}  // namespace tk

// Allocation-free coverage statistics; declared in include/trinkmer.h.
extern "C" int tk_coverage_stats_noalloc(tk_table *table, const tk_reads *reads, uint32_t *median, float *mean,
                                         float *stdev) {
    if (!table || !reads || !median || !mean || !stdev) return TK_E_INVAL;
    tk_ctx *c = table->ctx;
    if (cudaSetDevice(c->device) != cudaSuccess) return tk::set_err(c, TK_E_CUDA, "cudaSetDevice");
    if (reads->ctx != c) return tk::set_err(c, TK_E_INVAL, "read set and table belong to different contexts");
    return tk::coverage_stats_noalloc(table, reads, median, mean, stdev);
}
