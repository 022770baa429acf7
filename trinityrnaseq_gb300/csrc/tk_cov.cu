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
// median by a warp radix select (tk_warp.cuh).  Longer reads: one block per
// read, values in a global scratch slab, block bitonic sort.
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
// the cache holds answer ~70% of the lookups.  (Most lookups the cache
// misses are k-mers seen once, whose answer is 1.  A 32 or 64 MB bit filter
// of the keys whose count is not 1, consulted before the table, made the pass
// ~8% slower on GB300: its lines share L2 with the cache's, and a lookup that
// passes it pays two dependent loads.)
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
    int rbits;         // hash bits below the bucket index (<= 32): an entry is (those bits << 32) | count
};

// A bijection of [0, 2^n) (n <= 62): a three-round Feistel network over the
// key's two halves with 32-bit multiply-xorshift round functions, so every
// step (xor of one half with a function of the other) is invertible and the
// (bucket, remainder) pair identifies the key.  32-bit arithmetic keeps it to
// a dozen instructions.
__host__ __device__ __forceinline__ uint32_t feistel_f(uint32_t x, uint32_t m) {
    x *= m;
    return x ^ (x >> 15);
}

__host__ __device__ __forceinline__ uint64_t kmix_n(uint64_t key, int n) {
    const int hl = n >> 1, hh = n - hl;   // 1 <= hl <= hh <= 31
    const uint32_t ml = (uint32_t)((1ULL << hl) - 1), mh = (uint32_t)((1ULL << hh) - 1);
    uint32_t lo = (uint32_t)key & ml, hi = (uint32_t)(key >> hl) & mh;
    lo ^= feistel_f(hi, 0x9E3779B1u) & ml;
    hi ^= feistel_f(lo, 0x85EBCA77u) & mh;
    lo ^= feistel_f(hi, 0xC2B2AE3Du) & ml;
    return ((uint64_t)hi << hl) | lo;
}

// The cache's bucket of `key` and the 32-bit tag its entry carries.
__device__ __forceinline__ const uint64_t *cache_bucket(const CovCache &cc, uint64_t key, uint32_t *tag) {
    const uint64_t h = kmix_n(key, cc.n);
    *tag = (uint32_t)(h & ((1ULL << cc.rbits) - 1));
    return cc.ent + ((h >> cc.rbits) << 2);
}

// the count of the bucket entry tagged `tag`, or 0 (an entry's count is >= 2,
// so an empty entry matches nothing)
__device__ __forceinline__ uint32_t cache_match(const uint64_t *b, uint32_t tag) {
    uint64_t e0, e1, e2, e3, pol;
    // L2 evict-last: the cache's lines outlive the table lines streamed past them
    asm("createpolicy.fractional.L2::evict_last.b64 %0, 1.0;" : "=l"(pol));
    asm("ld.global.L2::cache_hint.v4.u64 {%0,%1,%2,%3}, [%4], %5;"
        : "=l"(e0), "=l"(e1), "=l"(e2), "=l"(e3)
        : "l"(b), "l"(pol));
    uint32_t c = 0;
    c = (uint32_t)(e0 >> 32) == tag ? (uint32_t)e0 : c;
    c = (uint32_t)(e1 >> 32) == tag ? (uint32_t)e1 : c;
    c = (uint32_t)(e2 >> 32) == tag ? (uint32_t)e2 : c;
    c = (uint32_t)(e3 >> 32) == tag ? (uint32_t)e3 : c;
    return c;
}

// the count of `key` for the statistics: the cache, else the table (1 when absent)
__device__ __forceinline__ uint32_t cov_lookup(const CovCache &cc, DevTable t, uint64_t key) {
    if (cc.ent) {
        uint32_t tag;
        const uint64_t *b = cache_bucket(cc, key, &tag);
        const uint32_t v = cache_match(b, tag);
        if (v) return v;
    }
    return tbl_get(t, key, 1u);
}

// Offers one (key, count) to its bucket: into an empty entry, else in place
// of the smallest count when larger.  A CAS lost to another thread re-reads
// the bucket; after 32 rounds the key is left out (the cache stays valid).
__device__ __forceinline__ void cache_offer(const CovCache &cc, uint64_t key, uint32_t count) {
    uint32_t tag;
    unsigned long long *b =
        reinterpret_cast<unsigned long long *>(const_cast<uint64_t *>(cache_bucket(cc, key, &tag)));
    const unsigned long long mine = ((unsigned long long)tag << 32) | count;
    for (int round = 0; round < 32; round++) {
        int at = 0;
        unsigned long long old = 0;
        uint32_t least = ~0u;
#pragma unroll
        for (int j = 0; j < 4; j++) {
            const unsigned long long e = *reinterpret_cast<volatile unsigned long long *>(b + j);
            const uint32_t c = (uint32_t)e;   // 0 for an empty entry
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
    for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < cap; i += stride) {
        const ulonglong2 s = __ldcs(reinterpret_cast<const ulonglong2 *>(slots + i));
        const uint32_t c = (uint32_t)s.y;
        if (s.x == EMPTY_KEY || c < 2) continue;
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
    if (n - hbits < 1 || n - hbits > 32) return TK_OK;   // tiny key spaces; k > 26 at 64 MB
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

// A read's windows in three stages.  Stage 1: the lane's keys and their
// validity, and the cache's count for each (0 = not in the cache).  Stage 2:
// the table for the windows the cache did not answer.  Stage 3: the read's
// statistics.  The lookups of a stage are independent loads issued together.
// (Pipelining two reads -- the next read's cache answers and table prefetches
// before the current read's statistics -- was 2.4x slower on GB300: the
// registers it holds across stages spill.)
template <int S, bool CANON>
__device__ __forceinline__ void cov_stage1(const CovCache &cc, const uint64_t *__restrict__ codes,
                                           const uint32_t *__restrict__ inv, uint64_t start, uint32_t nwin, int k,
                                           uint64_t (&key)[S], uint32_t (&v)[S], uint32_t &vm) {
    const uint32_t span = (nwin + 31) / 32;
    vm = 0;
    lane_windows_codes<S, CANON>(codes, inv, start, nwin, span, k, [&](int j, bool valid, uint64_t kk) {
        key[j] = kk;
        vm |= (valid ? 1u : 0u) << j;
    });
#pragma unroll
    for (int j = 0; j < S; j++) {
        v[j] = 0;
        if (cc.ent && ((vm >> j) & 1u)) {
            uint32_t tag;
            const uint64_t *b = cache_bucket(cc, key[j], &tag);
            v[j] = cache_match(b, tag);
        }
    }
}

template <int S>
__device__ __forceinline__ void cov_stage2(DevTable t, const uint64_t (&key)[S], uint32_t (&v)[S], uint32_t vm) {
#pragma unroll
    for (int j = 0; j < S; j++)
        if (((vm >> j) & 1u) && v[j] == 0) v[j] = tbl_get(t, key[j], 1u);
}

template <int S>
__device__ __forceinline__ ReadSums cov_stage3(const uint32_t (&v)[S], uint32_t vm) {
    ReadSums rs;
    rs.cnt = __reduce_add_sync(0xffffffffu, (uint32_t)__popc(vm));
    uint32_t lmax = 0;
#pragma unroll
    for (int j = 0; j < S; j++)
        if ((vm >> j) & 1u) lmax = max(lmax, v[j]);
    const uint32_t mx = __reduce_max_sync(0xffffffffu, lmax);
    if (mx < (1u << 23)) {
        // every count below 2^23: a lane's sum fits 32 bits and its sum of
        // squares 64 bits, and the warp totals (< 2^31 and < 2^54) are exact
        // through warp-wide adds of 16-bit pieces
        uint32_t sum = 0;
        uint64_t sq = 0;
#pragma unroll
        for (int j = 0; j < S; j++)
            if ((vm >> j) & 1u) {
                sum += v[j];
                sq += (uint64_t)v[j] * v[j];
            }
        rs.sum = __reduce_add_sync(0xffffffffu, sum);
        const uint64_t q0 = __reduce_add_sync(0xffffffffu, (uint32_t)(sq & 0xFFFF));
        const uint64_t q1 = __reduce_add_sync(0xffffffffu, (uint32_t)((sq >> 16) & 0xFFFF));
        const uint64_t q2 = __reduce_add_sync(0xffffffffu, (uint32_t)((sq >> 32) & 0xFFFF));
        const uint64_t q3 = __reduce_add_sync(0xffffffffu, (uint32_t)(sq >> 48));
        rs.lo = q0 + (q1 << 16) + (q2 << 32) + (q3 << 48);
        rs.hi = 0;
    } else {
        uint64_t sum = 0, hi = 0, lo = 0;
#pragma unroll
        for (int j = 0; j < S; j++)
            if ((vm >> j) & 1u) {
                sum += v[j];
                const uint64_t sq = (uint64_t)v[j] * v[j], nlo = lo + sq;
                hi += nlo < lo;
                lo = nlo;
            }
        rs.sum = warp_sum(sum);
        warp_sum_u128(hi, lo);
        rs.hi = hi;
        rs.lo = lo;
    }
    rs.med = rs.cnt ? warp_select<S>(v, vm, rs.cnt / 2, mx) : 0u;
    return rs;
}

template <int S, bool CANON>
__device__ __forceinline__ ReadSums cov_warp_read(const CovCache &cc, DevTable t, const uint64_t *__restrict__ codes,
                                                  const uint32_t *__restrict__ inv, uint64_t start, uint32_t nwin,
                                                  int k) {
    uint64_t key[S];
    uint32_t v[S], vm;
    cov_stage1<S, CANON>(cc, codes, inv, start, nwin, k, key, v, vm);
    cov_stage2<S>(t, key, v, vm);
    return cov_stage3<S>(v, vm);
}

// One warp, 32 consecutive reads [r0, r0 + 32): the warp computes each read's
// sums in turn and lane i keeps read r0 + i's; then every lane finishes its own
// read.  The floating-point finish runs on the FP64 pipe, whose cost is per
// warp instruction whatever the number of active lanes, so finishing 32 reads
// in one pass costs what one read alone would.  Reads with more than
// CV_WARP_MAX windows are appended to long_list (or, with no list, left to a
// separate pass) and not written here.  MAXS = the largest window class
// compiled in (windows per lane); a read set whose reads all have at most
// 32 * MAXS windows needs no larger one.
template <bool CANON, int MAXS = 8>
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
        else if (nwin <= 96) rs = cov_warp_read<3, CANON>(cc, t, codes, inv, start, nwin, k);
        else if (MAXS >= 4 && nwin <= 128) rs = cov_warp_read<(MAXS >= 4 ? 4 : 1), CANON>(cc, t, codes, inv, start, nwin, k);
        else if (MAXS >= 6 && nwin <= 192) rs = cov_warp_read<(MAXS >= 6 ? 6 : 1), CANON>(cc, t, codes, inv, start, nwin, k);
        else if (MAXS >= 8 && nwin <= CV_WARP_MAX) rs = cov_warp_read<(MAXS >= 8 ? 8 : 1), CANON>(cc, t, codes, inv, start, nwin, k);
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

// MAXS 3 / 4: read sets whose reads have at most 96 / 128 windows (up to 120 /
// 152 nt at k = 25), 8 blocks per SM; MAXS 8: every read, 6 blocks per SM.
template <bool CANON, int MAXS>
__global__ void __launch_bounds__(CV_THREADS, MAXS <= 4 ? 8 : 6) k_coverage(CovCache cc, DevTable t, const uint64_t *__restrict__ codes,
                                                        const uint32_t *__restrict__ inv,
                                                        const uint64_t *__restrict__ rd_off, uint64_t n_reads, int k,
                                                        uint32_t *__restrict__ median, float *__restrict__ mean,
                                                        float *__restrict__ stdev, uint32_t *__restrict__ long_list,
                                                        unsigned long long *__restrict__ long_n) {
    __shared__ ReadSums held[CV_THREADS];
    const uint64_t warps = (uint64_t)gridDim.x * (CV_THREADS / 32);
    const uint64_t chunks = (n_reads + 31) / 32;
    for (uint64_t ch = (uint64_t)blockIdx.x * (CV_THREADS / 32) + (threadIdx.x >> 5); ch < chunks; ch += warps)
        cov_warp_chunk<CANON, MAXS>(cc, t, codes, inv, rd_off, n_reads, k, ch * 32, median, mean, stdev, long_list,
                                    long_n, held + (threadIdx.x & ~31u));
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
        // one wave of resident blocks, each warp striding over the 32-read
        // chunks (a grid of several partial waves leaves SMs idle at its end)
        // the narrowest kernel that holds the longest read's windows
        static int per_sm[6] = {0, 0, 0, 0, 0, 0};
        const uint64_t max_win = rd->max_len >= (uint32_t)k ? rd->max_len - k + 1 : 0;
        const int ci = (t->canonical ? 1 : 0) + (max_win <= 96 ? 4 : max_win <= 128 ? 2 : 0);
        if (!per_sm[ci]) {
            int b = 0;
            switch (ci) {
            case 0: cudaOccupancyMaxActiveBlocksPerMultiprocessor(&b, k_coverage<false, 8>, CV_THREADS, 0); break;
            case 1: cudaOccupancyMaxActiveBlocksPerMultiprocessor(&b, k_coverage<true, 8>, CV_THREADS, 0); break;
            case 2: cudaOccupancyMaxActiveBlocksPerMultiprocessor(&b, k_coverage<false, 4>, CV_THREADS, 0); break;
            case 3: cudaOccupancyMaxActiveBlocksPerMultiprocessor(&b, k_coverage<true, 4>, CV_THREADS, 0); break;
            case 4: cudaOccupancyMaxActiveBlocksPerMultiprocessor(&b, k_coverage<false, 3>, CV_THREADS, 0); break;
            default: cudaOccupancyMaxActiveBlocksPerMultiprocessor(&b, k_coverage<true, 3>, CV_THREADS, 0); break;
            }
            per_sm[ci] = std::max(1, b);
        }
        const uint64_t chunks = (n + 31) / 32;
        const unsigned grid = (unsigned)std::max<uint64_t>(
            1, std::min<uint64_t>((chunks + CV_THREADS / 32 - 1) / (CV_THREADS / 32),
                                  (uint64_t)c->sm_count * (uint64_t)per_sm[ci]));
        cudaEvent_t ev;
        prof_begin(c, TK_KID_COVERAGE, &ev);
#define TK_COV_LAUNCH(C, M)                                                                                   \
    k_coverage<C, M><<<grid, CV_THREADS, 0, c->stream>>>(cc, dt, rd->d_codes, rd->d_inv, rd->d_rd_off, n, k, d_median, \
                                                         d_mean, d_stdev, long_list, long_n)
        switch (ci) {
        case 0: TK_COV_LAUNCH(false, 8); break;
        case 1: TK_COV_LAUNCH(true, 8); break;
        case 2: TK_COV_LAUNCH(false, 4); break;
        case 3: TK_COV_LAUNCH(true, 4); break;
        case 4: TK_COV_LAUNCH(false, 3); break;
        default: TK_COV_LAUNCH(true, 3); break;
        }
#undef TK_COV_LAUNCH
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
