// tk_table.cu -- the k-mer count table: K2 count-insert, HLL sizing, rehash,
// K3 filter/histogram, sorted dump and the K4 ">COUNT\nKMER\n" formatter,
// and catalogue loading (a stored database or a jellyfish-style dump).
//
// Replaces `jellyfish count/histo/dump` as Trinity drives them
// (Trinity:2612-2638, util/insilico_read_normalization.pl:617-643).
//
// K2 walks the packed read array as one flat stream: each thread owns 32
// window end positions, reads the 64 bytes [p0-32, p0+32) as four 16-byte
// vectors, and rolls the forward and reverse-complement 2-bit words in
// registers; a window is valid after k consecutive A/C/G/T, so read
// separators and N bases break k-mers with no per-read bookkeeping.  Lanes of
// a warp that hold the same key in the same step are merged (match.any) and
// the leader adds the multiplicity with one atomic.  A key that finds no slot
// within max_probes goes to an overflow list; the host then doubles the table
// and re-inserts it, so no k-mer is ever dropped silently.
#include "tk_internal.cuh"

#include <algorithm>
#include <cmath>
#include <cstdlib>

namespace tk {

constexpr int CT_THREADS = 256;
constexpr int CT_SPAN = 32;              // window end positions per thread
constexpr int HLL_P = 12;
constexpr int HLL_M = 1 << HLL_P;
constexpr int NBUCKETS = 1 << BUCKET_BITS;
constexpr int INS_PER_THREAD = 1;
// bucket passes: one 512-thread block per SM; each block stages up to
// SC_BUF keys per bucket in shared memory between flushes
constexpr int SC_THREADS = 512;
constexpr int SC_BUF = 24;                                       // a multiple of 4 (whole 32-byte sectors)
static_assert(SC_BUF % 4 == 0 && SC_BUF <= 32, "a half-warp flushes a bucket in two 16-key stores");
constexpr int SC_BUCKETS_PER_WARP = NBUCKETS / (SC_THREADS / 32);
static_assert((NBUCKETS / (SC_THREADS / 32)) % 2 == 0, "buckets are flushed in pairs");
constexpr size_t SC_SMEM = (size_t)NBUCKETS * SC_BUF * 8 + (size_t)NBUCKETS * 8 + (size_t)NBUCKETS * 4;
constexpr uint64_t INS_CHUNK = (uint64_t)CT_THREADS * INS_PER_THREAD;
enum NextMode { NEXT_NONE = 0, NEXT_FILL = 1, NEXT_PREFETCH = 2 };

// Windows of the 2-bit code form of a packed read array.  A thread owns the
// 32 window end positions [32w, 32w + 32); the 64 positions [32w - 32, 32w + 32)
// (code words w-1 and w, invalid bits likewise) hold every base those windows
// use (k <= 31).  Each window is cut out of the 128-bit code pair with one
// funnel shift, its reverse complement out of the pair's reverse complement,
// and it is valid when none of its k positions has its invalid bit set.
// Calls f(key) for every valid window, in position order.
template <bool CANON, typename F>
__device__ __forceinline__ void thread_windows(const uint64_t *__restrict__ codes, const uint32_t *__restrict__ inv,
                                               uint64_t w, bool active, int k, F &&f) {
    uint64_t hi = 0, lo = 0, m = ~0ULL;
    if (active) {
        hi = __ldg(codes + w - 1);
        lo = __ldg(codes + w);
        m = ((uint64_t)__ldg(inv + w - 1) << 32) | __ldg(inv + w);
    }
    // bit b of `bad`: some position among bits b .. b+k-1 of m (position
    // 32w - 32 + x sits at bit 63 - x) is not A/C/G/T
    uint64_t bad = 0, span = m;
    int sh = 0;
#pragma unroll
    for (int l = 0; l < 5; l++) {
        if (k & (1 << l)) {
            bad |= span >> sh;
            sh += 1 << l;
        }
        span |= span >> (1 << l);
    }
    // reverse complement of the 64 positions: complement, then reverse the
    // order of the 2-bit groups
    uint64_t rhi = __brevll(~lo), rlo = __brevll(~hi);
    rhi = ((rhi >> 1) & 0x5555555555555555ULL) | ((rhi & 0x5555555555555555ULL) << 1);
    rlo = ((rlo >> 1) & 0x5555555555555555ULL) | ((rlo & 0x5555555555555555ULL) << 1);
    const uint64_t kmask = (1ULL << (2 * k)) - 1;
#pragma unroll
    for (int i = 0; i < 32; i++) {
        if ((bad >> (31 - i)) & 1ULL) continue;
        // forward: the window ends at position 32 + i of the 64
        const int s = 62 - 2 * i;
        const uint64_t fw = (s ? ((lo >> s) | (hi << (64 - s))) : lo) & kmask;
        uint64_t key = fw;
        if (CANON) {
            // reverse complement: it ends where the window starts, 33 + i - k
            const int r = 66 + 2 * i - 2 * k;   // 4 .. 126
            const uint64_t rc = (r >= 64 ? (rhi >> (r - 64)) : ((rlo >> r) | (rhi << (64 - r)))) & kmask;
            key = rc < fw ? rc : fw;
        }
        f(key);
    }
}

// Pass 1a: k-mers per (hash bucket, column) and the HLL sketch of the batch.
// hist is bucket-major with `cols` columns per bucket; the read set uses the
// columns [col0, col0 + gridDim.x), one per block: hist[bucket * cols + col0 + block]
// (each read set has a histogram and key buffer of its own, col0 = 0).
// Each count is rounded up to a multiple of 4 keys, so every (bucket, column)
// region of the key buffer starts on a 32-byte sector; pass 1b pads the
// rounding with EMPTY_KEY, which the insert skips.  Pass 1b's block of
// SC_THREADS owns tiles b, b+G, b+2G, ... (G blocks); this pass covers the same
// tiles with two tiles at a time per block (HIST_THREADS = 2 x SC_THREADS), for
// twice the resident warps (pass 1b is held to one block per SM by its
// shared-memory staging).
constexpr int HIST_THREADS = 2 * SC_THREADS;
template <bool CANON>
__global__ void __launch_bounds__(HIST_THREADS) k_part_hist(const uint64_t *__restrict__ codes,
                                                           const uint32_t *__restrict__ inv, uint64_t n, int k,
                                                           uint32_t *__restrict__ hist, uint64_t cols, uint64_t col0,
                                                           uint32_t *__restrict__ regs,
                                                           unsigned long long *__restrict__ windows_out) {
    __shared__ uint32_t sh[NBUCKETS];
    __shared__ uint32_t sreg[HLL_M];
    for (int i = threadIdx.x; i < NBUCKETS; i += HIST_THREADS) sh[i] = 0;
    for (int i = threadIdx.x; i < HLL_M; i += HIST_THREADS) sreg[i] = 0;
    __syncthreads();
    uint32_t windows = 0;
    const uint64_t tile = (uint64_t)SC_THREADS * CT_SPAN;
    const uint32_t half = threadIdx.x / SC_THREADS, t = threadIdx.x % SC_THREADS;
    for (uint64_t base = ((uint64_t)blockIdx.x + (uint64_t)half * gridDim.x) * tile; base < n;
         base += 2ull * gridDim.x * tile) {
        const uint64_t p0 = base + (uint64_t)t * CT_SPAN;
        thread_windows<CANON>(codes, inv, p0 >> 5, p0 < n, k, [&](uint64_t key) {
            uint64_t h = mix64(key);
            atomicAdd(&sh[h >> (64 - BUCKET_BITS)], 1u);
            uint32_t idx = (uint32_t)(h & (HLL_M - 1));
            uint32_t rank = (uint32_t)__clzll((long long)(h >> HLL_P)) - HLL_P + 1u;
            if (rank > sreg[idx]) atomicMax(&sreg[idx], rank);
            windows++;
        });
    }
    __syncthreads();
    for (int i = threadIdx.x; i < NBUCKETS; i += HIST_THREADS) hist[(uint64_t)i * cols + col0 + blockIdx.x] = (sh[i] + 3u) & ~3u;
    for (int i = threadIdx.x; i < HLL_M; i += HIST_THREADS)
        if (sreg[i]) atomicMax(&regs[i], sreg[i]);
    windows = warp_sum(windows);
    if (lane_id() == 0 && windows) atomicAdd(windows_out, (unsigned long long)windows);
}

// Pass 1b: the same windows (same grid, same tiles as pass 1a), written
// bucket-major into the key buffer.  A random 8-byte store leaves its 32-byte
// sector partly written, and L2 then reads the sector from DRAM before it can
// write it back; so the keys of a tile are staged per bucket in shared memory
// and leave the block as whole, aligned sectors.  Per bucket the block keeps
// gpos (where its next staged key goes; a multiple of 4 keys) and cnt (keys
// staged, including up to 3 carried over from the previous tile).  A key
// ranked past SC_BUF in one tile (a bucket flooded by a repeat) is stored
// directly at its final position.  After each tile the warp that owns a
// bucket writes its whole sectors and moves the 0-3 key remainder to the
// front; at the end the remainders go out padded with EMPTY_KEY.
template <bool CANON>
__global__ void __launch_bounds__(SC_THREADS, 1) k_part_scatter(const uint64_t *__restrict__ codes,
                                                               const uint32_t *__restrict__ inv, uint64_t n, int k,
                                                               const uint64_t *__restrict__ offs, uint64_t cols,
                                                               uint64_t col0, uint64_t *__restrict__ keys) {
    extern __shared__ __align__(16) unsigned char sc_smem[];
    uint64_t *buf = reinterpret_cast<uint64_t *>(sc_smem);                       // [NBUCKETS][SC_BUF]
    unsigned long long *gpos = reinterpret_cast<unsigned long long *>(buf + (size_t)NBUCKETS * SC_BUF);
    uint32_t *cnt = reinterpret_cast<uint32_t *>(gpos + NBUCKETS);
    for (int i = threadIdx.x; i < NBUCKETS; i += SC_THREADS) {
        gpos[i] = offs[(uint64_t)i * cols + col0 + blockIdx.x];
        cnt[i] = 0;
    }
    __syncthreads();
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const uint64_t stride = (uint64_t)gridDim.x * SC_THREADS * CT_SPAN;
    for (uint64_t base = (uint64_t)blockIdx.x * SC_THREADS * CT_SPAN; base < n; base += stride) {
        const uint64_t p0 = base + (uint64_t)threadIdx.x * CT_SPAN;
        thread_windows<CANON>(codes, inv, p0 >> 5, p0 < n, k, [&](uint64_t key) {
            const uint32_t b = (uint32_t)(mix64(key) >> (64 - BUCKET_BITS));
            const uint32_t r = atomicAdd(&cnt[b], 1u);
            if (r < SC_BUF) buf[b * SC_BUF + r] = key;
            else keys[gpos[b] + r] = key;
        });
        __syncthreads();
        // two buckets per step, one per half-warp
        const unsigned hl = lane & 15u;
        for (int i = 0; i < SC_BUCKETS_PER_WARP; i += 2) {
            const int b = warp * SC_BUCKETS_PER_WARP + i + (int)(lane >> 4);
            const uint32_t nk = cnt[b];
            const uint32_t full = nk & ~3u;
            const uint64_t g = gpos[b];
            const uint64_t *bb = buf + (size_t)b * SC_BUF;
            const uint32_t nb = min(full, (uint32_t)SC_BUF);
            if (hl < nb) keys[g + hl] = bb[hl];
            if (hl + 16 < nb) keys[g + hl + 16] = bb[hl + 16];
            const uint32_t tail = nk - full;
            uint64_t v = 0;
            if (hl < tail) {
                const uint32_t idx = full + hl;
                v = idx < SC_BUF ? bb[idx] : __ldcg(keys + g + idx);
            }
            __syncwarp();
            if (hl < tail) buf[(size_t)b * SC_BUF + hl] = v;
            if (hl == 0) {
                cnt[b] = tail;
                gpos[b] = g + full;
            }
            __syncwarp();
        }
        __syncthreads();
    }
    for (int i = 0; i < SC_BUCKETS_PER_WARP; i++) {
        const int b = warp * SC_BUCKETS_PER_WARP + i;
        const uint32_t nk = cnt[b];
        if (nk && lane < 4) keys[gpos[b] + lane] = lane < nk ? buf[(size_t)b * SC_BUF + lane] : EMPTY_KEY;
    }
}

__device__ __forceinline__ void l2_prefetch_bulk(const void *p, uint32_t bytes) {
    asm volatile("cp.async.bulk.prefetch.L2.global [%0], %1;" ::"l"(p), "r"(bytes) : "memory");
}

// Pass 2, per partition p: a launch that prepares slice p (fill >= 0, p = -1)
// -- on a fresh table it writes the empty slots (those writes allocate in L2,
// so the slice is never read from DRAM); on a table that already holds keys it
// bulk-prefetches the slice to L2 -- then a launch that inserts partition p's
// keys (fill = -1).  Stream order between the launches is the only
// synchronisation.
__global__ void __launch_bounds__(CT_THREADS) k_part_step(const uint64_t *__restrict__ keys,
                                                         const uint64_t *__restrict__ offs, uint64_t cols, int p,
                                                         int fill, DevTable t, int next_mode, int max_probes,
                                                         uint64_t *__restrict__ ovf_keys, uint32_t *__restrict__ ovf_cnt,
                                                         uint64_t ovf_cap, unsigned long long *__restrict__ counters) {
    const int nparts = 1 << t.pbits;
    const uint64_t nslot = t.lmask + 1;
    if (fill >= 0 && fill < nparts) {
        Slot *nxt = t.slots + ((uint64_t)fill << t.lbits);
        if (next_mode == NEXT_FILL) {
            ulonglong2 e;
            e.x = EMPTY_KEY;
            e.y = 0;
            ulonglong2 *v = reinterpret_cast<ulonglong2 *>(nxt);
            for (uint64_t i = (uint64_t)blockIdx.x * CT_THREADS + threadIdx.x; i < nslot; i += (uint64_t)gridDim.x * CT_THREADS)
                v[i] = e;
        } else if (next_mode == NEXT_PREFETCH && threadIdx.x == 0) {
            const uint64_t bytes = nslot * sizeof(Slot);
            const uint64_t share = ((bytes + gridDim.x - 1) / gridDim.x + 15) & ~15ULL;
            uint64_t lo = (uint64_t)blockIdx.x * share;
            const uint64_t hi = min(bytes, lo + share);
            const char *base = reinterpret_cast<const char *>(nxt);
            for (int q = 0; q < 8 && lo < hi; q++) {   // 16-byte aligned start, multiple-of-16 size, <= 64 KB each
                uint64_t b = min(hi - lo, (uint64_t)65536);
                l2_prefetch_bulk(base + lo, (uint32_t)b);
                lo += b;
            }
        }
    }
    if (p < 0) return;
    const uint64_t bpp = (uint64_t)(NBUCKETS >> t.pbits);
    const uint64_t ps = offs[(uint64_t)p * bpp * cols];
    const uint64_t pe = offs[(uint64_t)(p + 1) * bpp * cols];
    for (uint64_t base = ps + (uint64_t)blockIdx.x * INS_CHUNK; base < pe; base += (uint64_t)gridDim.x * INS_CHUNK) {
        uint64_t kk[INS_PER_THREAD], s[INS_PER_THREAD];
        unsigned long long cur[INS_PER_THREAD];
#pragma unroll
        for (int j = 0; j < INS_PER_THREAD; j++) {
            uint64_t i = base + (uint64_t)j * CT_THREADS + threadIdx.x;
            kk[j] = i < pe ? __ldcs(keys + i) : EMPTY_KEY;
            s[j] = tbl_home(t, mix64(kk[j]));
        }
        // first probes of all keys issued back to back
#pragma unroll
        for (int j = 0; j < INS_PER_THREAD; j++) cur[j] = kk[j] != EMPTY_KEY ? tbl_claim(&t.slots[s[j]], kk[j]) : 0ULL;
#pragma unroll
        for (int j = 0; j < INS_PER_THREAD; j++) {
            if (kk[j] == EMPTY_KEY) continue;
            const uint64_t key = kk[j];
            uint64_t slot = s[j];
            unsigned long long c = cur[j];
            bool done = false;
            for (int probe = 0; probe < max_probes; probe++) {
                if (probe) c = tbl_claim(&t.slots[slot], key);
                if (c == key) {
                    atomicAdd(&t.slots[slot].val, 1u);
                    done = true;
                    break;
                }
                slot = tbl_next(t, slot);
            }
            if (!done) {
                unsigned long long o = atomicAdd(&counters[0], 1ULL);
                if (o < ovf_cap) { ovf_keys[o] = key; ovf_cnt[o] = 1u; }
            }
        }
    }
}

// ---- pass 2 by ranges (slices of at least 2^SR_MIN_LBITS slots).  Per
// partition p the keys are regrouped by the range of the slice their home slot
// falls in (a slice is cut into SR_BUILD_PER_SM ranges per SM, so that the
// build runs as one wave; k_sr_hist, k_sr_scatter), and one block per range then
// builds that range in shared memory (k_sr_build): it loads the range (all
// empty on a fresh table), inserts the range's keys with shared-memory CAS
// and add, and writes the range back whole.  A key whose probe run reaches the
// end of its range (its chain goes on into the next range, which another block
// owns) is merged into a small per-block table and then appended with its
// multiplicity to a deferred list that is inserted into the global table once
// every range is written; the global probe order (home, home+1, ... wrapping
// in the slice) is the one every reader uses, so the layout is an ordinary
// linear-probing table.  Global atomics drop from two per occurrence to the
// deferred keys alone, and a fresh slice needs no separate fill.
constexpr int SR_MIN_LBITS = 12;        // slices below 4096 slots keep the atomic path
// Two build blocks of 1024 threads per SM (32 registers, 110 KB of shared
// memory each) with ranges of up to 9200 slots: half the ranges per slice of
// four 512-thread blocks with 4600, so the regrouping passes' per-range work
// (counts, cursor atomics, runs) halves; 58.1 -> 50.9 ms per step at 20M pairs.
constexpr int SR_BUILD_PER_SM = 2;      // build blocks resident per SM: the slice is cut into one wave of ranges
constexpr int SR_MAX_SLOTS = 9200;      // slots of one range in shared memory (12 bytes each)
constexpr int SR_THREADS = 1024;        // regrouping passes (2 blocks per SM: few per-block range counts)
constexpr int SR_BUILD_THREADS = 1024;
constexpr int SR_MINI = 64;
constexpr size_t SR_SMEM = (size_t)(SR_MAX_SLOTS + SR_MINI) * 12;

// A slice of 2^lbits slots is cut into nsub ranges: slot s belongs to range
// floor(s * nsub / 2^lbits), so range r is [ceil(r 2^lbits / nsub),
// ceil((r+1) 2^lbits / nsub)).
__device__ __forceinline__ uint32_t slot_range(const DevTable &t, uint64_t s, uint32_t nsub) {
    return (uint32_t)((s * nsub) >> t.lbits);
}
__device__ __forceinline__ uint64_t range_first(const DevTable &t, uint32_t r, uint32_t nsub) {
    return (((uint64_t)r << t.lbits) + nsub - 1) / nsub;
}
__device__ __forceinline__ uint32_t key_range(const DevTable &t, uint64_t key, uint32_t nsub) {
    return slot_range(t, mix64(key) & t.lmask, nsub);
}

// A partition's keys: one segment of each read set's bucket buffer, taken
// as one sequence (index i of segment s is key cum[s] + i of the sequence).
struct KeySeg {
    const uint64_t *keys;
    uint64_t len;
};
constexpr int MAX_KEY_SEGS = (int)COUNT_MAX_SETS;   // read sets counted in one pass (more are counted in groups)

struct SegView {
    const uint64_t *ptr[MAX_KEY_SEGS];
    uint64_t cum[MAX_KEY_SEGS + 1];
    uint32_t n;
};

// Loads the partition's segment table into shared memory (all threads).
__device__ __forceinline__ void seg_view_load(SegView &v, const KeySeg *__restrict__ segs, uint32_t nseg) {
    if (threadIdx.x == 0) {
        uint64_t c = 0;
        for (uint32_t s = 0; s < nseg; s++) {
            v.ptr[s] = segs[s].keys;
            v.cum[s] = c;
            c += segs[s].len;
        }
        v.cum[nseg] = c;
        v.n = nseg;
    }
    __syncthreads();
}

// A thread's walk over ascending sequence indices: the current segment's
// pointer, first index and end in registers; shared memory is read only when
// the walk crosses into a later segment.
struct SegCursor {
    const uint64_t *ptr;
    uint64_t first, end;
    uint32_t s;
};

__device__ __forceinline__ void seg_cursor_at(const SegView &v, SegCursor &c, uint32_t s) {
    c.s = s;
    c.ptr = v.ptr[s];
    c.first = v.cum[s];
    c.end = v.cum[s + 1];
}

// Key i of the sequence (i at or after every index the cursor gave before).
__device__ __forceinline__ uint64_t seg_key(const SegView &v, SegCursor &c, uint64_t i) {
    while (i >= c.end && c.s + 1 < v.n) seg_cursor_at(v, c, c.s + 1);
    return __ldcs(c.ptr + (i - c.first));
}

// The segment holding sequence index i.
__device__ __forceinline__ uint32_t seg_of(const SegView &v, uint64_t i) {
    uint32_t s = 0;
    while (s + 1 < v.n && i >= v.cum[s + 1]) s++;
    return s;
}

// The partition's keys split evenly over the blocks.  Per block, keys per
// range (counts[range * gridDim.x + block]) and, summed over blocks after
// rounding each up to a multiple of 4, per range (totals, zeroed beforehand).
__global__ void __launch_bounds__(SR_THREADS) k_sr_hist(const KeySeg *__restrict__ segs, uint32_t nseg,
                                                       DevTable t, uint32_t nsub, uint32_t *__restrict__ counts,
                                                       uint32_t *__restrict__ totals) {
    extern __shared__ uint32_t sr_h[];
    __shared__ SegView sv;
    for (uint32_t i = threadIdx.x; i < nsub; i += SR_THREADS) sr_h[i] = 0;
    seg_view_load(sv, segs, nseg);   // synchronises
    const uint64_t n = sv.cum[sv.n];
    const uint64_t chunk = (n + gridDim.x - 1) / gridDim.x;
    const uint64_t lo = (uint64_t)blockIdx.x * chunk, hi = min(n, lo + chunk);
    SegCursor cur;
    seg_cursor_at(sv, cur, seg_of(sv, lo));
    for (uint64_t i0 = lo + threadIdx.x; i0 < hi; i0 += 4 * SR_THREADS) {
        uint64_t k4[4];
#pragma unroll
        for (int u = 0; u < 4; u++) {
            const uint64_t i = i0 + (uint64_t)u * SR_THREADS;   // ascending over u and over the loop
            k4[u] = i < hi ? seg_key(sv, cur, i) : EMPTY_KEY;
        }
#pragma unroll
        for (int u = 0; u < 4; u++)
            if (k4[u] != EMPTY_KEY) atomicAdd(&sr_h[key_range(t, k4[u], nsub)], 1u);
    }
    __syncthreads();
    for (uint32_t i = threadIdx.x; i < nsub; i += SR_THREADS) {
        counts[(uint64_t)i * gridDim.x + blockIdx.x] = sr_h[i];
        if (sr_h[i]) atomicAdd(&totals[i], (sr_h[i] + 3u) & ~3u);   // each block's run padded to whole sectors
    }
}

// exclusive prefix of totals[0..nsub) into out[0..nsub) (block-wide scan;
// thread t sums a run of consecutive ranges)
__device__ __forceinline__ void range_starts(const uint32_t *__restrict__ totals, uint32_t nsub, uint64_t *out) {
    __shared__ uint64_t sm[SR_THREADS / 32 + 1];
    const uint32_t per = (nsub + SR_THREADS - 1) / SR_THREADS;
    const uint32_t lo = min(nsub, threadIdx.x * per), hi = min(nsub, lo + per);
    uint64_t sum = 0;
    for (uint32_t j = lo; j < hi; j++) sum += totals[j];
    uint64_t tot;
    uint64_t run = block_excl_scan<uint64_t>(sum, sm, &tot);
    for (uint32_t j = lo; j < hi; j++) {
        out[j] = run;
        run += totals[j];
    }
    __syncthreads();
}

// The same keys into range order.  Each block reserves its share of every
// range (rounded up to whole 32-byte sectors) with one atomic on the range's
// cursor, counting-sorts its chunk by range in shared memory, and writes each
// range's run as whole sectors, the rounding filled with EMPTY_KEY (the build
// skips it).  Scattered single-key stores instead cost one L2 request per key.
constexpr int SRS_MAX = 12288;   // keys of one block's chunk (the host sizes the grid to fit)
static inline size_t SRS_SMEM(uint32_t nsub) { return (size_t)SRS_MAX * 8 + (size_t)nsub * 16; }

__global__ void __launch_bounds__(SR_THREADS) k_sr_scatter(const KeySeg *__restrict__ segs, uint32_t nseg,
                                                          DevTable t, uint32_t nsub, const uint32_t *__restrict__ counts,
                                                          const uint32_t *__restrict__ totals,
                                                          unsigned long long *__restrict__ cursor,
                                                          uint64_t *__restrict__ range_keys) {
    extern __shared__ __align__(16) unsigned char srs_smem[];
    uint64_t *skeys = reinterpret_cast<uint64_t *>(srs_smem);                          // [SRS_MAX]
    unsigned long long *gbase = reinterpret_cast<unsigned long long *>(skeys + SRS_MAX);  // [nsub]
    uint32_t *lstart = reinterpret_cast<uint32_t *>(gbase + nsub);                      // [nsub]
    uint32_t *lcur = lstart + nsub;                                                      // [nsub]
    __shared__ uint32_t sm[SR_THREADS / 32 + 1];
    __shared__ SegView sv;
    seg_view_load(sv, segs, nseg);   // synchronises
    range_starts(totals, nsub, reinterpret_cast<uint64_t *>(gbase));
    // this block's run of every range, and where its keys sit in shared memory
    const uint32_t per = (nsub + SR_THREADS - 1) / SR_THREADS;
    const uint32_t lo_r = min(nsub, threadIdx.x * per), hi_r = min(nsub, lo_r + per);
    uint32_t sum = 0;
    for (uint32_t r = lo_r; r < hi_r; r++) {
        const uint32_t mine = counts[(uint64_t)r * gridDim.x + blockIdx.x];
        if (mine) gbase[r] += atomicAdd(&cursor[r], (unsigned long long)((mine + 3u) & ~3u));
        lcur[r] = mine;
        sum += mine;
    }
    uint32_t tot;
    uint32_t run = block_excl_scan<uint32_t>(sum, sm, &tot);
    for (uint32_t r = lo_r; r < hi_r; r++) {
        lstart[r] = run;
        run += lcur[r];
        lcur[r] = 0;
    }
    __syncthreads();
    const uint64_t n = sv.cum[sv.n];
    const uint64_t chunk = (n + gridDim.x - 1) / gridDim.x;
    const uint64_t lo = (uint64_t)blockIdx.x * chunk, hi = min(n, lo + chunk);
    SegCursor cur;
    seg_cursor_at(sv, cur, seg_of(sv, lo));
    for (uint64_t i0 = lo + threadIdx.x; i0 < hi; i0 += 4 * SR_THREADS) {
        uint64_t k4[4];
#pragma unroll
        for (int u = 0; u < 4; u++) {
            const uint64_t i = i0 + (uint64_t)u * SR_THREADS;   // ascending over u and over the loop
            k4[u] = i < hi ? seg_key(sv, cur, i) : EMPTY_KEY;
        }
#pragma unroll
        for (int u = 0; u < 4; u++) {
            if (k4[u] == EMPTY_KEY) continue;
            const uint32_t r = key_range(t, k4[u], nsub);
            skeys[lstart[r] + atomicAdd(&lcur[r], 1u)] = k4[u];
        }
    }
    __syncthreads();
    // one warp per range at a time: consecutive lanes store consecutive keys
    const unsigned lane = lane_id();
    for (uint32_t r = threadIdx.x >> 5; r < nsub; r += SR_THREADS / 32) {
        const uint32_t n = lcur[r], n4 = (n + 3u) & ~3u;
        const uint64_t g = gbase[r];
        const uint32_t l0 = lstart[r];
        for (uint32_t j = lane; j < n4; j += 32) range_keys[g + j] = j < n ? skeys[l0 + j] : EMPTY_KEY;
    }
}

// Shared-memory probe from `loc` up to `end` in a table kept as separate key
// and count arrays (8-byte keys: a warp's random probes hit half as many banks
// per slot as 16-byte slots would); adds `inc` where the key lives or lands.
// A slot's key never changes once set, so a plain load that sees the key (most
// occurrences repeat a key already placed) needs only the add; an empty slot
// is claimed with CAS.  Returns false if the probe ran off the end.
__device__ __forceinline__ bool smem_add(unsigned long long *keys, uint32_t *vals, uint32_t loc, uint32_t end,
                                         uint64_t key, uint32_t inc) {
    for (; loc < end; loc++) {
        unsigned long long cur = *reinterpret_cast<volatile unsigned long long *>(&keys[loc]);
        if (cur == EMPTY_KEY) cur = atomicCAS(&keys[loc], EMPTY_KEY, (unsigned long long)key);
        if (cur == EMPTY_KEY || cur == key) {
            atomicAdd(&vals[loc], inc);
            return true;
        }
    }
    return false;
}

__global__ void __launch_bounds__(SR_BUILD_THREADS) k_sr_build(const uint64_t *__restrict__ range_keys,
                                                        const uint32_t *__restrict__ totals, uint32_t nsub, int p,
                                                        DevTable t, int fresh, uint32_t *__restrict__ next_totals,
                                                        unsigned long long *__restrict__ next_cursor,
                                                        uint64_t *__restrict__ defer_keys, uint32_t *__restrict__ defer_cnt,
                                                        uint64_t defer_cap, unsigned long long *__restrict__ defer_n) {
    extern __shared__ __align__(16) unsigned char sr_smem[];
    unsigned long long *tkey = reinterpret_cast<unsigned long long *>(sr_smem);   // [SR_MAX_SLOTS]
    unsigned long long *mkey = tkey + SR_MAX_SLOTS;                                // [SR_MINI]
    uint32_t *tval = reinterpret_cast<uint32_t *>(mkey + SR_MINI);                 // [SR_MAX_SLOTS]
    uint32_t *mval = tval + SR_MAX_SLOTS;                                          // [SR_MINI]
    __shared__ uint64_t ab[2];
    const uint32_t r = blockIdx.x;
    const uint64_t r0 = range_first(t, r, nsub);
    const uint32_t len = (uint32_t)(range_first(t, r + 1, nsub) - r0);   // <= SR_MAX_SLOTS (host checks)
    if (r == 0) {
        // the next partition's range counters (their last users finished before this launch)
        for (uint32_t i = threadIdx.x; i < nsub; i += SR_BUILD_THREADS) {
            next_totals[i] = 0;
            next_cursor[i] = 0;
        }
    }
    {
        // this range's keys: [start, start + total) of the range-ordered buffer
        uint64_t sum = 0;
        for (uint32_t i = threadIdx.x; i < r; i += SR_BUILD_THREADS) sum += totals[i];
        sum = warp_sum(sum);
        __shared__ uint64_t part[SR_BUILD_THREADS / 32];
        if (lane_id() == 0) part[threadIdx.x >> 5] = sum;
        __syncthreads();
        if (threadIdx.x == 0) {
            uint64_t a = 0;
            for (int w = 0; w < SR_BUILD_THREADS / 32; w++) a += part[w];
            ab[0] = a;
            ab[1] = a + totals[r];
        }
    }
    ulonglong2 *g = reinterpret_cast<ulonglong2 *>(t.slots + ((uint64_t)p << t.lbits) + r0);
    for (uint32_t i = threadIdx.x; i < len; i += SR_BUILD_THREADS) {
        if (fresh) {
            tkey[i] = EMPTY_KEY;
            tval[i] = 0;
        } else {
            const ulonglong2 v = g[i];
            tkey[i] = v.x;
            tval[i] = (uint32_t)v.y;
        }
    }
    for (int i = threadIdx.x; i < SR_MINI; i += SR_BUILD_THREADS) {
        mkey[i] = EMPTY_KEY;
        mval[i] = 0;
    }
    __syncthreads();
    const uint64_t a = ab[0], b = ab[1];
    for (uint64_t i0 = a + threadIdx.x; i0 < b; i0 += 4 * SR_BUILD_THREADS) {
        uint64_t k4[4];
#pragma unroll
        for (int u = 0; u < 4; u++) {
            const uint64_t i = i0 + (uint64_t)u * SR_BUILD_THREADS;
            k4[u] = i < b ? __ldcs(range_keys + i) : EMPTY_KEY;
        }
#pragma unroll
        for (int u = 0; u < 4; u++) {
            const uint64_t key = k4[u];
            if (key == EMPTY_KEY || smem_add(tkey, tval, (uint32_t)((mix64(key) & t.lmask) - r0), len, key, 1u)) continue;
            // the probe left the range: count it in the per-block table, or defer it singly
            const uint32_t m = (uint32_t)(mix64(key ^ 0x5851F42D4C957F2DULL) & (SR_MINI - 1));
            if (smem_add(mkey, mval, m, SR_MINI, key, 1u) || (m && smem_add(mkey, mval, 0, m, key, 1u))) continue;
            const unsigned long long j = atomicAdd(defer_n, 1ULL);
            if (j < defer_cap) {
                defer_keys[j] = key;
                defer_cnt[j] = 1u;
            }
        }
    }
    __syncthreads();
    for (uint32_t i = threadIdx.x; i < len; i += SR_BUILD_THREADS) {
        ulonglong2 v;
        v.x = tkey[i];
        v.y = tval[i];
        g[i] = v;
    }
    for (int i = threadIdx.x; i < SR_MINI; i += SR_BUILD_THREADS) {
        if (mkey[i] == EMPTY_KEY) continue;
        const unsigned long long j = atomicAdd(defer_n, 1ULL);
        if (j < defer_cap) {
            defer_keys[j] = mkey[i];
            defer_cnt[j] = mval[i];
        }
    }
}

__global__ void k_rehash(const Slot *__restrict__ old, uint64_t old_cap, DevTable t, int max_probes,
                         uint64_t *__restrict__ ovf_keys, uint32_t *__restrict__ ovf_cnt, uint64_t ovf_cap,
                         unsigned long long *__restrict__ counters) {
    for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < old_cap; i += (uint64_t)gridDim.x * blockDim.x) {
        ulonglong2 v = __ldcs(reinterpret_cast<const ulonglong2 *>(&old[i]));
        if (v.x == EMPTY_KEY) continue;
        if (!tbl_add(t, v.x, (uint32_t)v.y, max_probes)) {
            unsigned long long j = atomicAdd(&counters[0], 1ULL);
            if (j < ovf_cap) { ovf_keys[j] = v.x; ovf_cnt[j] = (uint32_t)v.y; }
        }
    }
}

__global__ void k_insert_pairs(const uint64_t *__restrict__ keys, const uint32_t *__restrict__ cnt, uint64_t n, DevTable t,
                               int max_probes, uint64_t *__restrict__ ovf_keys, uint32_t *__restrict__ ovf_cnt,
                               uint64_t ovf_cap, unsigned long long *__restrict__ counters) {
    for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (uint64_t)gridDim.x * blockDim.x) {
        uint64_t key = keys[i];
        uint32_t c = cnt ? cnt[i] : 1u;
        if (!tbl_add(t, key, c, max_probes)) {
            unsigned long long j = atomicAdd(&counters[0], 1ULL);
            if (j < ovf_cap) { ovf_keys[j] = key; ovf_cnt[j] = c; }
        }
    }
}

__global__ void k_fill_empty(Slot *slots, uint64_t cap, uint32_t init_val) {
    for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < cap; i += (uint64_t)gridDim.x * blockDim.x) {
        ulonglong2 v;
        v.x = EMPTY_KEY;
        v.y = init_val;
        reinterpret_cast<ulonglong2 *>(slots)[i] = v;
    }
}

__global__ void k_occupied(const Slot *__restrict__ slots, uint64_t cap, unsigned long long *out) {
    uint32_t n = 0;
    for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < cap; i += (uint64_t)gridDim.x * blockDim.x)
        n += __ldcs(&slots[i].key) != EMPTY_KEY;
    n = warp_sum(n);
    if (lane_id() == 0 && n) atomicAdd(out, (unsigned long long)n);
}

// K3: keys with count >= min_count.  A block takes a chunk of CP_ITEMS slots
// per thread, ranks its selected slots with a block scan and reserves their
// output range with one atomicAdd per chunk (a per-warp counter atomic on one
// address serialises in L2 on a 2G-slot table).  Output order is fixed by the
// sort that follows.
constexpr int CP_ITEMS = 16;

__global__ void __launch_bounds__(256) k_compact(const Slot *__restrict__ slots, uint64_t cap, uint32_t min_count,
                                                 uint64_t *__restrict__ okeys, uint32_t *__restrict__ ovals,
                                                 unsigned long long *__restrict__ n_out) {
    __shared__ uint32_t sm[256 / 32 + 1];
    __shared__ unsigned long long s_base;
    const uint64_t chunk = (uint64_t)blockDim.x * CP_ITEMS;
    for (uint64_t base = (uint64_t)blockIdx.x * chunk; base < cap; base += (uint64_t)gridDim.x * chunk) {
        ulonglong2 v[CP_ITEMS];
        uint32_t nsel = 0;
#pragma unroll
        for (int j = 0; j < CP_ITEMS; j++) {
            const uint64_t i = base + (uint64_t)j * blockDim.x + threadIdx.x;   // coalesced, striped
            v[j].x = EMPTY_KEY;
            v[j].y = 0;
            if (i < cap) v[j] = __ldcs(reinterpret_cast<const ulonglong2 *>(&slots[i]));
            nsel += v[j].x != EMPTY_KEY && (uint32_t)v[j].y >= min_count;
        }
        uint32_t tot;
        uint32_t pre = block_excl_scan<uint32_t>(nsel, sm, &tot);
        if (tot == 0) continue;                   // uniform over the block
        if (threadIdx.x == 0) s_base = atomicAdd(n_out, (unsigned long long)tot);
        __syncthreads();
        uint64_t o = s_base + pre;
#pragma unroll
        for (int j = 0; j < CP_ITEMS; j++) {
            if (v[j].x != EMPTY_KEY && (uint32_t)v[j].y >= min_count) {
                okeys[o] = v[j].x;
                ovals[o] = (uint32_t)v[j].y;
                o++;
            }
        }
        __syncthreads();
    }
}

// jellyfish histo bins: [0] below low, [1 + c - low], [nb - 1] above high
__global__ void k_histo(const Slot *__restrict__ slots, uint64_t cap, uint64_t low, uint64_t high,
                        unsigned long long *__restrict__ hist, int use_smem) {
    extern __shared__ uint32_t sh[];
    const uint64_t nb = high - low + 3;
    if (use_smem) {
        for (uint64_t i = threadIdx.x; i < nb; i += blockDim.x) sh[i] = 0;
        __syncthreads();
    }
    for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < cap; i += (uint64_t)gridDim.x * blockDim.x) {
        ulonglong2 v = __ldcs(reinterpret_cast<const ulonglong2 *>(&slots[i]));
        if (v.x == EMPTY_KEY) continue;
        uint64_t c = (uint32_t)v.y;
        uint64_t bin = c < low ? 0 : (c > high ? nb - 1 : 1 + c - low);
        if (use_smem) atomicAdd(&sh[bin], 1u);
        else atomicAdd(&hist[bin], 1ULL);
    }
    if (use_smem) {
        __syncthreads();
        for (uint64_t i = threadIdx.x; i < nb; i += blockDim.x)
            if (sh[i]) atomicAdd(&hist[i], (unsigned long long)sh[i]);
    }
}

__device__ __forceinline__ uint32_t dec_digits(uint32_t v) {
    uint32_t d = 1;
    while (v >= 10) { v /= 10; d++; }
    return d;
}

// K4 pass 1: record lengths ">" digits "\n" k "\n"
__global__ void k_dump_len(const uint32_t *__restrict__ cnt, uint64_t n, int k, uint32_t *__restrict__ len) {
    uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) len[i] = 3u + dec_digits(cnt[i]) + (uint32_t)k;
}

// K4 pass 2: each lane formats one record into its warp's shared-memory
// buffer, then the warp stores the 32 records' bytes contiguously (every store
// instruction covers 32 consecutive bytes).
constexpr int DW_THREADS = 256;
constexpr int DW_WARP_BYTES = 32 * (3 + 10 + MAX_K);

__global__ void __launch_bounds__(DW_THREADS) k_dump_write(const uint64_t *__restrict__ keys,
                                                          const uint32_t *__restrict__ cnt,
                                                          const uint64_t *__restrict__ off, uint64_t n, int k,
                                                          uint64_t total, char *__restrict__ out) {
    __shared__ char buf[DW_THREADS / 32][DW_WARP_BYTES];
    const unsigned lane = lane_id(), warp = threadIdx.x >> 5;
    const uint64_t i0 = (uint64_t)blockIdx.x * DW_THREADS + warp * 32;   // first record of this warp
    if (i0 >= n) return;
    const uint64_t i = i0 + lane;
    const uint64_t w0 = off[i0];
    char *p = buf[warp];
    if (i < n) {
        p += off[i] - w0;
        uint32_t c = cnt[i];
        uint32_t nd = dec_digits(c);
        p[0] = '>';
        for (int d = (int)nd; d >= 1; d--) { p[d] = (char)('0' + c % 10); c /= 10; }
        p[nd + 1] = '\n';
        uint64_t key = keys[i];
        char *q = p + nd + 2;
        for (int j = 0; j < k; j++) q[j] = "ACGT"[(key >> (2 * (k - 1 - j))) & 3];
        q[k] = '\n';
    }
    __syncwarp();
    const uint64_t last = min(i0 + 32, n);
    const uint64_t w1 = last < n ? off[last] : total;
    for (uint64_t b = lane; b < w1 - w0; b += 32) out[w0 + b] = buf[warp][b];
}

// dump records parsed as reads: name = decimal count, sequence = k-mer
__global__ void k_load_dump(const char *__restrict__ text, const uint64_t *__restrict__ name_off,
                            const uint32_t *__restrict__ name_len, const uint8_t *__restrict__ seq,
                            const uint64_t *__restrict__ rd_off, uint64_t n, int k, int canonical,
                            uint64_t *__restrict__ keys, uint32_t *__restrict__ cnt, uint32_t *__restrict__ err) {
    uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const char *h = text + name_off[i];
    uint32_t hl = name_len[i];
    uint64_t c = 0;
    bool bad = hl == 0;
    for (uint32_t j = 0; j < hl; j++) {
        uint32_t d = (uint8_t)h[j] - (uint32_t)'0';
        if (d > 9) { bad = true; break; }
        c = c * 10 + d;
        if (c > 0xFFFFFFFFull) c = 0xFFFFFFFFull;
    }
    uint64_t s = rd_off[i], L = rd_off[i + 1] - s - 1;
    if (L != (uint64_t)k) bad = true;
    uint64_t fw = 0, rc = 0;
    if (!bad) {
        for (int j = 0; j < k; j++) {
            uint32_t b = base_code(seq[s + j]);
            if (b > 3) { bad = true; break; }
            fw = (fw << 2) | b;
            rc |= (uint64_t)(3u - b) << (2 * j);
        }
    }
    if (bad) {
        atomicExch(&err[DE_PARSE], 1u);
        atomicMin(&err[DE_PARSE + 1], (uint32_t)min((uint64_t)0xFFFFFFFEull, i + 1));
        keys[i] = EMPTY_KEY;
        cnt[i] = 0;
        return;
    }
    keys[i] = (canonical && rc < fw) ? rc : fw;
    cnt[i] = (uint32_t)c;
}

// drop EMPTY keys written for bad records (there are none when err is clear)
static inline unsigned grid_for(uint64_t n, int threads) { return (unsigned)((n + threads - 1) / threads); }

static unsigned stream_grid(tk_ctx *c, uint64_t n, int threads) {
    uint64_t g = (n + threads - 1) / threads;
    uint64_t cap = (uint64_t)c->sm_count * 8;
    return (unsigned)std::max<uint64_t>(1, std::min(g, cap));
}

// ------------------------------------------------------------------ host side

// fill = false leaves the slots unwritten: the partitioned count pass fills
// each slice right before its inserts (a "fresh" table)
static int table_alloc_geom(tk_table *t, uint64_t capacity, uint32_t init_val, bool fill) {
    tk_ctx *c = t->ctx;
    Slot *s = nullptr;
    TK_TRY(dmalloc(c, (void **)&s, capacity * sizeof(Slot), "k-mer table"));
    if (fill) {
        k_fill_empty<<<stream_grid(c, capacity, 256), 256, 0, c->stream>>>(s, capacity, init_val);
        c->launches++;
    }
    t->fresh = !fill;
    int bits = 0;
    while ((1ULL << bits) < capacity) bits++;
    int lbits = std::min(bits, MAX_LBITS);
    if (bits - lbits > BUCKET_BITS) lbits = bits - BUCKET_BITS;   // > 2^33 slots: larger partitions
    t->t.slots = s;
    t->t.lbits = lbits;
    t->t.pbits = bits - lbits;
    t->t.lmask = (1ULL << lbits) - 1;
    t->capacity = capacity;
    return check_launch(c, "table fill");
}

int table_alloc_init(tk_table *t, uint64_t capacity, uint32_t init_val) {
    return table_alloc_geom(t, capacity, init_val, true);
}

int table_alloc(tk_table *t, uint64_t capacity) { return table_alloc_geom(t, capacity, 0, true); }

static int overflow_reset(tk_table *t) {
    return cuda_check(t->ctx, cudaMemsetAsync(t->d_counters, 0, sizeof(unsigned long long), t->ctx->stream), "ovf reset");
}

static int overflow_read(tk_table *t, unsigned long long *n) {
    tk_ctx *c = t->ctx;
    TK_CUDA(c, cudaMemcpyAsync(n, t->d_counters, sizeof(unsigned long long), cudaMemcpyDeviceToHost, c->stream));
    TK_CUDA(c, cudaStreamSynchronize(c->stream));
    return TK_OK;
}

// Moves every entry to a table of new_capacity slots.
int table_rehash(tk_table *t, uint64_t new_capacity) {
    tk_ctx *c = t->ctx;
    for (int attempt = 0; attempt < 8; attempt++) {
        Slot *old = t->t.slots;
        const DevTable old_t = t->t;
        uint64_t old_cap = t->capacity;
        TK_TRY(table_alloc(t, new_capacity));
        TK_TRY(overflow_reset(t));
        if (old) {
            k_rehash<<<stream_grid(c, old_cap, 256), 256, 0, c->stream>>>(old, old_cap, t->t, c->max_probes, t->d_ovf,
                                                                           (uint32_t *)(t->d_ovf + t->ovf_cap), t->ovf_cap,
                                                                           t->d_counters);
            c->launches++;
        }
        unsigned long long ovf = 0;
        TK_TRY(overflow_read(t, &ovf));
        if (ovf == 0) {
            dfree(c, old);
            return TK_OK;
        }
        // a probe run too long even in the larger table: go bigger from the old copy
        dfree(c, t->t.slots);
        t->t = old_t;
        t->capacity = old_cap;
        new_capacity *= 2;
    }
    return set_err(c, TK_E_TABLE_FULL, "rehash could not place every key");
}

// Re-inserts the overflow list after doubling the table, until it drains.
static int drain_overflow(tk_table *t) {
    tk_ctx *c = t->ctx;
    for (int round = 0; round < 8; round++) {
        unsigned long long ovf = 0;
        TK_TRY(overflow_read(t, &ovf));
        if (ovf == 0) return TK_OK;
        if (ovf > t->ovf_cap)
            return set_err(c, TK_E_TABLE_FULL,
                           "table overflow list overran (" + std::to_string(ovf) + " keys); create the table with a larger capacity");
        // copy the pending pairs aside, grow, and insert them
        uint64_t *pk = nullptr;
        uint32_t *pc = nullptr;
        TK_TRY(dmalloc(c, (void **)&pk, ovf * 8, "overflow keys"));
        int e = dmalloc(c, (void **)&pc, ovf * 4, "overflow counts");
        if (!e) {
            cudaMemcpyAsync(pk, t->d_ovf, ovf * 8, cudaMemcpyDeviceToDevice, c->stream);
            cudaMemcpyAsync(pc, t->d_ovf + t->ovf_cap, ovf * 4, cudaMemcpyDeviceToDevice, c->stream);
            e = table_rehash(t, t->capacity * 2);
        }
        if (!e) e = overflow_reset(t);
        if (!e) {
            k_insert_pairs<<<stream_grid(c, ovf, 256), 256, 0, c->stream>>>(pk, pc, ovf, t->t, c->max_probes, t->d_ovf,
                                                                             (uint32_t *)(t->d_ovf + t->ovf_cap), t->ovf_cap,
                                                                             t->d_counters);
            c->launches++;
            e = check_launch(c, "overflow insert");
        }
        dfree(c, pk);
        dfree(c, pc);
        if (e) return e;
    }
    return set_err(c, TK_E_TABLE_FULL, "overflow did not drain");
}

static double hll_estimate(const uint32_t *regs) {
    double sum = 0;
    int zeros = 0;
    for (int i = 0; i < HLL_M; i++) {
        sum += std::ldexp(1.0, -(int)regs[i]);
        zeros += regs[i] == 0;
    }
    double m = HLL_M, alpha = 0.7213 / (1.0 + 1.079 / m);
    double est = alpha * m * m / sum;
    if (est <= 2.5 * m && zeros) est = m * std::log(m / zeros);
    return est;
}

static uint64_t pow2_at_least(uint64_t x) {
    uint64_t p = 1024;
    while (p < x) p <<= 1;
    return p;
}

// Pass 2 with global atomics, one partition after another: a launch prepares
// slice p (fills a fresh slice, or prefetches a filled one to L2), then a
// launch CAS-probes and adds partition p's keys into it.  Preparing slice p+1
// inside the insert of p instead (the writes of one slice competing in L2 with
// the atomics on the other) measured ~12% slower.
static int count_by_atomics(tk_table *t, const std::vector<BucketKeys> &bk) {
    tk_ctx *c = t->ctx;
    const int nparts = 1 << t->t.pbits;
    const int mode = t->fresh ? NEXT_FILL : (t->t.pbits > 0 ? NEXT_PREFETCH : NEXT_NONE);
    const unsigned igrid = (unsigned)c->sm_count * 8;
    for (int p = 0; p < nparts; p++) {
        if (mode != NEXT_NONE) {   // slice p filled (fresh) or prefetched once, then every set's keys of partition p
            k_part_step<<<igrid, CT_THREADS, 0, c->stream>>>(bk[0].keys, bk[0].offs, bk[0].cols, -1, p, t->t, mode,
                                                             c->max_probes, t->d_ovf, (uint32_t *)(t->d_ovf + t->ovf_cap),
                                                             t->ovf_cap, t->d_counters);
            c->launches++;
        }
        for (const BucketKeys &b : bk) {
            if (!b.keys) continue;
            k_part_step<<<igrid, CT_THREADS, 0, c->stream>>>(b.keys, b.offs, b.cols, p, -1, t->t, mode, c->max_probes,
                                                             t->d_ovf, (uint32_t *)(t->d_ovf + t->ovf_cap), t->ovf_cap,
                                                             t->d_counters);
            c->launches++;
        }
    }
    return check_launch(c, "count insert");
}

// Pass 2 by ranges on a fresh table (see k_sr_build).  *done is false when
// the deferred list overran its capacity: the table is then emptied again and
// the caller counts with count_by_atomics instead, so nothing is lost.
static int count_by_ranges(tk_table *t, const std::vector<BucketKeys> &bk, bool *done) {
    tk_ctx *c = t->ctx;
    *done = false;
    const int nparts = 1 << t->t.pbits;
    // ranges per slice: one wave of SR_BUILD_PER_SM build blocks per SM, more if a range
    // would not fit in shared memory
    const uint64_t slice = 1ULL << t->t.lbits, wave = (uint64_t)c->sm_count * SR_BUILD_PER_SM;
    uint32_t nsub;
    if (slice / 1024 < wave) nsub = (uint32_t)(slice / 1024);   // a small slice: ranges of 1024 slots
    else nsub = (uint32_t)(wave * ((slice + wave * SR_MAX_SLOTS - 1) / (wave * SR_MAX_SLOTS)));   // whole waves
    const uint64_t bpp = (uint64_t)(NBUCKETS >> t->t.pbits);
    // partition boundaries on the host: the first offset of each partition's
    // buckets in each set's buffer; partition p's keys are one segment of each
    const uint32_t nsets = (uint32_t)bk.size();
    std::vector<std::vector<uint64_t>> pb(nsets, std::vector<uint64_t>(nparts + 1));
    for (uint32_t q = 0; q < nsets; q++)
        if (bk[q].keys)
            TK_CUDA(c, cudaMemcpy2DAsync(pb[q].data(), 8, bk[q].offs, bpp * bk[q].cols * 8, 8, nparts + 1,
                                         cudaMemcpyDeviceToHost, c->stream));
    TK_CUDA(c, cudaStreamSynchronize(c->stream));
    std::vector<KeySeg> segs((size_t)nparts * nsets);
    uint64_t max_part = 0, all_keys = 0;
    for (int p = 0; p < nparts; p++) {
        uint64_t part = 0;
        for (uint32_t q = 0; q < nsets; q++) {
            KeySeg &g = segs[(size_t)p * nsets + q];
            g.keys = bk[q].keys ? bk[q].keys + pb[q][p] : nullptr;
            g.len = bk[q].keys ? pb[q][p + 1] - pb[q][p] : 0;
            part += g.len;
        }
        max_part = std::max(max_part, part);
        all_keys += part;
    }
    // blocks of the regrouping passes: two per SM, more if a block's chunk
    // would not fit in the scatter's shared memory (rounding that up to whole
    // waves of two blocks per SM was slower: 52.5 against 50.9 ms per step)
    const unsigned G = (unsigned)std::max<uint64_t>((uint64_t)c->sm_count * 2, (max_part + SRS_MAX - 1) / SRS_MAX);
    const uint64_t cells = (uint64_t)nsub * G;
    uint64_t defer_cap = std::max<uint64_t>(1u << 16, std::min<uint64_t>(all_keys / 64, 1u << 24));
    if (const char *v = getenv("TRINKMER_DEFER_CAP")) defer_cap = std::max<uint64_t>(1, strtoull(v, nullptr, 10));   // tests: force the fallback
    uint64_t *range_keys = nullptr, *defer_keys = nullptr;
    uint32_t *counts = nullptr, *defer_cnt = nullptr, *totals = nullptr;
    unsigned long long *defer_n = nullptr, *cursor = nullptr;
    KeySeg *d_segs = nullptr;
    // a partition's keys plus the sector rounding of every (range, block) run
    int e = dmalloc(c, (void **)&range_keys, (max_part + 3 * cells + 1) * 8, "range keys");
    if (!e) e = dmalloc(c, (void **)&d_segs, segs.size() * sizeof(KeySeg), "partition segments");
    if (!e) e = cuda_check(c, cudaMemcpyAsync(d_segs, segs.data(), segs.size() * sizeof(KeySeg), cudaMemcpyHostToDevice,
                                              c->stream), "partition segments h2d");
    if (!e) e = dmalloc(c, (void **)&counts, cells * 4, "range counts");
    if (!e) e = dmalloc(c, (void **)&totals, 2ull * nsub * 4, "range totals");
    if (!e) e = dmalloc(c, (void **)&cursor, 2ull * nsub * 8, "range cursors");
    if (!e) e = dmalloc(c, (void **)&defer_keys, defer_cap * 8, "deferred keys");
    if (!e) e = dmalloc(c, (void **)&defer_cnt, defer_cap * 4, "deferred counts");
    if (!e) e = dmalloc(c, (void **)&defer_n, 8, "deferred count");
    if (!e) e = cuda_check(c, cudaMemsetAsync(defer_n, 0, 8, c->stream), "defer reset");
    if (!e) e = cuda_check(c, cudaMemsetAsync(totals, 0, 2ull * nsub * 4, c->stream), "totals reset");
    if (!e) e = cuda_check(c, cudaMemsetAsync(cursor, 0, 2ull * nsub * 8, c->stream), "cursor reset");
    if (!e) e = cuda_check(c, cudaFuncSetAttribute(k_sr_build, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)SR_SMEM),
                           "range build smem");
    if (!e) e = cuda_check(c, cudaFuncSetAttribute(k_sr_scatter, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                                   (int)SRS_SMEM(nsub)), "range scatter smem");
    for (int p = 0; !e && p < nparts; p++) {
        uint64_t part = 0;
        for (uint32_t q = 0; q < nsets; q++) part += segs[(size_t)p * nsets + q].len;
        const KeySeg *ps = d_segs + (size_t)p * nsets;
        uint32_t *tot = totals + (uint64_t)(p & 1) * nsub, *tot_next = totals + (uint64_t)((p + 1) & 1) * nsub;
        unsigned long long *cur = cursor + (uint64_t)(p & 1) * nsub, *cur_next = cursor + (uint64_t)((p + 1) & 1) * nsub;
        if (part) {
            k_sr_hist<<<G, SR_THREADS, nsub * 4, c->stream>>>(ps, nsets, t->t, nsub, counts, tot);
            k_sr_scatter<<<G, SR_THREADS, SRS_SMEM(nsub), c->stream>>>(ps, nsets, t->t, nsub, counts, tot, cur, range_keys);
            c->launches += 2;
        }
        k_sr_build<<<nsub, SR_BUILD_THREADS, SR_SMEM, c->stream>>>(range_keys, tot, nsub, p, t->t, 1, tot_next, cur_next,
                                                             defer_keys, defer_cnt, defer_cap, defer_n);
        c->launches++;
    }
    unsigned long long nd = 0;
    if (!e) e = check_launch(c, "range build");
    if (!e) e = cuda_check(c, cudaMemcpyAsync(&nd, defer_n, 8, cudaMemcpyDeviceToHost, c->stream), "defer d2h");
    if (!e) e = cuda_check(c, cudaStreamSynchronize(c->stream), "defer sync");
    if (!e && nd > defer_cap) {
        // the deferred list overran: empty the table again and count with atomics
        k_fill_empty<<<stream_grid(c, t->capacity, 256), 256, 0, c->stream>>>(t->t.slots, t->capacity, 0);
        c->launches++;
        t->fresh = false;
        e = check_launch(c, "table refill");
    } else if (!e) {
        t->fresh = false;
        if (nd) {
            k_insert_pairs<<<stream_grid(c, nd, 256), 256, 0, c->stream>>>(defer_keys, defer_cnt, nd, t->t, c->max_probes,
                                                                            t->d_ovf, (uint32_t *)(t->d_ovf + t->ovf_cap),
                                                                            t->ovf_cap, t->d_counters);
            c->launches++;
            e = check_launch(c, "deferred insert");
        }
        if (!e) *done = true;
    }
    dfree(c, range_keys);
    if (d_segs) dfree(c, d_segs);
    dfree(c, counts);
    dfree(c, totals);
    dfree(c, cursor);
    dfree(c, defer_keys);
    dfree(c, defer_cnt);
    dfree(c, defer_n);
    return e;
}

// Pass 1 for one read set: the bucket histogram of its windows with the HLL
// sketch (a union into t->d_hll) and the window count (added to
// t->d_counters[1]), then its windows into a key buffer of its own, bucket
// by bucket.  The two kernels use one fixed grid, so every tile goes to the
// same block (histogram column) in both.
int table_bucket_pass(tk_table *t, const tk_reads *r, BucketKeys *out) {
    tk_ctx *c = t->ctx;
    *out = BucketKeys();
    const uint64_t len = r->seq_len;
    if (len == 0) return TK_OK;
    const uint64_t tile = (uint64_t)SC_THREADS * CT_SPAN;
    const unsigned grid = (unsigned)std::max<uint64_t>(1, std::min<uint64_t>((len + tile - 1) / tile, (uint64_t)c->sm_count));
    const uint64_t cols = grid, cells = (uint64_t)NBUCKETS * cols;
    uint32_t *hist = nullptr;
    uint64_t *offs = nullptr, *keys = nullptr;
    TK_TRY(dmalloc(c, (void **)&hist, cells * 4, "bucket histogram"));
    int e = dmalloc(c, (void **)&offs, (cells + 1) * 8, "bucket offsets");
    cudaEvent_t ev;
    if (!e) {
        prof_begin(c, TK_KID_HLL, &ev);
        if (t->canonical)
            k_part_hist<true><<<grid, HIST_THREADS, 0, c->stream>>>(r->d_codes, r->d_inv, len, t->k, hist, cols, 0,
                                                                  t->d_hll, t->d_counters + 1);
        else
            k_part_hist<false><<<grid, HIST_THREADS, 0, c->stream>>>(r->d_codes, r->d_inv, len, t->k, hist, cols, 0,
                                                                   t->d_hll, t->d_counters + 1);
        c->launches++;
        prof_end(c, TK_KID_HLL, ev, len);
        e = check_launch(c, "bucket histogram");
    }
    // key-buffer entries: the windows plus the EMPTY_KEY padding of every
    // region (0 exactly when the set has no windows)
    uint64_t padded = 0;
    if (!e) e = scan_excl_u32_to_u64(c, hist, offs, cells, &padded);   // synchronises
    if (!e && padded) {
        cudaMemcpyAsync(offs + cells, &padded, 8, cudaMemcpyHostToDevice, c->stream);
        e = dmalloc(c, (void **)&keys, padded * 8, "bucketed k-mers");
        static_assert(SC_SMEM <= 227 * 1024, "bucket staging exceeds shared memory");
        if (!e) e = cuda_check(c, cudaFuncSetAttribute(k_part_scatter<true>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                                       (int)SC_SMEM), "scatter smem");
        if (!e) e = cuda_check(c, cudaFuncSetAttribute(k_part_scatter<false>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                                       (int)SC_SMEM), "scatter smem");
        if (!e) {
            prof_begin(c, TK_KID_SCATTER, &ev);
            if (t->canonical)
                k_part_scatter<true><<<grid, SC_THREADS, SC_SMEM, c->stream>>>(r->d_codes, r->d_inv, len, t->k, offs, cols,
                                                                              0, keys);
            else
                k_part_scatter<false><<<grid, SC_THREADS, SC_SMEM, c->stream>>>(r->d_codes, r->d_inv, len, t->k, offs, cols,
                                                                               0, keys);
            c->launches++;
            prof_end(c, TK_KID_SCATTER, ev, padded);
            e = check_launch(c, "bucket scatter");
        }
    }
    dfree(c, hist);
    if (e || !padded) {
        if (keys) dfree(c, keys);
        if (offs) dfree(c, offs);
        return e;
    }
    out->keys = keys;
    out->offs = offs;
    out->cols = cols;
    return TK_OK;
}

void table_bucket_free(tk_table *t, BucketKeys *bk) {
    if (bk->keys) dfree(t->ctx, bk->keys);
    if (bk->offs) dfree(t->ctx, bk->offs);
    *bk = BucketKeys();
}

// Pass 2 for the sets whose pass 1 ran since the window counter was reset:
// the table sized from the HLL sketch (allocated fresh, or grown), then every
// set's keys counted partition by partition; frees the key buffers.
int table_count_buckets(tk_table *t, std::vector<BucketKeys> &bk) {
    tk_ctx *c = t->ctx;
    uint64_t windows = 0;
    std::vector<uint32_t> regs(HLL_M);
    int e = cuda_check(c, cudaMemcpyAsync(regs.data(), t->d_hll, HLL_M * 4, cudaMemcpyDeviceToHost, c->stream), "hll d2h");
    if (!e) e = cuda_check(c, cudaMemcpyAsync(&windows, t->d_counters + 1, 8, cudaMemcpyDeviceToHost, c->stream),
                           "window count d2h");
    if (!e) e = cuda_check(c, cudaStreamSynchronize(c->stream), "hll sync");
    if (!e) {
        double est = hll_estimate(regs.data());
        uint64_t want = pow2_at_least((uint64_t)(est * 1.08 / t->max_load) + 1);
        if (t->capacity == 0) e = table_alloc_geom(t, want, 0, false);   // fresh: filled slice by slice below
        else if (want > t->capacity) e = table_rehash(t, want);
    }
    cudaEvent_t ev;
    if (!e && windows) {
        e = overflow_reset(t);
        prof_begin(c, TK_KID_COUNT, &ev);
        bool done = false;
        if (!e && t->fresh && t->t.lbits >= SR_MIN_LBITS) e = count_by_ranges(t, bk, &done);
        if (!e && !done) e = count_by_atomics(t, bk);
        prof_end(c, TK_KID_COUNT, ev, windows);
        if (!e) e = check_launch(c, "count insert");
        if (!e) t->fresh = false;
    } else if (!e && t->fresh) {
        // nothing to insert: still leave every slot empty
        k_fill_empty<<<stream_grid(c, t->capacity, 256), 256, 0, c->stream>>>(t->t.slots, t->capacity, 0);
        c->launches++;
        t->fresh = false;
        e = check_launch(c, "table fill");
    }
    for (BucketKeys &b : bk) table_bucket_free(t, &b);
    if (e && t->fresh && t->t.slots) {
        // a failed first pass must not leave unwritten slots behind
        k_fill_empty<<<stream_grid(c, t->capacity, 256), 256, 0, c->stream>>>(t->t.slots, t->capacity, 0);
        c->launches++;
        t->fresh = false;
    }
    if (e) return e;
    t->total += windows;
    t->distinct_valid = false;
    return drain_overflow(t);
}

// Resets the window counter before a group of pass-1 calls.
int table_count_begin(tk_table *t) {
    return cuda_check(t->ctx, cudaMemsetAsync(t->d_counters + 1, 0, 8, t->ctx->stream), "window counter");
}

// Counts every window of one or more packed read arrays into the table: pass
// 1 per set, then one partitioned pass 2 over all of them (the table is
// touched once for all of them); sets beyond MAX_KEY_SEGS are counted in
// further groups.
int table_count_many(tk_table *t, const tk_reads *const *sets, int nsets) {
    for (int g0 = 0; g0 < nsets; g0 += MAX_KEY_SEGS) {
        const int g1 = std::min(nsets, g0 + MAX_KEY_SEGS);
        uint64_t total_len = 0;
        for (int s = g0; s < g1; s++) total_len += sets[s]->seq_len;
        if (total_len == 0) continue;
        TK_TRY(table_count_begin(t));
        std::vector<BucketKeys> bk(g1 - g0);
        int e = TK_OK;
        for (int s = g0; s < g1 && !e; s++) e = table_bucket_pass(t, sets[s], &bk[s - g0]);
        if (e) {
            for (BucketKeys &b : bk) table_bucket_free(t, &b);
            return e;
        }
        TK_TRY(table_count_buckets(t, bk));
    }
    return TK_OK;
}

int table_count_seq(tk_table *t, const tk_reads *r) { return table_count_many(t, &r, 1); }

static int table_distinct(tk_table *t) {
    tk_ctx *c = t->ctx;
    if (t->distinct_valid) return TK_OK;
    if (!t->capacity) {
        t->distinct = 0;
        t->distinct_valid = true;
        return TK_OK;
    }
    unsigned long long *d = nullptr, h = 0;
    TK_TRY(dmalloc(c, (void **)&d, 8, "occupied"));
    cudaMemsetAsync(d, 0, 8, c->stream);
    k_occupied<<<stream_grid(c, t->capacity, 256), 256, 0, c->stream>>>(t->t.slots, t->capacity, d);
    c->launches++;
    int e = cuda_check(c, cudaMemcpyAsync(&h, d, 8, cudaMemcpyDeviceToHost, c->stream), "occupied d2h");
    if (!e) e = cuda_check(c, cudaStreamSynchronize(c->stream), "occupied sync");
    dfree(c, d);
    if (!e) {
        t->distinct = h;
        t->distinct_valid = true;
    }
    return e;
}

int table_info(tk_table *t, uint64_t *distinct, uint64_t *total, uint64_t *capacity) {
    if (distinct) {
        TK_TRY(table_distinct(t));   // a scan of the table, only when asked for
        *distinct = t->distinct;
    }
    if (total) *total = t->total;
    if (capacity) *capacity = t->capacity;
    return TK_OK;
}

int table_histo(tk_table *t, uint64_t low, uint64_t high, uint64_t *hist) {
    tk_ctx *c = t->ctx;
    if (high < low) return set_err(c, TK_E_INVAL, "histo: high < low");
    uint64_t nb = high - low + 3;
    unsigned long long *d = nullptr;
    TK_TRY(dmalloc(c, (void **)&d, nb * 8, "histo"));
    cudaMemsetAsync(d, 0, nb * 8, c->stream);
    int e = TK_OK;
    if (t->capacity) {
        cudaEvent_t ev;
        prof_begin(c, TK_KID_COMPACT, &ev);
        size_t smem = nb * 4;
        int use_smem = smem <= 96 * 1024;
        if (use_smem && smem > 48 * 1024)
            cudaFuncSetAttribute(k_histo, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        k_histo<<<(unsigned)c->sm_count * 2, 512, use_smem ? smem : 0, c->stream>>>(t->t.slots, t->capacity, low, high, d,
                                                                                    use_smem);
        c->launches++;
        prof_end(c, TK_KID_COMPACT, ev, t->capacity);
        e = check_launch(c, "histo");
    }
    if (!e) e = cuda_check(c, cudaMemcpyAsync(hist, d, nb * 8, cudaMemcpyDeviceToHost, c->stream), "histo d2h");
    if (!e) e = cuda_check(c, cudaStreamSynchronize(c->stream), "histo sync");
    dfree(c, d);
    if (!e) {
        // every occupied slot fell in one bin: the bins add up to the distinct k-mers
        uint64_t distinct = 0;
        for (uint64_t i = 0; i < nb; i++) distinct += hist[i];
        t->distinct = distinct;
        t->distinct_valid = true;
    }
    return e;
}

// Sorted (key, count) pairs with count >= min_count into freshly allocated
// device arrays (caller frees with dfree).
int table_sorted_pairs(tk_table *t, uint32_t min_count, uint64_t **keys_out, uint32_t **cnt_out, uint64_t *n_out) {
    tk_ctx *c = t->ctx;
    *keys_out = nullptr;
    *cnt_out = nullptr;
    *n_out = 0;
    TK_TRY(table_distinct(t));
    uint64_t upper = std::max<uint64_t>(t->distinct, 1);
    uint64_t *k0 = nullptr, *k1 = nullptr;
    uint32_t *v0 = nullptr, *v1 = nullptr;
    unsigned long long *d_n = nullptr;
    int e = dmalloc(c, (void **)&k0, upper * 8, "dump keys");
    if (!e) e = dmalloc(c, (void **)&v0, upper * 4, "dump counts");
    if (!e) e = dmalloc(c, (void **)&k1, upper * 8, "dump keys tmp");
    if (!e) e = dmalloc(c, (void **)&v1, upper * 4, "dump counts tmp");
    if (!e) e = dmalloc(c, (void **)&d_n, 8, "dump n");
    unsigned long long hn = 0;
    if (!e && t->capacity) {
        cudaMemsetAsync(d_n, 0, 8, c->stream);
        cudaEvent_t ev;
        prof_begin(c, TK_KID_COMPACT, &ev);
        k_compact<<<stream_grid(c, (t->capacity + CP_ITEMS - 1) / CP_ITEMS, 256), 256, 0, c->stream>>>(
            t->t.slots, t->capacity, min_count, k0, v0, d_n);
        c->launches++;
        prof_end(c, TK_KID_COMPACT, ev, t->capacity);
        e = cuda_check(c, cudaMemcpyAsync(&hn, d_n, 8, cudaMemcpyDeviceToHost, c->stream), "compact n");
        if (!e) e = cuda_check(c, cudaStreamSynchronize(c->stream), "compact sync");
    }
    bool in_tmp = false;
    if (!e && hn > 1) {
        cudaEvent_t ev;
        prof_begin(c, TK_KID_SORT, &ev);
        e = radix_sort_pairs(c, k0, v0, hn, 2 * t->k, k1, v1, &in_tmp);
        prof_end(c, TK_KID_SORT, ev, hn);
    }
    if (d_n) dfree(c, d_n);
    if (e) {
        dfree(c, k0); dfree(c, k1); dfree(c, v0); dfree(c, v1);
        return e;
    }
    if (in_tmp) {
        std::swap(k0, k1);
        std::swap(v0, v1);
    }
    dfree(c, k1);
    dfree(c, v1);
    *keys_out = k0;
    *cnt_out = v0;
    *n_out = hn;
    return TK_OK;
}

// K4: format sorted pairs as ">COUNT\nKMER\n" into a device buffer (the low
// 2k bits of each key); with offs_out, the n record start offsets are handed
// to the caller (its device block to free) instead of freed.
int format_dump(tk_ctx *c, const uint64_t *keys, const uint32_t *cnt, uint64_t n, int k, char **text_out,
                uint64_t *len_out, uint64_t **offs_out) {
    *text_out = nullptr;
    *len_out = 0;
    if (offs_out) *offs_out = nullptr;
    if (n == 0) return TK_OK;
    uint32_t *lens = nullptr;
    uint64_t *offs = nullptr;
    TK_TRY(dmalloc(c, (void **)&lens, n * 4, "dump lengths"));
    int e = dmalloc(c, (void **)&offs, n * 8, "dump offsets");
    uint64_t total = 0;
    cudaEvent_t ev;
    prof_begin(c, TK_KID_DUMP, &ev);
    if (!e) {
        k_dump_len<<<grid_for(n, 256), 256, 0, c->stream>>>(cnt, n, k, lens);
        c->launches++;
        e = scan_excl_u32_to_u64(c, lens, offs, n, &total);
    }
    char *text = nullptr;
    if (!e) e = dmalloc(c, (void **)&text, total, "dump text");
    if (!e) {
        k_dump_write<<<grid_for(n, DW_THREADS), DW_THREADS, 0, c->stream>>>(keys, cnt, offs, n, k, total, text);
        c->launches++;
        e = check_launch(c, "dump write");
    }
    prof_end(c, TK_KID_DUMP, ev, n);
    dfree(c, lens);
    if (e) {
        if (offs) dfree(c, offs);
        if (text) dfree(c, text);
        return e;
    }
    if (offs_out) *offs_out = offs;
    else dfree(c, offs);
    *text_out = text;
    *len_out = total;
    return TK_OK;
}

int table_insert_pairs(tk_table *t, const uint64_t *d_keys, const uint32_t *d_cnt, uint64_t n) {
    tk_ctx *c = t->ctx;
    if (n == 0) return TK_OK;
    TK_TRY(table_distinct(t));
    uint64_t need = pow2_at_least((uint64_t)((double)(t->distinct + n) / t->max_load) + 1);
    if (t->capacity == 0) TK_TRY(table_alloc(t, need));
    else if (need > t->capacity) TK_TRY(table_rehash(t, need));
    TK_TRY(overflow_reset(t));
    cudaEvent_t ev;
    prof_begin(c, TK_KID_LOAD, &ev);
    k_insert_pairs<<<stream_grid(c, n, 256), 256, 0, c->stream>>>(d_keys, d_cnt, n, t->t, c->max_probes, t->d_ovf,
                                                                   (uint32_t *)(t->d_ovf + t->ovf_cap), t->ovf_cap,
                                                                   t->d_counters);
    c->launches++;
    prof_end(c, TK_KID_LOAD, ev, n);
    TK_TRY(check_launch(c, "insert pairs"));
    t->distinct_valid = false;
    return drain_overflow(t);
}

int table_load_dump_reads(tk_table *t, const tk_reads *r) {
    tk_ctx *c = t->ctx;
    uint64_t n = r->n_reads;
    if (n == 0) return TK_OK;
    uint64_t *keys = nullptr;
    uint32_t *cnt = nullptr;
    TK_TRY(dmalloc(c, (void **)&keys, n * 8, "catalogue keys"));
    int e = dmalloc(c, (void **)&cnt, n * 4, "catalogue counts");
    if (!e) e = cuda_check(c, cudaMemsetAsync(c->d_err, 0, DE_COUNT * 4, c->stream), "err reset");
    if (!e) {
        uint32_t big = 0xFFFFFFFFu;
        cudaMemcpyAsync(c->d_err + DE_PARSE + 1, &big, 4, cudaMemcpyHostToDevice, c->stream);
        k_load_dump<<<grid_for(n, 256), 256, 0, c->stream>>>(r->d_text, r->d_name_off, r->d_name_len, r->d_seq, r->d_rd_off,
                                                             n, t->k, t->canonical, keys, cnt, c->d_err);
        c->launches++;
        uint32_t herr[2] = {0, 0};
        e = cuda_check(c, cudaMemcpyAsync(herr, c->d_err + DE_PARSE, 8, cudaMemcpyDeviceToHost, c->stream), "load err");
        if (!e) e = cuda_check(c, cudaStreamSynchronize(c->stream), "load sync");
        if (!e && herr[0])
            e = set_err(c, TK_E_PARSE, "k-mer catalogue: record " + std::to_string(herr[1]) +
                                           " is not '>COUNT' followed by a " + std::to_string(t->k) + "-mer of A/C/G/T");
    }
    if (!e) e = table_insert_pairs(t, keys, cnt, n);
    dfree(c, keys);
    if (cnt) dfree(c, cnt);
    return e;
}

}  // namespace tk
