// tk_bins.cu -- K7: batched per-bin counting and dump.
//
// Trinity's phase 2 runs one `Trinity --single c<comp>.trinity.reads.fa
// --trinity_complete ...` per read bin through ParaFly (Trinity:3628-3658,
// 3662-3735), and each of those counts its own k-mers (inchworm --reads,
// Trinity:2669-2672).  Thousands of uneven bins make thousands of tiny
// processes.  Here all bins go through the GPU together:
//
//  1. one parse of the concatenated bins; each bin is a range of reads;
//  2. one sizing pass: a 32-register HyperLogLog sketch and the window count
//     per bin (bins found per thread by binary search over bin starts);
//  3. host autotuning: every bin gets its own table slice, a power of two at
//     most `load` full for its estimated distinct k-mers; the count kernel's
//     block size and the load factor are picked once per device by timing
//     candidates;
//  4. one counting launch over all bins (a block per chunk of the text, so
//     the bins in flight are those of a short stretch), captured in a CUDA graph
//     together with the slice fill (re-launched when a slice overflows, with
//     that slice doubled); the context keeps the executable graph and each
//     later batch updates it in place rather than instantiating it again;
//  5. one compaction of every slice into ((local bin << 2k) | key, count), in
//     groups of 2^(64 - 2k) bins so that the pair fits 64 bits, one radix sort
//     per group, one K4 formatting pass; bin b's dump is a contiguous byte
//     range.
//
// Each bin's dump equals a separate plain `jellyfish count` + `dump -L m` of
// that bin (sorted by key).
#include "tk_internal.cuh"

#include <algorithm>
#include <atomic>
#include <chrono>
#include <cmath>

namespace tk {

constexpr int BIN_HLL_P = 5;
constexpr int BIN_HLL_M = 1 << BIN_HLL_P;
constexpr int BC_SPAN = 32;

struct BinGeom {
    const uint64_t *seq0;      // n_bins + 1 packed-read offsets of the bin starts
    const uint64_t *base;      // slot offset of each bin's slice
    const uint8_t *lbits;      // slice size 2^lbits
    uint32_t n_bins;
};

__device__ __forceinline__ uint32_t bin_of(const uint64_t *__restrict__ seq0, uint32_t n_bins, uint64_t p) {
    uint32_t lo = 0, hi = n_bins;   // largest b with seq0[b] <= p
    while (hi - lo > 1) {
        uint32_t mid = (lo + hi) >> 1;
        if (seq0[mid] <= p) lo = mid; else hi = mid;
    }
    return lo;
}

// first read of every bin: reads whose header starts at or after bin_off[b]
__global__ void k_bin_starts(const uint64_t *__restrict__ name_off, uint64_t n_reads, const uint64_t *__restrict__ bin_off,
                             uint32_t n_bins, const uint64_t *__restrict__ rd_off, uint64_t *__restrict__ seq0) {
    uint32_t b = blockIdx.x * blockDim.x + threadIdx.x;
    if (b > n_bins) return;
    uint64_t lo = 0, hi = n_reads;   // first read with header at or after bin_off[b]
    const uint64_t target = bin_off[b];
    while (lo < hi) {
        uint64_t mid = (lo + hi) >> 1;
        if (name_off[mid] - 1 < target) lo = mid + 1; else hi = mid;
    }
    seq0[b] = rd_off[lo];
}

// Calls f(bin, key) for every valid window ending in [p0, p0 + 32).
template <bool CANON, typename F>
__device__ __forceinline__ void bin_windows(const uint8_t *__restrict__ seq, uint64_t p0, uint64_t n, int k,
                                            const uint64_t *__restrict__ seq0, uint32_t n_bins, F &&f) {
    const uint64_t kmask = (1ULL << (2 * k)) - 1;
    const int shift = 2 * (k - 1);
    uint32_t bin = bin_of(seq0, n_bins, p0);
    uint64_t next = seq0[bin + 1];
    const uint8_t *p = seq + p0 - 32;
    uint64_t fw = 0, rc = 0;
    int run = 0;
    for (int j = 0; j < 64; j++) {
        uint32_t c = base_code(p[j]);
        if (c > 3) {
            run = 0;
        } else {
            fw = ((fw << 2) | c) & kmask;
            rc = (rc >> 2) | ((uint64_t)(3u - c) << shift);
            run++;
        }
        if (j >= 32 && run >= k) {
            const uint64_t e = p0 - 32 + j;
            while (e >= next && bin + 1 < n_bins) { bin++; next = seq0[bin + 1]; }
            f(bin, (CANON && rc < fw) ? rc : fw);
        }
    }
}

template <bool CANON>
__global__ void k_bin_sketch(const uint8_t *__restrict__ seq, uint64_t n, int k, const uint64_t *__restrict__ seq0,
                             uint32_t n_bins, uint32_t *__restrict__ regs, unsigned long long *__restrict__ windows) {
    const uint64_t stride = (uint64_t)gridDim.x * blockDim.x * BC_SPAN;
    for (uint64_t p0 = ((uint64_t)blockIdx.x * blockDim.x + threadIdx.x) * BC_SPAN; p0 < n; p0 += stride) {
        uint32_t cur = 0xFFFFFFFFu, cnt = 0;
        bin_windows<CANON>(seq, p0, n, k, seq0, n_bins, [&](uint32_t bin, uint64_t key) {
            if (bin != cur) {
                if (cnt) atomicAdd(&windows[cur], (unsigned long long)cnt);
                cur = bin;
                cnt = 0;
            }
            cnt++;
            uint64_t h = mix64(key ^ 0x2545F4914F6CDD1DULL);
            uint32_t idx = (uint32_t)(h >> (64 - BIN_HLL_P));
            uint32_t rank = (uint32_t)__clzll((long long)(h << BIN_HLL_P)) + 1u;
            if (rank > 64 - BIN_HLL_P) rank = 64 - BIN_HLL_P + 1;
            uint32_t *r = &regs[(uint64_t)bin * BIN_HLL_M + idx];
            if (rank > *r) atomicMax(r, rank);
        });
        if (cnt) atomicAdd(&windows[cur], (unsigned long long)cnt);
    }
}

__global__ void k_bin_fill(Slot *slots, uint64_t n) {
    for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (uint64_t)gridDim.x * blockDim.x) {
        ulonglong2 e;
        e.x = EMPTY_KEY;
        e.y = 0;
        reinterpret_cast<ulonglong2 *>(slots)[i] = e;
    }
}

// The counting launch: all bins, each k-mer into its bin's slice (a block per
// chunk of BC_SPAN positions per thread; the loop also serves smaller grids).
template <bool CANON>
__global__ void k_bin_count(const uint8_t *__restrict__ seq, uint64_t n, int k, BinGeom g, Slot *__restrict__ slots,
                            int max_probes, uint32_t *__restrict__ overflow) {
    const uint64_t stride = (uint64_t)gridDim.x * blockDim.x * BC_SPAN;
    for (uint64_t p0 = ((uint64_t)blockIdx.x * blockDim.x + threadIdx.x) * BC_SPAN; p0 < n; p0 += stride) {
        uint32_t cur = 0xFFFFFFFFu;
        DevTable t;
        t.pbits = 0;
        bin_windows<CANON>(seq, p0, n, k, g.seq0, g.n_bins, [&](uint32_t bin, uint64_t key) {
            if (bin != cur) {
                cur = bin;
                t.slots = slots + g.base[bin];
                t.lbits = g.lbits[bin];
                t.lmask = (1ULL << t.lbits) - 1;
            }
            if (!tbl_add(t, key, 1u, max_probes)) overflow[bin] = 1u;
        });
    }
}

constexpr uint64_t BIN_HISTO = 10002;   // jellyfish histo bins for low 1, high 10000
constexpr int BCP_ITEMS = 8;            // slots per thread per compaction tile (2048-slot tiles)

// largest b in [lo, hi) with base[b] <= p (base[lo] <= p)
__device__ __forceinline__ uint32_t bin_in(const uint64_t *__restrict__ base, uint32_t lo, uint32_t hi, uint64_t p) {
    while (hi - lo > 1) {
        uint32_t mid = (lo + hi) >> 1;
        if (base[mid] <= p) lo = mid; else hi = mid;
    }
    return lo;
}

// Every occupied slot with count >= its bin's minimum, as (local bin << 2k) |
// key with its count, into its bin group's output range.  Bins are grouped
// 2^gshift at a time so that the local bin and the key fit one 64-bit sort
// key; group g's records go to [group_cur[g] at launch, ...).  Slices are
// powers of two of at least 32 slots laid out back to back, so every 32-slot
// aligned run (one warp's load) lies in one bin.  A 2048-slot tile inside one
// group reserves its output with one atomic; a tile that crosses a group
// boundary reserves per warp load.  WRITE false: only the per-group counts
// (group_cur zeroed at launch).  With `histo` (WRITE only), every occupied
// slot's count also goes into its bin's histogram.
template <bool WRITE>
__global__ void __launch_bounds__(256) k_bin_compact(const Slot *__restrict__ slots, uint64_t cap,
                                                     const uint64_t *__restrict__ base, uint32_t n_bins, int k,
                                                     int gshift, const uint32_t *__restrict__ min_count,
                                                     unsigned long long *__restrict__ group_cur,
                                                     uint64_t *__restrict__ okeys, uint32_t *__restrict__ ovals,
                                                     unsigned long long *__restrict__ histo) {
    __shared__ uint32_t sm[256 / 32 + 1];
    __shared__ unsigned long long s_base;
    const unsigned lane = lane_id(), warp = threadIdx.x >> 5;
    const uint64_t chunk = 256ull * BCP_ITEMS;
    const uint32_t lmask = (uint32_t)((1ull << gshift) - 1ull);
    for (uint64_t t0 = (uint64_t)blockIdx.x * chunk; t0 < cap; t0 += (uint64_t)gridDim.x * chunk) {
        const uint64_t tl = min(t0 + chunk, cap) - 1;
        const uint32_t b0 = bin_of(base, n_bins, t0), b1 = bin_of(base, n_bins, tl);
        const uint32_t g0 = (uint32_t)((uint64_t)b0 >> gshift), g1 = (uint32_t)((uint64_t)b1 >> gshift);
        ulonglong2 v[BCP_ITEMS];
        uint32_t bin[BCP_ITEMS];
        uint32_t selm = 0, nsel = 0;
#pragma unroll
        for (int j = 0; j < BCP_ITEMS; j++) {
            const uint64_t run = t0 + (uint64_t)j * 256 + warp * 32;   // this warp's 32-slot run
            const uint64_t i = run + lane;
            v[j].x = EMPTY_KEY;
            v[j].y = 0;
            bin[j] = run <= tl ? bin_in(base, b0, b1 + 1, run) : b1;
            if (i < cap) v[j] = __ldcs(reinterpret_cast<const ulonglong2 *>(&slots[i]));
            const bool occ = v[j].x != EMPTY_KEY;
            const uint32_t c = (uint32_t)v[j].y;
            const bool sel = occ && c >= min_count[bin[j]];
            selm |= (sel ? 1u : 0u) << j;
            nsel += sel;
            if (WRITE && histo) {
                // warp-merged increments: equal buckets (one bin per run) add once
                const uint64_t cell = (uint64_t)bin[j] * BIN_HISTO + (c > 10000u ? 10001u : c);
                const unsigned act = __ballot_sync(0xffffffffu, occ);
                if (occ) {
                    const unsigned peers = __match_any_sync(act, cell);
                    if (lane == (unsigned)(__ffs(peers) - 1)) atomicAdd(&histo[cell], (unsigned long long)__popc(peers));
                }
            }
        }
        if (g0 == g1) {
            uint32_t tot;
            const uint32_t pre = block_excl_scan<uint32_t>(nsel, sm, &tot);
            if (tot == 0) continue;                   // uniform over the block
            if (threadIdx.x == 0) s_base = atomicAdd(&group_cur[g0], (unsigned long long)tot);
            __syncthreads();
            if (WRITE) {
                uint64_t o = s_base + pre;
#pragma unroll
                for (int j = 0; j < BCP_ITEMS; j++)
                    if ((selm >> j) & 1u) {
                        okeys[o] = ((uint64_t)(bin[j] & lmask) << (2 * k)) | v[j].x;
                        ovals[o] = (uint32_t)v[j].y;
                        o++;
                    }
            }
            __syncthreads();
        } else {
#pragma unroll
            for (int j = 0; j < BCP_ITEMS; j++) {
                const unsigned m = __ballot_sync(0xffffffffu, (selm >> j) & 1u);
                if (!m) continue;
                unsigned long long wb = 0;
                if (lane == 0) wb = atomicAdd(&group_cur[(uint64_t)bin[j] >> gshift], (unsigned long long)__popc(m));
                wb = __shfl_sync(0xffffffffu, wb, 0);
                if (WRITE && ((selm >> j) & 1u)) {
                    const uint64_t o = wb + __popc(m & ((1u << lane) - 1u));
                    okeys[o] = ((uint64_t)(bin[j] & lmask) << (2 * k)) | v[j].x;
                    ovals[o] = (uint32_t)v[j].y;
                }
            }
        }
    }
}

// first sorted record of every bin (and n at the end): bin b is local bin
// b & (2^gshift - 1) of group b >> gshift, whose records are
// [goff[g], goff[g + 1]) sorted by (local bin << 2k) | key
__global__ void k_bin_bounds(const uint64_t *__restrict__ keys, const uint64_t *__restrict__ goff, int gshift, int k,
                             uint32_t n_bins, uint64_t n, uint64_t *__restrict__ first) {
    uint32_t b = blockIdx.x * blockDim.x + threadIdx.x;
    if (b > n_bins) return;
    if (b == n_bins) {
        first[b] = n;
        return;
    }
    const uint32_t g = (uint32_t)((uint64_t)b >> gshift);
    const uint64_t target = (uint64_t)(b & (uint32_t)((1ull << gshift) - 1ull)) << (2 * k);
    uint64_t lo = goff[g], hi = goff[g + 1];
    while (lo < hi) {
        uint64_t mid = (lo + hi) >> 1;
        if (keys[mid] < target) lo = mid + 1; else hi = mid;
    }
    first[b] = lo;
}

__global__ void k_bin_text_bounds(const uint64_t *__restrict__ first, const uint64_t *__restrict__ off, uint64_t n,
                                  uint64_t total, uint32_t n_bins, uint64_t *__restrict__ text0) {
    uint32_t b = blockIdx.x * blockDim.x + threadIdx.x;
    if (b > n_bins) return;
    text0[b] = first[b] < n ? off[first[b]] : total;
}

static double hll32(const uint32_t *r) {
    double sum = 0;
    int zeros = 0;
    for (int i = 0; i < BIN_HLL_M; i++) {
        sum += std::ldexp(1.0, -(int)r[i]);
        zeros += r[i] == 0;
    }
    const double m = BIN_HLL_M, alpha = 0.697;
    double est = alpha * m * m / sum;
    if (est <= 2.5 * m && zeros) est = m * std::log(m / zeros);
    return est;
}

}  // namespace tk

// ------------------------------------------------------------------ host side

struct tk_bins {
    tk_ctx *ctx = nullptr;
    uint32_t n_bins = 0;
    int k = 25;
    char *d_text = nullptr;                 // dump text of all bins, bin after bin
    uint64_t text_len = 0;
    std::vector<uint64_t> text0;            // n_bins + 1 byte offsets
    uint64_t kmers = 0;                     // windows counted
    uint64_t table_slots = 0;
    int block = 256;
    int load_pm = 0;                        // slice load factor, per mille
    int relaunches = 0;
};

namespace tk {
int parse_reads(tk_ctx *c, tk_reads *r);

// block sizes the count kernel is tuned over, per device (0 = not tuned yet)
static std::atomic<int> g_tuned_block[64];   // several contexts (server slots) may share a device
// slice load factor (per mille) chosen per device on the first batch of at
// least BIN_TUNE_MIN windows (0 = not tuned yet: the caller's default)
static std::atomic<int> g_tuned_load[64];
constexpr uint64_t BIN_TUNE_MIN = 50ull << 20;

template <bool CANON>
static void launch_count(tk_ctx *c, int block, const uint8_t *seq, uint64_t n, int k, BinGeom g, Slot *slots,
                         uint32_t *ovf) {
    // one block per chunk of block x 32 positions: the blocks start in index
    // order as earlier ones finish, so the bins being counted at any moment
    // are those of a short stretch of the text and their slices stay in L2
    // (a persistent grid's warps drift apart over the text)
    const uint64_t span = (uint64_t)block * BC_SPAN;
    const unsigned grid = (unsigned)std::max<uint64_t>(1, std::min<uint64_t>((n + span - 1) / span, 0x7FFFFFFFull));
    k_bin_count<CANON><<<grid, block, 0, c->stream>>>(seq, n, k, g, slots, c->max_probes, ovf);
    c->launches++;
}

static int bins_run(tk_ctx *c, const char *text, uint64_t len, int where, const uint64_t *bin_off_h, uint32_t n_bins,
                    int k, int canonical, const uint32_t *min_counts_h, uint64_t *histos_h, double load,
                    tk_bins *out) {
    // 1. parse everything once
    tk_reads r;
    r.ctx = c;
    r.text_len = len;
    std::vector<void *> tmp;
    auto alloc = [&](void **p, size_t bytes, const char *what) {
        int ee = dmalloc(c, p, bytes ? bytes : 16, what);
        if (!ee) tmp.push_back(*p);
        return ee;
    };
    auto cleanup = [&]() {
        for (void *p : tmp) dfree(c, p);
        if (r.d_seq_alloc) dfree(c, r.d_seq_alloc);
        if (r.d_pack_alloc) dfree(c, r.d_pack_alloc);
        if (r.d_rd_off) dfree(c, r.d_rd_off);
        if (r.d_name_off) dfree(c, r.d_name_off);
        if (r.d_name_len) dfree(c, r.d_name_len);
    };
    int e = TK_OK;
    if (where == TK_DEVICE) r.d_text = const_cast<char *>(text);
    else {
        e = alloc((void **)&r.d_text, len + 64, "bins text");
        if (!e && len) e = cuda_check(c, cudaMemcpyAsync(r.d_text, text, len, cudaMemcpyHostToDevice, c->stream), "bins h2d");
    }
    if (!e) e = parse_reads(c, &r);
    uint64_t *d_bin_off = nullptr, *d_seq0 = nullptr;
    if (!e) e = alloc((void **)&d_bin_off, (n_bins + 1) * 8, "bin offsets");
    if (!e) e = alloc((void **)&d_seq0, (n_bins + 2) * 8, "bin starts");
    if (!e) {
        cudaMemcpyAsync(d_bin_off, bin_off_h, (n_bins + 1) * 8, cudaMemcpyHostToDevice, c->stream);
        if (r.n_reads) {
            k_bin_starts<<<(n_bins + 256) / 256, 256, 0, c->stream>>>(r.d_name_off, r.n_reads, d_bin_off, n_bins,
                                                                       r.d_rd_off, d_seq0);
            c->launches++;
        } else {
            cudaMemsetAsync(d_seq0, 0, (n_bins + 1) * 8, c->stream);
        }
        // sentinel past the last bin so seq0[bin + 1] is always readable
        uint64_t tail = r.seq_len;
        cudaMemcpyAsync(d_seq0 + n_bins, &tail, 8, cudaMemcpyHostToDevice, c->stream);
        cudaMemcpyAsync(d_seq0 + n_bins + 1, &tail, 8, cudaMemcpyHostToDevice, c->stream);
        e = check_launch(c, "bin starts");
    }
    const uint64_t n = r.seq_len;
    // 2. sizing sketch per bin
    uint32_t *d_regs = nullptr;
    unsigned long long *d_win = nullptr;
    std::vector<uint32_t> regs((size_t)n_bins * BIN_HLL_M);
    std::vector<unsigned long long> win(n_bins);
    if (!e) e = alloc((void **)&d_regs, regs.size() * 4, "bin sketches");
    if (!e) e = alloc((void **)&d_win, n_bins * 8, "bin windows");
    if (!e) {
        cudaMemsetAsync(d_regs, 0, regs.size() * 4, c->stream);
        cudaMemsetAsync(d_win, 0, n_bins * 8, c->stream);
        if (n) {
            const unsigned grid = (unsigned)std::max<uint64_t>(1, std::min<uint64_t>((n + 256 * BC_SPAN - 1) / (256 * BC_SPAN),
                                                                                     (uint64_t)c->sm_count * 8));
            cudaEvent_t ev;
            prof_begin(c, TK_KID_HLL, &ev);
            if (canonical) k_bin_sketch<true><<<grid, 256, 0, c->stream>>>(r.d_seq, n, k, d_seq0, n_bins, d_regs, d_win);
            else k_bin_sketch<false><<<grid, 256, 0, c->stream>>>(r.d_seq, n, k, d_seq0, n_bins, d_regs, d_win);
            c->launches++;
            prof_end(c, TK_KID_HLL, ev, n);
        }
        e = cuda_check(c, cudaMemcpyAsync(regs.data(), d_regs, regs.size() * 4, cudaMemcpyDeviceToHost, c->stream), "sketch d2h");
        if (!e) e = cuda_check(c, cudaMemcpyAsync(win.data(), d_win, n_bins * 8, cudaMemcpyDeviceToHost, c->stream), "windows d2h");
        if (!e) e = cuda_check(c, cudaStreamSynchronize(c->stream), "sketch sync");
    }
    // 3. slice per bin, sized from its sketch (never above its window count)
    //    for a load factor: estimated distinct k-mers / load, a power of two
    std::vector<uint64_t> base(n_bins + 1);
    std::vector<uint8_t> lbits(n_bins);
    uint64_t total = 0, kmers = 0;
    for (uint32_t b = 0; !e && b < n_bins; b++) kmers += win[b];
    auto size_slices = [&](double L) {
        total = 0;
        for (uint32_t b = 0; b < n_bins; b++) {
            double est = std::min<double>(hll32(&regs[(size_t)b * BIN_HLL_M]) * 1.35, (double)win[b]);
            uint64_t want = (uint64_t)(est / L) + 1;
            int lb = 5;
            while ((1ULL << lb) < want) lb++;
            lbits[b] = (uint8_t)lb;
            base[b] = total;
            total += 1ULL << lb;
        }
        base[n_bins] = total;
    };
    Slot *slots = nullptr;
    uint64_t *d_base = nullptr;
    uint8_t *d_lbits = nullptr;
    uint32_t *d_ovf = nullptr;
    if (!e) e = alloc((void **)&d_base, (n_bins + 1) * 8, "bin slice bases");
    if (!e) e = alloc((void **)&d_lbits, n_bins, "bin slice sizes");
    if (!e) e = alloc((void **)&d_ovf, n_bins * 4, "bin overflow flags");
    std::vector<uint32_t> ovf(n_bins);
    if (!e && !g_tuned_load[c->device & 63].load() && n && kmers >= BIN_TUNE_MIN) {
        // autotune the slice load factor once per device on a batch of this
        // size: fill + count timed for each candidate (fuller slices are
        // smaller to fill and sweep but probe longer); the dumps do not
        // depend on it, every bin's records being sorted by key
        const int tb0 = g_tuned_block[c->device & 63].load();
        const int tb = tb0 ? tb0 : 256;
        double best = 1e30;
        int best_pm = (int)(load * 1000 + 0.5);
        for (int pm : {450, 600, 750}) {
            size_slices(pm / 1000.0);
            Slot *ts = nullptr;
            if ((e = dmalloc(c, (void **)&ts, total * sizeof(Slot), "bin tables (tuning)"))) break;
            cudaMemcpyAsync(d_base, base.data(), (n_bins + 1) * 8, cudaMemcpyHostToDevice, c->stream);
            cudaMemcpyAsync(d_lbits, lbits.data(), n_bins, cudaMemcpyHostToDevice, c->stream);
            cudaMemsetAsync(d_ovf, 0, n_bins * 4, c->stream);
            BinGeom g{d_seq0, d_base, d_lbits, n_bins};
            cudaEvent_t a, b2;
            cudaEventCreate(&a);
            cudaEventCreate(&b2);
            cudaEventRecord(a, c->stream);
            k_bin_fill<<<(unsigned)c->sm_count * 8, 256, 0, c->stream>>>(ts, total);
            if (canonical) launch_count<true>(c, tb, r.d_seq, n, k, g, ts, d_ovf);
            else launch_count<false>(c, tb, r.d_seq, n, k, g, ts, d_ovf);
            cudaEventRecord(b2, c->stream);
            e = cuda_check(c, cudaEventSynchronize(b2), "load tuning");
            float ms = 0;
            cudaEventElapsedTime(&ms, a, b2);
            cudaEventDestroy(a);
            cudaEventDestroy(b2);
            dfree(c, ts);
            if (e) break;
            if (ms < best) { best = ms; best_pm = pm; }
        }
        if (!e) g_tuned_load[c->device & 63].store(best_pm);
    }
    const int tl = g_tuned_load[c->device & 63].load();
    const int load_pm = tl ? tl : (int)(load * 1000 + 0.5);
    if (!e) size_slices(load_pm / 1000.0);
    // 4. fill + count, captured in a CUDA graph; a slice that
    //    overflowed is doubled and the graph rebuilt and relaunched
    int relaunch = 0;
    const int tblk = g_tuned_block[c->device & 63].load();
    int block = tblk ? tblk : 256;
    for (int round = 0; !e && round < 6; round++) {
        if (slots) { dfree(c, slots); slots = nullptr; }
        if ((e = dmalloc(c, (void **)&slots, total * sizeof(Slot), "bin tables"))) break;
        cudaMemcpyAsync(d_base, base.data(), (n_bins + 1) * 8, cudaMemcpyHostToDevice, c->stream);
        cudaMemcpyAsync(d_lbits, lbits.data(), n_bins, cudaMemcpyHostToDevice, c->stream);
        cudaMemsetAsync(d_ovf, 0, n_bins * 4, c->stream);
        BinGeom g{d_seq0, d_base, d_lbits, n_bins};
        if (round == 0 && !tblk && n) {
            // autotune the block shape once per device on this batch (timed launches, same result each time)
            double best = 1e30;
            for (int cand : {128, 256, 512}) {
                k_bin_fill<<<(unsigned)c->sm_count * 8, 256, 0, c->stream>>>(slots, total);
                cudaEvent_t a, b2;
                cudaEventCreate(&a);
                cudaEventCreate(&b2);
                cudaEventRecord(a, c->stream);
                if (canonical) launch_count<true>(c, cand, r.d_seq, n, k, g, slots, d_ovf);
                else launch_count<false>(c, cand, r.d_seq, n, k, g, slots, d_ovf);
                cudaEventRecord(b2, c->stream);
                cudaEventSynchronize(b2);
                float ms = 0;
                cudaEventElapsedTime(&ms, a, b2);
                cudaEventDestroy(a);
                cudaEventDestroy(b2);
                if (ms < best) { best = ms; block = cand; }
            }
            g_tuned_block[c->device & 63].store(block);
            cudaMemsetAsync(d_ovf, 0, n_bins * 4, c->stream);
            if ((e = check_launch(c, "bin autotune"))) break;
        }
        cudaGraph_t graph = nullptr;
        cudaGraphExec_t exec = nullptr;
        cudaEvent_t ev;
        prof_begin(c, TK_KID_BINS, &ev);
        if ((e = cuda_check(c, cudaStreamBeginCapture(c->stream, cudaStreamCaptureModeThreadLocal), "capture begin"))) break;
        k_bin_fill<<<(unsigned)c->sm_count * 8, 256, 0, c->stream>>>(slots, total);
        c->launches++;
        if (n) {
            if (canonical) launch_count<true>(c, block, r.d_seq, n, k, g, slots, d_ovf);
            else launch_count<false>(c, block, r.d_seq, n, k, g, slots, d_ovf);
        }
        e = cuda_check(c, cudaStreamEndCapture(c->stream, &graph), "capture end");
        // the context's executable graph takes this batch's parameters in
        // place (same two nodes, new pointers and sizes); a refused update
        // means a new instantiation
        if (!e && c->bins_exec) {
            cudaGraphExecUpdateResultInfo info;
            if (cudaGraphExecUpdate(c->bins_exec, graph, &info) != cudaSuccess) {
                cudaGetLastError();
                cudaGraphExecDestroy(c->bins_exec);
                c->bins_exec = nullptr;
            }
        }
        if (!e && !c->bins_exec) e = cuda_check(c, cudaGraphInstantiate(&c->bins_exec, graph, 0), "graph instantiate");
        if (!e) exec = c->bins_exec;
        if (!e) e = cuda_check(c, cudaGraphLaunch(exec, c->stream), "graph launch");
        prof_end(c, TK_KID_BINS, ev, kmers);
        if (graph) cudaGraphDestroy(graph);
        if (!e) e = cuda_check(c, cudaMemcpyAsync(ovf.data(), d_ovf, n_bins * 4, cudaMemcpyDeviceToHost, c->stream), "ovf d2h");
        if (!e) e = cuda_check(c, cudaStreamSynchronize(c->stream), "bins count sync");
        if (e) break;
        bool any = false;
        total = 0;
        for (uint32_t b = 0; b < n_bins; b++) {
            if (ovf[b]) { lbits[b]++; any = true; }
            base[b] = total;
            total += 1ULL << lbits[b];
        }
        base[n_bins] = total;
        if (!any) break;
        // undo the size change of the final layout bookkeeping: recount with bigger slices
        relaunch++;
        if (round == 5) e = set_err(c, TK_E_TABLE_FULL, "bin slices kept overflowing");
    }
    // restore the layout actually used by the last (successful) count
    if (!e) {
        total = 0;
        for (uint32_t b = 0; b < n_bins; b++) { base[b] = total; total += 1ULL << lbits[b]; }
        base[n_bins] = total;
    }
    // 5. compact, sort by (bin, key), format.  (bin << 2k) | key is one
    //    64-bit sort key while it fits: up to 2^(64 - 2k) bins (16384 at
    //    k = 25, 4 at k = 31).  Past that, bins are taken in groups of
    //    2^(64 - 2k): each group's records get their own output range (a
    //    counting pass first) and are sorted by (local bin << 2k) | key.
    uint64_t *k0 = nullptr, *k1 = nullptr;
    uint32_t *v0 = nullptr, *v1 = nullptr;
    unsigned long long *d_gcur = nullptr;
    uint32_t *d_minc = nullptr;
    unsigned long long *d_histo = nullptr;
    int bin_bits = 0;
    while ((1ULL << bin_bits) < n_bins) bin_bits++;
    const int gshift = std::min(bin_bits, 64 - 2 * k);
    const uint32_t n_groups = (uint32_t)(((uint64_t)n_bins + (1ULL << gshift) - 1) >> gshift);
    std::vector<unsigned long long> gcount(n_groups, 0), goff(n_groups + 1, 0);
    if (!e) e = alloc((void **)&d_gcur, (n_groups + 1) * 8, "bin group cursors");
    if (!e) e = alloc((void **)&d_minc, n_bins * 4, "bin minimum counts");
    if (!e) e = cuda_check(c, cudaMemcpyAsync(d_minc, min_counts_h, n_bins * 4, cudaMemcpyHostToDevice, c->stream), "min counts");
    if (!e && histos_h) {
        e = alloc((void **)&d_histo, (uint64_t)n_bins * BIN_HISTO * 8, "bin histograms");
        if (!e) cudaMemsetAsync(d_histo, 0, (uint64_t)n_bins * BIN_HISTO * 8, c->stream);
    }
    // occupied slots <= min(windows, slots)
    const uint64_t upper = std::max<uint64_t>(1, std::min<uint64_t>(kmers, total));
    if (!e) e = alloc((void **)&k0, upper * 8, "bin keys");
    if (!e) e = alloc((void **)&v0, upper * 4, "bin counts");
    if (!e) e = alloc((void **)&k1, upper * 8, "bin keys tmp");
    if (!e) e = alloc((void **)&v1, upper * 4, "bin counts tmp");
    const unsigned cgrid = (unsigned)c->sm_count * 8;
    if (!e) {
        cudaEvent_t ev;
        prof_begin(c, TK_KID_COMPACT, &ev);
        cudaMemsetAsync(d_gcur, 0, (n_groups + 1) * 8, c->stream);
        if (n_groups > 1) {
            k_bin_compact<false><<<cgrid, 256, 0, c->stream>>>(slots, total, d_base, n_bins, k, gshift, d_minc, d_gcur,
                                                               nullptr, nullptr, nullptr);
            c->launches++;
            e = cuda_check(c, cudaMemcpyAsync(gcount.data(), d_gcur, n_groups * 8, cudaMemcpyDeviceToHost, c->stream),
                           "bin group counts d2h");
            if (!e) e = cuda_check(c, cudaStreamSynchronize(c->stream), "bin group counts sync");
            for (uint32_t g = 0; !e && g < n_groups; g++) goff[g + 1] = goff[g] + gcount[g];
            if (!e) e = cuda_check(c, cudaMemcpyAsync(d_gcur, goff.data(), n_groups * 8, cudaMemcpyHostToDevice, c->stream),
                                   "bin group offsets h2d");
        }
        if (!e) {
            k_bin_compact<true><<<cgrid, 256, 0, c->stream>>>(slots, total, d_base, n_bins, k, gshift, d_minc, d_gcur, k0,
                                                              v0, d_histo);
            c->launches++;
        }
        prof_end(c, TK_KID_COMPACT, ev, total);
        if (!e && n_groups == 1) {
            e = cuda_check(c, cudaMemcpyAsync(gcount.data(), d_gcur, 8, cudaMemcpyDeviceToHost, c->stream), "bins n d2h");
            goff[1] = 0;
        }
        if (!e && d_histo)
            e = cuda_check(c, cudaMemcpyAsync(histos_h, d_histo, (uint64_t)n_bins * BIN_HISTO * 8, cudaMemcpyDeviceToHost,
                                              c->stream), "bin histograms d2h");
        if (!e) e = cuda_check(c, cudaStreamSynchronize(c->stream), "bins compact sync");
        if (!e && n_groups == 1) goff[1] = gcount[0];
    }
    const uint64_t hn = goff[n_groups];
    // every group sorts the same number of bits, so the groups of more than
    // one record end in the same buffer; a group that ended in the other one
    // (a single record: no pass) is moved there
    uint64_t *keys = k0;
    uint32_t *cnts = v0;
    if (!e && hn > 1) {
        cudaEvent_t ev;
        prof_begin(c, TK_KID_SORT, &ev);
        const int bits = 2 * k + gshift;
        std::vector<char> in_tmp(n_groups, 0);
        int final_tmp = -1;
        for (uint32_t g = 0; !e && g < n_groups; g++) {
            const uint64_t o = goff[g], m = goff[g + 1] - o;
            if (m == 0) continue;
            bool t = false;
            e = radix_sort_pairs(c, k0 + o, v0 + o, m, bits, k1 + o, v1 + o, &t);
            in_tmp[g] = t;
            if (m > 1 && final_tmp < 0) final_tmp = t ? 1 : 0;
        }
        if (final_tmp < 0) final_tmp = 0;
        for (uint32_t g = 0; !e && g < n_groups; g++) {
            const uint64_t o = goff[g], m = goff[g + 1] - o;
            if (m == 0 || in_tmp[g] == final_tmp) continue;
            uint64_t *ks = in_tmp[g] ? k1 : k0, *kd = final_tmp ? k1 : k0;
            uint32_t *vs = in_tmp[g] ? v1 : v0, *vd = final_tmp ? v1 : v0;
            e = cuda_check(c, cudaMemcpyAsync(kd + o, ks + o, m * 8, cudaMemcpyDeviceToDevice, c->stream), "bin key move");
            if (!e) e = cuda_check(c, cudaMemcpyAsync(vd + o, vs + o, m * 4, cudaMemcpyDeviceToDevice, c->stream), "bin count move");
        }
        keys = final_tmp ? k1 : k0;
        cnts = final_tmp ? v1 : v0;
        prof_end(c, TK_KID_SORT, ev, hn);
    }
    uint64_t *first = nullptr, *d_text0 = nullptr, *d_goff = nullptr, *offs = nullptr;
    uint64_t text_len = 0;
    char *d_dump = nullptr;
    if (!e) e = alloc((void **)&first, (n_bins + 1) * 8, "bin first record");
    if (!e) e = alloc((void **)&d_text0, (n_bins + 1) * 8, "bin text offsets");
    if (!e) e = alloc((void **)&d_goff, (n_groups + 1) * 8, "bin group offsets");
    if (!e) e = cuda_check(c, cudaMemcpyAsync(d_goff, goff.data(), (n_groups + 1) * 8, cudaMemcpyHostToDevice, c->stream),
                           "bin group offsets");
    if (!e) {
        k_bin_bounds<<<(n_bins + 256) / 256, 256, 0, c->stream>>>(keys, d_goff, gshift, k, n_bins, hn, first);
        c->launches++;
        // K4 formats the low 2k bits of each key
        e = format_dump(c, keys, cnts, hn, k, &d_dump, &text_len, &offs);
    }
    if (!e) {
        k_bin_text_bounds<<<(n_bins + 256) / 256, 256, 0, c->stream>>>(first, offs, hn, text_len, n_bins, d_text0);
        c->launches++;
        out->text0.resize(n_bins + 1);
        e = cuda_check(c, cudaMemcpyAsync(out->text0.data(), d_text0, (n_bins + 1) * 8, cudaMemcpyDeviceToHost, c->stream),
                       "text bounds");
        if (!e) e = cuda_check(c, cudaStreamSynchronize(c->stream), "bins dump sync");
    }
    if (offs) dfree(c, offs);
    if (slots) dfree(c, slots);
    cleanup();
    if (e) {
        if (d_dump) dfree(c, d_dump);
        return e;
    }
    out->d_text = d_dump;
    out->text_len = text_len;
    out->kmers = kmers;
    out->table_slots = total;
    out->block = block;
    out->load_pm = load_pm;
    out->relaunches = relaunch;
    return TK_OK;
}

}  // namespace tk

extern "C" {

int tk_count_bins_ex(tk_ctx *ctx, const char *text, uint64_t len, int where, const uint64_t *bin_off,
                     uint32_t n_bins, int k, int canonical, const uint32_t *min_counts, uint64_t *histos,
                     tk_bins **out) {
    if (!ctx || !out || !bin_off || !min_counts || n_bins == 0 || (!text && len)) return TK_E_INVAL;
    *out = nullptr;
    if (cudaSetDevice(ctx->device) != cudaSuccess) return tk::set_err(ctx, TK_E_CUDA, "cudaSetDevice");
    if (k < 1 || k > tk::MAX_K) return tk::set_err(ctx, TK_E_INVAL, "k must be in 1..31");
    for (uint32_t b = 0; b < n_bins; b++)
        if (bin_off[b] > bin_off[b + 1] || bin_off[b + 1] > len)
            return tk::set_err(ctx, TK_E_INVAL, "bin offsets must be non-decreasing and within the text");
    tk_bins *z = new (std::nothrow) tk_bins();
    if (!z) return TK_E_OOM;
    z->ctx = ctx;
    z->n_bins = n_bins;
    z->k = k;
    int e = tk::bins_run(ctx, text, len, where, bin_off, n_bins, k, canonical, min_counts, histos, 0.6, z);
    if (e) {
        delete z;
        return e;
    }
    *out = z;
    return TK_OK;
}

int tk_count_bins(tk_ctx *ctx, const char *text, uint64_t len, int where, const uint64_t *bin_off, uint32_t n_bins,
                  int k, int canonical, uint32_t min_count, tk_bins **out) {
    if (n_bins == 0) return TK_E_INVAL;
    std::vector<uint32_t> mc(n_bins, min_count ? min_count : 1);
    return tk_count_bins_ex(ctx, text, len, where, bin_off, n_bins, k, canonical, mc.data(), nullptr, out);
}

int tk_bins_info(const tk_bins *z, uint64_t *text_len, uint64_t *kmers) {
    if (!z) return TK_E_INVAL;
    if (text_len) *text_len = z->text_len;
    if (kmers) *kmers = z->kmers;
    return TK_OK;
}

int tk_bins_dump_offsets(const tk_bins *z, uint64_t *offsets) {
    if (!z || !offsets) return TK_E_INVAL;
    std::copy(z->text0.begin(), z->text0.end(), offsets);
    return TK_OK;
}

int tk_bins_dump_text(const tk_bins *z, char *dst, uint64_t cap) {
    if (!z || (!dst && z->text_len)) return TK_E_INVAL;
    tk_ctx *c = z->ctx;
    if (cap < z->text_len) return tk::set_err(c, TK_E_RANGE, "tk_bins_dump_text: buffer smaller than the dumps");
    if (z->text_len) TK_CUDA(c, cudaMemcpyAsync(dst, z->d_text, z->text_len, cudaMemcpyDeviceToHost, c->stream));
    return tk::cuda_check(c, cudaStreamSynchronize(c->stream), "bins text sync");
}

int tk_bins_tuning(const tk_bins *z, int *block, int *load_per_mille, int *relaunches) {
    if (!z) return TK_E_INVAL;
    if (block) *block = z->block;
    if (load_per_mille) *load_per_mille = z->load_pm;
    if (relaunches) *relaunches = z->relaunches;
    return TK_OK;
}

void tk_bins_free(tk_bins *z) {
    if (!z) return;
    cudaSetDevice(z->ctx->device);
    if (z->d_text) tk::dfree(z->ctx, z->d_text);
    delete z;
}

}  // extern "C"
