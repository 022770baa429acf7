// tk_r2t.cu -- K6: Chrysalis ReadsToTranscripts read-to-component assignment
// (called at Trinity:2237-2251).
//
// Build: the bundle (one '>s_<component>' record per component, contigs
// joined by 'X', util/support_scripts/add_LR_reads_to_iworm_bundle.pl:19-47)
// is parsed like reads; every window of k A/C/G/T bases is inserted with
// value = its record index through atomicMin, so a k-mer held by several
// records belongs to the first of them whatever the insertion order.
// Assign: one warp per read packs the read's bases 2 bits each into shared
// memory, cuts each lane's windows out of it, looks them up, sorts the record
// indices in registers and takes the longest run: the record with most votes,
// ties to the smaller index.  Reads with more than 256 windows use one block
// and a global scratch slab.
#include "tk_warp.cuh"

#include <algorithm>

namespace tk {

constexpr int RT_THREADS = 256;
constexpr int RT_SPAN = 32;
constexpr uint32_t RT_WARP_MAX = 256;

int parse_reads(tk_ctx *c, tk_reads *r);
int table_alloc_init(tk_table *t, uint64_t capacity, uint32_t init_val);

template <bool CANON>
__global__ void __launch_bounds__(RT_THREADS) k_r2t_build(const uint8_t *__restrict__ seq, uint64_t n,
                                                         const uint64_t *__restrict__ rd_off, uint64_t n_rec, int k,
                                                         DevTable t, int max_probes, uint32_t *__restrict__ err) {
    const uint64_t kmask = (1ULL << (2 * k)) - 1;
    const int shift = 2 * (k - 1);
    const uint64_t stride = (uint64_t)gridDim.x * RT_THREADS * RT_SPAN;
    for (uint64_t p0 = ((uint64_t)blockIdx.x * RT_THREADS + threadIdx.x) * RT_SPAN; p0 < n; p0 += stride) {
        // record holding position p0: largest r with rd_off[r] <= p0
        uint64_t lo = 0, hi = n_rec;
        while (hi - lo > 1) {
            uint64_t mid = (lo + hi) >> 1;
            if (rd_off[mid] <= p0) lo = mid; else hi = mid;
        }
        uint64_t rec = lo;
        uint64_t next = rd_off[rec + 1];
        uint64_t fw = 0, rc = 0;
        int run = 0;
        const uint8_t *p = seq + p0 - 32;
#pragma unroll 4
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
                uint64_t e = p0 - 32 + j;
                while (e >= next && rec + 1 < n_rec) { rec++; next = rd_off[rec + 1]; }
                uint64_t key = (CANON && rc < fw) ? rc : fw;
                if (!tbl_min(t, key, (uint32_t)rec, max_probes)) atomicExch(&err[DE_OVERFLOW], 1u);
            }
        }
    }
}

template <int S, bool CANON>
__device__ __forceinline__ void r2t_warp_read(DevTable t, const uint8_t *__restrict__ seq, uint64_t start, uint32_t nwin,
                                              int k, uint64_t r, int32_t *__restrict__ rec, uint32_t *__restrict__ hits,
                                              uint64_t *words) {
    const unsigned lane = lane_id();
    const uint32_t span = (nwin + 31) / 32;
    uint32_t v[S];
    auto body = [&](int j, bool valid, uint64_t key) { v[j] = valid ? tbl_get(t, key, PAD_VAL) : PAD_VAL; };
    // k-mers cut from the read packed in shared memory; reads with another
    // character take the byte path
    if (!lane_windows_packed<S, CANON>(seq, start, nwin, span, k, words, body))
        lane_windows<S, CANON>(seq, start, nwin, span, k, body);
    warp_bitonic_sort<S>(v);
    // longest run of equal values; run start indices by an inclusive max-scan
    uint32_t prev_last = __shfl_up_sync(0xffffffffu, v[S - 1], 1);
    int last_start = -1;
    int st[S];
#pragma unroll
    for (int j = 0; j < S; j++) {
        uint32_t prev = j ? v[j - 1] : prev_last;
        bool is_start = (lane == 0 && j == 0) || v[j] != prev;
        if (is_start) last_start = (int)(lane * S + j);
        st[j] = last_start;
    }
    int carry = last_start;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        int x = __shfl_up_sync(0xffffffffu, carry, o);
        if ((int)lane >= o) carry = max(carry, x);
    }
    int before = __shfl_up_sync(0xffffffffu, carry, 1);
    if (lane == 0) before = -1;
    uint64_t best = 0;   // (run length << 32) | (0xFFFFFFFF - value)
#pragma unroll
    for (int j = 0; j < S; j++) {
        int s0 = st[j] < 0 ? before : st[j];
        uint32_t len = (uint32_t)((int)(lane * S + j) - s0 + 1);
        if (v[j] != PAD_VAL) {
            uint64_t cand = ((uint64_t)len << 32) | (uint64_t)(0xFFFFFFFFu - v[j]);
            best = max(best, cand);
        }
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) best = max(best, __shfl_xor_sync(0xffffffffu, best, o));
    if (lane == 0) {
        if (best == 0) {
            rec[r] = -1;
            hits[r] = 0;
        } else {
            rec[r] = (int32_t)(0xFFFFFFFFu - (uint32_t)best);
            hits[r] = (uint32_t)(best >> 32);
        }
    }
}

template <bool CANON>
__global__ void __launch_bounds__(RT_THREADS, 6) k_r2t_assign(DevTable t, const uint8_t *__restrict__ seq,
                                                             const uint64_t *__restrict__ rd_off, uint64_t n_reads,
                                                             int k, int32_t *__restrict__ rec,
                                                             uint32_t *__restrict__ hits, uint32_t *__restrict__ nwin_out,
                                                             uint32_t *__restrict__ long_list,
                                                             unsigned long long *__restrict__ long_n) {
    __shared__ uint64_t words[RT_THREADS / 32][12];
    uint64_t *w = words[threadIdx.x >> 5];
    const uint64_t warps = (uint64_t)gridDim.x * (RT_THREADS / 32);
    for (uint64_t r = (uint64_t)blockIdx.x * (RT_THREADS / 32) + (threadIdx.x >> 5); r < n_reads; r += warps) {
        const uint64_t start = rd_off[r];
        const uint64_t L = rd_off[r + 1] - start - 1;
        const uint32_t nwin = L >= (uint64_t)k ? (uint32_t)(L - k + 1) : 0u;
        if (lane_id() == 0) nwin_out[r] = nwin;
        if (nwin <= 32) r2t_warp_read<1, CANON>(t, seq, start, nwin, k, r, rec, hits, w);
        else if (nwin <= 64) r2t_warp_read<2, CANON>(t, seq, start, nwin, k, r, rec, hits, w);
        else if (nwin <= 128) r2t_warp_read<4, CANON>(t, seq, start, nwin, k, r, rec, hits, w);
        else if (nwin <= RT_WARP_MAX) r2t_warp_read<8, CANON>(t, seq, start, nwin, k, r, rec, hits, w);
        else if (lane_id() == 0) long_list[atomicAdd(long_n, 1ULL)] = (uint32_t)r;
    }
}

template <bool CANON>
__global__ void __launch_bounds__(RT_THREADS) k_r2t_long(DevTable t, const uint8_t *__restrict__ seq,
                                                        const uint64_t *__restrict__ rd_off,
                                                        const uint32_t *__restrict__ list, uint64_t n_long, int k,
                                                        uint32_t *__restrict__ scratch, uint64_t n2max,
                                                        int32_t *__restrict__ rec, uint32_t *__restrict__ hits) {
    uint32_t *slab = scratch + (uint64_t)blockIdx.x * n2max;
    for (uint64_t i = blockIdx.x; i < n_long; i += gridDim.x) {
        const uint32_t r = list[i];
        const uint64_t start = rd_off[r];
        const uint32_t nwin = (uint32_t)(rd_off[r + 1] - start - 1 - (k - 1));
        uint32_t n2 = 1;
        while (n2 < nwin) n2 <<= 1;
        block_window_values<CANON>(seq, start, nwin, n2, k, slab, [&](uint64_t key) { return tbl_get(t, key, PAD_VAL); });
        block_bitonic_sort(slab, n2);
        if (threadIdx.x == 0) {
            uint32_t best_len = 0, best_v = PAD_VAL;
            for (uint32_t a = 0; a < n2 && slab[a] != PAD_VAL;) {
                uint32_t b = a;
                while (b < n2 && slab[b] == slab[a]) b++;
                if (b - a > best_len) { best_len = b - a; best_v = slab[a]; }
                a = b;
            }
            rec[r] = best_len ? (int32_t)best_v : -1;
            hits[r] = best_len;
        }
        __syncthreads();
    }
}

int r2t_build(tk_r2t *z, const tk_reads *b) {
    tk_ctx *c = z->ctx;
    tk_table *t = z->table;
    uint64_t want = 1024;
    while (want < 2 * std::max<uint64_t>(b->n_bases, 1)) want <<= 1;
    TK_TRY(table_alloc_init(t, want, PAD_VAL));
    if (b->n_reads == 0 || b->seq_len == 0) return TK_OK;
    TK_CUDA(c, cudaMemsetAsync(c->d_err, 0, DE_COUNT * 4, c->stream));
    const uint64_t n = b->seq_len;
    const unsigned grid = (unsigned)std::max<uint64_t>(
        1, std::min<uint64_t>((n + RT_THREADS * RT_SPAN - 1) / (RT_THREADS * RT_SPAN), (uint64_t)c->sm_count * 16));
    cudaEvent_t ev;
    prof_begin(c, TK_KID_R2T_BUILD, &ev);
    if (!z->strand)
        k_r2t_build<true><<<grid, RT_THREADS, 0, c->stream>>>(b->d_seq, n, b->d_rd_off, b->n_reads, z->k, t->t,
                                                              c->max_probes, c->d_err);
    else
        k_r2t_build<false><<<grid, RT_THREADS, 0, c->stream>>>(b->d_seq, n, b->d_rd_off, b->n_reads, z->k, t->t,
                                                               c->max_probes, c->d_err);
    c->launches++;
    prof_end(c, TK_KID_R2T_BUILD, ev, b->n_bases);
    TK_TRY(check_launch(c, "r2t build"));
    uint32_t herr[DE_COUNT];
    TK_CUDA(c, cudaMemcpyAsync(herr, c->d_err, sizeof(herr), cudaMemcpyDeviceToHost, c->stream));
    TK_CUDA(c, cudaStreamSynchronize(c->stream));
    if (herr[DE_OVERFLOW]) return set_err(c, TK_E_TABLE_FULL, "bundle k-mer table: probe limit reached");
    t->distinct_valid = false;
    return TK_OK;
}

int r2t_assign(tk_r2t *z, const tk_reads *rd, int32_t *d_rec, uint32_t *d_hits, uint32_t *d_nwin) {
    tk_ctx *c = z->ctx;
    const uint64_t n = rd->n_reads;
    if (n == 0) return TK_OK;
    const int k = z->k;
    const bool may_long = rd->max_len >= (uint32_t)k && rd->max_len - k + 1 > RT_WARP_MAX;
    uint32_t *long_list = nullptr;
    unsigned long long *long_n = nullptr;
    TK_TRY(dmalloc(c, (void **)&long_n, 8, "long-read count"));
    int e = TK_OK;
    if (may_long) e = dmalloc(c, (void **)&long_list, n * 4, "long-read list");
    if (!e) e = cuda_check(c, cudaMemsetAsync(long_n, 0, 8, c->stream), "long reset");
    if (!e) {
        const unsigned grid = (unsigned)std::max<uint64_t>(
            1, std::min<uint64_t>((n + RT_THREADS / 32 - 1) / (RT_THREADS / 32), (uint64_t)c->sm_count * 16));
        cudaEvent_t ev;
        prof_begin(c, TK_KID_R2T_ASSIGN, &ev);
        if (!z->strand)
            k_r2t_assign<true><<<grid, RT_THREADS, 0, c->stream>>>(z->table->t, rd->d_seq, rd->d_rd_off, n, k, d_rec,
                                                                   d_hits, d_nwin, long_list, long_n);
        else
            k_r2t_assign<false><<<grid, RT_THREADS, 0, c->stream>>>(z->table->t, rd->d_seq, rd->d_rd_off, n, k, d_rec,
                                                                    d_hits, d_nwin, long_list, long_n);
        c->launches++;
        prof_end(c, TK_KID_R2T_ASSIGN, ev, rd->n_bases);
        e = check_launch(c, "r2t assign");
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
            if (!z->strand)
                k_r2t_long<true><<<(unsigned)grid, RT_THREADS, 0, c->stream>>>(z->table->t, rd->d_seq, rd->d_rd_off,
                                                                               long_list, hl, k, scratch, n2max, d_rec,
                                                                               d_hits);
            else
                k_r2t_long<false><<<(unsigned)grid, RT_THREADS, 0, c->stream>>>(z->table->t, rd->d_seq, rd->d_rd_off,
                                                                                long_list, hl, k, scratch, n2max, d_rec,
                                                                                d_hits);
            c->launches++;
            e = check_launch(c, "r2t long");
            dfree(c, scratch);
        }
    }
    if (long_list) dfree(c, long_list);
    dfree(c, long_n);
    return e;
}

}  // namespace tk
