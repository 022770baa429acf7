// tk_scan.cu -- device-wide exclusive scan and LSD radix sort of (u64 key,
// u32 value) pairs.  Both are plain streaming kernels (HBM-bound): the scan
// reads its input twice and writes once; each radix pass reads and writes the
// pairs once and scatters a tile's items per digit in input order (stable).
#include "tk_internal.cuh"

namespace tk {

constexpr int SC_THREADS = 256;
constexpr int SC_ITEMS = 16;
constexpr uint64_t SC_TILE = (uint64_t)SC_THREADS * SC_ITEMS;

template <typename Tin>
__global__ void k_scan_reduce(const Tin *__restrict__ in, uint64_t n, uint64_t *__restrict__ sums) {
    __shared__ uint64_t sm[SC_THREADS / 32 + 1];
    uint64_t base = (uint64_t)blockIdx.x * SC_TILE;
    uint64_t s = 0;
#pragma unroll
    for (int i = 0; i < SC_ITEMS; i++) {
        uint64_t idx = base + (uint64_t)i * SC_THREADS + threadIdx.x;
        if (idx < n) s += (uint64_t)in[idx];
    }
    uint64_t tot;
    block_excl_scan<uint64_t>(s, sm, &tot);
    if (threadIdx.x == 0) sums[blockIdx.x] = tot;
}

// single block; exclusive scan in place over nb sums, total to sums[nb]
__global__ void k_scan_sums(uint64_t *sums, uint64_t nb) {
    __shared__ uint64_t sm[SC_THREADS / 32 + 1];
    uint64_t carry = 0;
    for (uint64_t base = 0; base < nb; base += SC_THREADS) {
        uint64_t idx = base + threadIdx.x;
        uint64_t v = idx < nb ? sums[idx] : 0;
        uint64_t tot;
        uint64_t ex = block_excl_scan<uint64_t>(v, sm, &tot);
        if (idx < nb) sums[idx] = carry + ex;
        carry += tot;
    }
    if (threadIdx.x == 0) sums[nb] = carry;
}

template <typename Tin>
__global__ void k_scan_down(const Tin *__restrict__ in, uint64_t *__restrict__ out, uint64_t n,
                            const uint64_t *__restrict__ sums) {
    __shared__ uint64_t sm[SC_THREADS / 32 + 1];
    // blocked arrangement inside the tile: thread t owns items [t*ITEMS, (t+1)*ITEMS)
    uint64_t base = (uint64_t)blockIdx.x * SC_TILE + (uint64_t)threadIdx.x * SC_ITEMS;
    uint64_t v[SC_ITEMS];
    uint64_t s = 0;
#pragma unroll
    for (int i = 0; i < SC_ITEMS; i++) {
        uint64_t idx = base + i;
        v[i] = idx < n ? (uint64_t)in[idx] : 0;
        s += v[i];
    }
    uint64_t tot;
    uint64_t ex = block_excl_scan<uint64_t>(s, sm, &tot) + sums[blockIdx.x];
#pragma unroll
    for (int i = 0; i < SC_ITEMS; i++) {
        uint64_t idx = base + i;
        if (idx < n) out[idx] = ex;
        ex += v[i];
    }
}

template <typename Tin>
static int scan_impl(tk_ctx *c, const Tin *in, uint64_t *out, uint64_t n, uint64_t *total_host) {
    if (n == 0) {
        if (total_host) *total_host = 0;
        return TK_OK;
    }
    uint64_t nb = (n + SC_TILE - 1) / SC_TILE;
    uint64_t *sums = nullptr;
    TK_TRY(dmalloc(c, (void **)&sums, (nb + 1) * sizeof(uint64_t), "scan sums"));
    k_scan_reduce<Tin><<<(unsigned)nb, SC_THREADS, 0, c->stream>>>(in, n, sums);
    c->launches++;
    int e = TK_OK;
    if (nb > 65536) {
        // scan the block sums with the same machinery, then fix up the total
        uint64_t *sums2 = nullptr;
        e = dmalloc(c, (void **)&sums2, (nb + 1) * sizeof(uint64_t), "scan sums2");
        if (!e) {
            uint64_t tot = 0;
            e = scan_impl<uint64_t>(c, sums, sums2, nb, &tot);
            if (!e) {
                cudaMemcpyAsync(sums, sums2, nb * sizeof(uint64_t), cudaMemcpyDeviceToDevice, c->stream);
                cudaMemcpyAsync(sums + nb, &tot, sizeof(uint64_t), cudaMemcpyHostToDevice, c->stream);
                e = cuda_check(c, cudaStreamSynchronize(c->stream), "scan sums sync");
            }
            dfree(c, sums2);
        }
    } else {
        k_scan_sums<<<1, SC_THREADS, 0, c->stream>>>(sums, nb);
        c->launches++;
    }
    if (!e) {
        k_scan_down<Tin><<<(unsigned)nb, SC_THREADS, 0, c->stream>>>(in, out, n, sums);
        c->launches++;
        e = check_launch(c, "scan");
    }
    if (!e && total_host) {
        e = cuda_check(c, cudaMemcpyAsync(total_host, sums + nb, sizeof(uint64_t), cudaMemcpyDeviceToHost, c->stream), "scan total");
        if (!e) e = cuda_check(c, cudaStreamSynchronize(c->stream), "scan total sync");
    }
    dfree(c, sums);
    return e;
}

int scan_excl_u64(tk_ctx *c, const uint64_t *in, uint64_t *out, uint64_t n, uint64_t *total_host) {
    return scan_impl<uint64_t>(c, in, out, n, total_host);
}

int scan_excl_u32_to_u64(tk_ctx *c, const uint32_t *in, uint64_t *out, uint64_t n, uint64_t *total_host) {
    return scan_impl<uint32_t>(c, in, out, n, total_host);
}

// ------------------------------------------------------------------ radix sort

constexpr int RS_THREADS = 256;
constexpr int RS_ROUNDS = 16;                 // items per thread per tile
constexpr int RS_BITS = 8;
constexpr int RS_BINS = 1 << RS_BITS;
constexpr uint64_t RS_TILE = (uint64_t)RS_THREADS * RS_ROUNDS;

// per tile digit histogram, stored digit-major: hist[d * ntiles + tile]
__global__ void k_rs_hist(const uint64_t *__restrict__ keys, uint64_t n, int shift, uint32_t *__restrict__ hist,
                          uint64_t ntiles) {
    __shared__ uint32_t h[RS_BINS];
    for (int i = threadIdx.x; i < RS_BINS; i += RS_THREADS) h[i] = 0;
    __syncthreads();
    uint64_t base = (uint64_t)blockIdx.x * RS_TILE;
#pragma unroll 4
    for (int r = 0; r < RS_ROUNDS; r++) {
        uint64_t idx = base + (uint64_t)r * RS_THREADS + threadIdx.x;
        if (idx < n) atomicAdd(&h[(keys[idx] >> shift) & (RS_BINS - 1)], 1u);
    }
    __syncthreads();
    for (int i = threadIdx.x; i < RS_BINS; i += RS_THREADS) hist[(uint64_t)i * ntiles + blockIdx.x] = h[i];
}

// stable scatter: items of a tile are ranked round by round (striped), and
// within a round by warp then lane, which is input order.
__global__ void k_rs_scatter(const uint64_t *__restrict__ keys, const uint32_t *__restrict__ vals,
                             uint64_t *__restrict__ okeys, uint32_t *__restrict__ ovals, uint64_t n, int shift,
                             const uint64_t *__restrict__ offs, uint64_t ntiles) {
    constexpr int NW = RS_THREADS / 32;
    __shared__ uint32_t wcnt[NW][RS_BINS];   // per warp digit counts, then their prefix over warps
    __shared__ uint32_t rtot[RS_BINS];       // this round's count per digit
    __shared__ uint32_t run[RS_BINS];        // items of each digit already placed by this tile
    __shared__ uint64_t gbase[RS_BINS];
    const unsigned lane = lane_id(), warp = threadIdx.x >> 5;
    for (int i = threadIdx.x; i < RS_BINS; i += RS_THREADS) {
        run[i] = 0;
        gbase[i] = offs[(uint64_t)i * ntiles + blockIdx.x];
    }
    const uint64_t base = (uint64_t)blockIdx.x * RS_TILE;
    const unsigned lt_mask = (1u << lane) - 1u;
    for (int r = 0; r < RS_ROUNDS; r++) {
        for (int i = threadIdx.x; i < NW * RS_BINS; i += RS_THREADS) (&wcnt[0][0])[i] = 0;
        __syncthreads();
        uint64_t idx = base + (uint64_t)r * RS_THREADS + threadIdx.x;
        bool valid = idx < n;
        uint64_t key = valid ? keys[idx] : 0;
        uint32_t val = valid ? vals[idx] : 0;
        uint32_t d = valid ? (uint32_t)((key >> shift) & (RS_BINS - 1)) : (uint32_t)RS_BINS;
        unsigned peers = __match_any_sync(0xffffffffu, d);
        uint32_t wrank = __popc(peers & lt_mask);
        if (valid && wrank == 0) wcnt[warp][d] = __popc(peers);
        __syncthreads();
        for (int dd = threadIdx.x; dd < RS_BINS; dd += RS_THREADS) {
            uint32_t acc = 0;
#pragma unroll
            for (int w = 0; w < NW; w++) {
                uint32_t cnt = wcnt[w][dd];
                wcnt[w][dd] = acc;
                acc += cnt;
            }
            rtot[dd] = acc;
        }
        __syncthreads();
        if (valid) {
            uint64_t pos = gbase[d] + run[d] + wcnt[warp][d] + wrank;
            okeys[pos] = key;
            ovals[pos] = val;
        }
        __syncthreads();
        for (int dd = threadIdx.x; dd < RS_BINS; dd += RS_THREADS) run[dd] += rtot[dd];
    }
}

int radix_sort_pairs(tk_ctx *c, uint64_t *keys, uint32_t *vals, uint64_t n, int bits, uint64_t *tmp_keys,
                     uint32_t *tmp_vals, bool *result_in_tmp) {
    *result_in_tmp = false;
    if (n <= 1 || bits <= 0) return TK_OK;
    uint64_t ntiles = (n + RS_TILE - 1) / RS_TILE;
    uint32_t *hist = nullptr;
    uint64_t *offs = nullptr;
    TK_TRY(dmalloc(c, (void **)&hist, ntiles * RS_BINS * sizeof(uint32_t), "radix hist"));
    int e = dmalloc(c, (void **)&offs, ntiles * RS_BINS * sizeof(uint64_t), "radix offsets");
    if (e) { dfree(c, hist); return e; }
    uint64_t *ka = keys, *kb = tmp_keys;
    uint32_t *va = vals, *vb = tmp_vals;
    for (int shift = 0; shift < bits && !e; shift += RS_BITS) {
        k_rs_hist<<<(unsigned)ntiles, RS_THREADS, 0, c->stream>>>(ka, n, shift, hist, ntiles);
        c->launches++;
        e = scan_excl_u32_to_u64(c, hist, offs, ntiles * RS_BINS, nullptr);
        if (e) break;
        k_rs_scatter<<<(unsigned)ntiles, RS_THREADS, 0, c->stream>>>(ka, va, kb, vb, n, shift, offs, ntiles);
        c->launches++;
        e = check_launch(c, "radix scatter");
        uint64_t *tk_ = ka; ka = kb; kb = tk_;
        uint32_t *tv = va; va = vb; vb = tv;
        *result_in_tmp = !*result_in_tmp;
    }
    dfree(c, hist);
    dfree(c, offs);
    return e;
}

}  // namespace tk
