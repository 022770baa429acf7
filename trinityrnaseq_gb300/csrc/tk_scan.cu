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
constexpr int RS_ROUNDS = 8;                  // items per thread per tile
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

// Stable scatter of one 2048-item tile.  Warp w ranks its 256 consecutive
// items in 8 rounds of 32 (match.any inside a round, a per-warp running count
// per digit in shared memory); a scan over (digit, warp) turns the ranks into
// positions of a digit-sorted tile, which is laid out in shared memory and then
// leaves as one run per digit, consecutive threads storing consecutive items
// (runs of ~8 keys instead of one scattered 8-byte store per item).
constexpr int RS_WARPS = RS_THREADS / 32;
constexpr int RS_PER_LANE = RS_TILE / RS_THREADS;   // rounds per warp
constexpr size_t RS_SMEM = (size_t)RS_WARPS * RS_BINS * 4 + RS_BINS * 4 + RS_BINS * 8 + RS_TILE * 8 + RS_TILE * 4;

__global__ void __launch_bounds__(RS_THREADS) k_rs_scatter(const uint64_t *__restrict__ keys,
                                                          const uint32_t *__restrict__ vals,
                                                          uint64_t *__restrict__ okeys, uint32_t *__restrict__ ovals,
                                                          uint64_t n, int shift, const uint64_t *__restrict__ offs,
                                                          uint64_t ntiles) {
    extern __shared__ __align__(16) unsigned char rs_smem[];
    uint64_t *skey = reinterpret_cast<uint64_t *>(rs_smem);                              // [RS_TILE]
    unsigned long long *gbase = reinterpret_cast<unsigned long long *>(skey + RS_TILE);  // [RS_BINS]
    uint32_t *sval = reinterpret_cast<uint32_t *>(gbase + RS_BINS);                      // [RS_TILE]
    uint32_t *wcnt = sval + RS_TILE;                                                     // [RS_WARPS][RS_BINS]
    uint32_t *dstart = wcnt + RS_WARPS * RS_BINS;                                        // [RS_BINS]
    __shared__ uint32_t scan_sm[RS_WARPS + 1];
    const unsigned lane = lane_id(), warp = threadIdx.x >> 5;
    for (int i = threadIdx.x; i < RS_WARPS * RS_BINS; i += RS_THREADS) wcnt[i] = 0;
    for (int i = threadIdx.x; i < RS_BINS; i += RS_THREADS) gbase[i] = offs[(uint64_t)i * ntiles + blockIdx.x];
    __syncthreads();
    const uint64_t tile0 = (uint64_t)blockIdx.x * RS_TILE;
    const uint64_t base = tile0 + (uint64_t)warp * (RS_TILE / RS_WARPS);
    const unsigned lt_mask = (1u << lane) - 1u;
    uint32_t *mycnt = wcnt + warp * RS_BINS;
    uint64_t k[RS_PER_LANE];
    uint32_t v[RS_PER_LANE], pos[RS_PER_LANE];
#pragma unroll
    for (int r = 0; r < RS_PER_LANE; r++) {
        const uint64_t idx = base + (uint64_t)r * 32 + lane;
        const bool valid = idx < n;
        k[r] = valid ? keys[idx] : 0;
        v[r] = valid ? vals[idx] : 0;
        const uint32_t d = valid ? (uint32_t)((k[r] >> shift) & (RS_BINS - 1)) : (uint32_t)RS_BINS;
        const unsigned peers = __match_any_sync(0xffffffffu, d);
        const uint32_t rank = __popc(peers & lt_mask);
        const uint32_t cur = valid ? mycnt[d] : 0u;
        pos[r] = cur + rank;
        __syncwarp();
        if (valid && rank == 0) mycnt[d] = cur + __popc(peers);
        __syncwarp();
    }
    __syncthreads();
    // per digit: earlier warps' counts (stable order), and the digit's start in the tile
    for (int d = threadIdx.x; d < RS_BINS; d += RS_THREADS) {
        uint32_t acc = 0;
#pragma unroll
        for (int w = 0; w < RS_WARPS; w++) {
            const uint32_t c = wcnt[w * RS_BINS + d];
            wcnt[w * RS_BINS + d] = acc;
            acc += c;
        }
        dstart[d] = acc;   // the digit's total for now
    }
    __syncthreads();
    static_assert(RS_BINS == RS_THREADS, "one digit per thread in the scan");
    {
        uint32_t tot;
        const uint32_t ex = block_excl_scan<uint32_t>(dstart[threadIdx.x], scan_sm, &tot);
        __syncthreads();
        dstart[threadIdx.x] = ex;
    }
    __syncthreads();
#pragma unroll
    for (int r = 0; r < RS_PER_LANE; r++) {
        const uint64_t idx = base + (uint64_t)r * 32 + lane;
        if (idx < n) {
            const uint32_t d = (uint32_t)((k[r] >> shift) & (RS_BINS - 1));
            const uint32_t lp = dstart[d] + mycnt[d] + pos[r];
            skey[lp] = k[r];
            sval[lp] = v[r];
        }
    }
    __syncthreads();
    const uint32_t m = n - tile0 < (uint64_t)RS_TILE ? (uint32_t)(n - tile0) : (uint32_t)RS_TILE;
    for (uint32_t i = threadIdx.x; i < m; i += RS_THREADS) {
        const uint64_t key = skey[i];
        const uint32_t d = (uint32_t)((key >> shift) & (RS_BINS - 1));
        const uint64_t o = gbase[d] + (i - dstart[d]);
        okeys[o] = key;
        ovals[o] = sval[i];
    }
}

// Sorts by key bits [first_bit, first_bit + bits), 8 bits per pass.
int radix_sort_pairs(tk_ctx *c, uint64_t *keys, uint32_t *vals, uint64_t n, int bits, uint64_t *tmp_keys,
                     uint32_t *tmp_vals, bool *result_in_tmp, int first_bit) {
    *result_in_tmp = false;
    if (n <= 1 || bits <= 0) return TK_OK;
    uint64_t ntiles = (n + RS_TILE - 1) / RS_TILE;
    uint32_t *hist = nullptr;
    uint64_t *offs = nullptr;
    TK_TRY(dmalloc(c, (void **)&hist, ntiles * RS_BINS * sizeof(uint32_t), "radix hist"));
    int e = dmalloc(c, (void **)&offs, ntiles * RS_BINS * sizeof(uint64_t), "radix offsets");
    if (e) { dfree(c, hist); return e; }
    if (!e) e = cuda_check(c, cudaFuncSetAttribute(k_rs_scatter, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)RS_SMEM),
                           "radix scatter smem");
    uint64_t *ka = keys, *kb = tmp_keys;
    uint32_t *va = vals, *vb = tmp_vals;
    for (int shift = first_bit; shift < first_bit + bits && shift < 64 && !e; shift += RS_BITS) {
        k_rs_hist<<<(unsigned)ntiles, RS_THREADS, 0, c->stream>>>(ka, n, shift, hist, ntiles);
        c->launches++;
        e = scan_excl_u32_to_u64(c, hist, offs, ntiles * RS_BINS, nullptr);
        if (e) break;
        k_rs_scatter<<<(unsigned)ntiles, RS_THREADS, RS_SMEM, c->stream>>>(ka, va, kb, vb, n, shift, offs, ntiles);
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
