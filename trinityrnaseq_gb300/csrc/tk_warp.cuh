// tk_warp.cuh -- per-read warp machinery shared by the coverage-statistics
// (K5) and read-to-component (K6) kernels.
//
// One warp owns one read.  Lane l owns `span` consecutive windows starting at
// window l*span: it primes the rolling forward/reverse-complement words with
// k-1 bases and then rolls one base per window, so each lane reads span+k-1
// bytes of the read (L1-resident) and its values stay in registers.  The
// warp then sorts its 32*S register values with a bitonic network (compare
// exchanges inside a lane for strides < S, xor-shuffles across lanes for the
// rest).  Element i of the sorted sequence lives in lane i / S, register i % S.
#pragma once
#include "tk_internal.cuh"

namespace tk {

// S = registers per lane (power of two) able to hold `span` windows
// f(j, valid, key) is called for j = 0..S-1 (window lane*span + j)
template <int S, bool CANON, typename F>
__device__ __forceinline__ void lane_windows(const uint8_t *__restrict__ seq, uint64_t start, uint32_t nwin,
                                             uint32_t span, int k, F &&f) {
    const unsigned lane = lane_id();
    const uint64_t kmask = (1ULL << (2 * k)) - 1;
    const int shift = 2 * (k - 1);
    const uint32_t w0 = lane * span;
    uint64_t fw = 0, rc = 0;
    int run = 0;
    const uint8_t *p = seq + start + w0;
    if (w0 < nwin) {
        for (int i = 0; i < k - 1; i++) {
            uint32_t c = base_code(__ldg(p + i));
            if (c > 3) {
                run = 0;
            } else {
                fw = ((fw << 2) | c) & kmask;
                rc = (rc >> 2) | ((uint64_t)(3u - c) << shift);
                run++;
            }
        }
    }
#pragma unroll
    for (int j = 0; j < S; j++) {
        bool in = (uint32_t)j < span && w0 + j < nwin;
        bool valid = false;
        uint64_t key = 0;
        if (in) {
            uint32_t c = base_code(__ldg(p + k - 1 + j));
            if (c > 3) {
                run = 0;
            } else {
                fw = ((fw << 2) | c) & kmask;
                rc = (rc >> 2) | ((uint64_t)(3u - c) << shift);
                run++;
            }
            valid = run >= k;
            key = (CANON && rc < fw) ? rc : fw;
        }
        f(j, valid, key);
    }
}

// Reverse complement of a k-mer in 2-bit A<C<G<T code (the low 2k bits):
// complement every base, then reverse the order of the 2-bit groups.
__device__ __forceinline__ uint64_t kmer_revcomp(uint64_t fw, int k) {
    uint64_t x = __brevll(~fw);   // group order reversed, the two bits of each group swapped
    x = ((x >> 1) & 0x5555555555555555ULL) | ((x & 0x5555555555555555ULL) << 1);
    return x >> (64 - 2 * k);
}

// Packed form of lane_windows for reads made of A/C/G/T only (the common
// case): the warp first writes the read as a 2-bit, first-base-most-
// significant bit string into `words` (per-warp shared memory, 12 words),
// then lane l cuts each of its k-mers out of two words with one funnel shift,
// with no k-1 base priming per lane.  Returns false, having called f for no
// window, when the read holds any other character or has no window; the
// caller then uses lane_windows.
template <int S, bool CANON, typename F>
__device__ __forceinline__ bool lane_windows_packed(const uint8_t *__restrict__ seq, uint64_t start, uint32_t nwin,
                                                    uint32_t span, int k, uint64_t *words, F &&f) {
    constexpr int ROUNDS = (32 * S + 30 + 127) / 128;   // 128 bases per round cover nwin + k - 1 <= 32*S + 30
    static_assert(ROUNDS * 4 <= 12 && S + 1 <= ROUNDS * 4, "packed word buffer");
    if (nwin == 0) return false;
    const unsigned lane = lane_id();
    const uint32_t L = nwin + (uint32_t)k - 1;
    uint8_t *bytes = reinterpret_cast<uint8_t *>(words);
    bool bad = false;
    __syncwarp();
#pragma unroll
    for (int rd = 0; rd < ROUNDS; rd++) {
        const uint32_t g = (uint32_t)rd * 32 + lane;   // bases 4g .. 4g+3
        uint32_t byte = 0;
#pragma unroll
        for (int i = 0; i < 4; i++) {
            const uint32_t p = 4 * g + i;
            if (p < L) {
                const uint32_t c = base_code(__ldg(seq + start + p));
                bad |= c > 3;
                byte |= (c & 3u) << (6 - 2 * i);
            }
        }
        bytes[(g & ~7u) + (7u - (g & 7u))] = (uint8_t)byte;   // group 8q+i -> byte 7-i of word q
    }
    if (__any_sync(0xffffffffu, bad)) return false;
    __syncwarp();
    const uint64_t kmask = (1ULL << (2 * k)) - 1;
    const uint32_t w0 = lane * span;
#pragma unroll
    for (int j = 0; j < S; j++) {
        const uint32_t w = w0 + j;
        const bool in = (uint32_t)j < span && w < nwin;
        uint64_t key = 0;
        if (in) {
            const uint32_t q = w >> 5, off = 2 * (w & 31);
            uint64_t x = words[q];
            if (off) x = (x << off) | (words[q + 1] >> (64 - off));
            const uint64_t fw = (x >> (64 - 2 * k)) & kmask;
            if (CANON) {
                const uint64_t rc = kmer_revcomp(fw, k);
                key = rc < fw ? rc : fw;
            } else {
                key = fw;
            }
        }
        f(j, in, key);
    }
    return true;
}

// Windows of one read cut from the read set's 2-bit codes (codes[j] holds
// positions 32j .. 32j+31, first position in the top bits; bit 31-i of inv[j]
// is set when position 32j+i is not A/C/G/T; word -1 exists).  Lane l owns
// windows [l*span, l*span + span) of the read starting at position `start`;
// with span <= 8 their end positions fall in two consecutive code words, so
// the lane loads three words (and their invalid bits) once and cuts each
// window out of a pair with one funnel shift.  f(j, valid, key) for
// j = 0..S-1 (window lane*span + j).
template <int S, bool CANON, typename F>
__device__ __forceinline__ void lane_windows_codes(const uint64_t *__restrict__ codes,
                                                   const uint32_t *__restrict__ inv, uint64_t start, uint32_t nwin,
                                                   uint32_t span, int k, F &&f) {
    static_assert(S <= 8, "a lane's windows end in at most two code words");
    const uint32_t w0 = lane_id() * span;
    const uint64_t e0 = start + w0 + (uint64_t)k - 1;   // end position of the lane's first window
    const int64_t q0 = (int64_t)(e0 >> 5);
    uint64_t c0 = 0, c1 = 0, c2 = 0;
    uint32_t i0 = ~0u, i1 = ~0u, i2 = ~0u;
    if (w0 < nwin) {
        c0 = __ldg(codes + q0 - 1);
        c1 = __ldg(codes + q0);
        c2 = __ldg(codes + q0 + 1);
        i0 = __ldg(inv + q0 - 1);
        i1 = __ldg(inv + q0);
        i2 = __ldg(inv + q0 + 1);
    }
    const uint64_t kmask = (1ULL << (2 * k)) - 1;
    const uint64_t vmask = (1ULL << k) - 1;
    const uint32_t e_off = (uint32_t)(e0 & 31);
#pragma unroll
    for (int j = 0; j < S; j++) {
        const bool in = (uint32_t)j < span && w0 + j < nwin;
        bool valid = false;
        uint64_t key = 0;
        if (in) {
            // the window ends at position 32 + i of the pair (words q-1, q)
            const uint32_t e = e_off + (uint32_t)j;
            const bool second = e >= 32;
            const int i = (int)(e & 31);
            const uint64_t hi = second ? c1 : c0, lo = second ? c2 : c1;
            const uint64_t m = second ? (((uint64_t)i1 << 32) | i2) : (((uint64_t)i0 << 32) | i1);
            valid = ((m >> (31 - i)) & vmask) == 0;
            const int s = 62 - 2 * i;
            const uint64_t fw = (s ? ((lo >> s) | (hi << (64 - s))) : lo) & kmask;
            key = fw;
            if (CANON) {
                const uint64_t rc = kmer_revcomp(fw, k);
                key = rc < fw ? rc : fw;
            }
        }
        f(j, valid, key);
    }
}

// Element m (0-based, ascending) of the warp's valid values -- value v[j] of a
// lane counts when bit j of its vm is set -- by a bit-serial radix select from
// the top bit of the largest value: per bit, the values still in the running
// (valid, and equal to the prefix chosen so far above this bit: bit j of
// `alive`) that have a 0 there are counted with one warp-wide add; the target
// has a 0 there when m is below that count, and the running set shrinks to
// the values on the target's side.  Costs one pass per significant bit of the
// largest count instead of a full sort.
template <int S>
__device__ __forceinline__ uint32_t warp_select(const uint32_t (&v)[S], uint32_t vm, uint32_t m, uint32_t mx) {
    // mx: the largest valid value of the warp
    uint32_t prefix = 0, alive = vm;
    for (int b = 31 - __clz(mx); b >= 0; b--) {   // no pass when every value is 0
        uint32_t ones = 0;
#pragma unroll
        for (int j = 0; j < S; j++) ones |= ((v[j] >> b) & 1u) << j;
        const uint32_t zeros = alive & ~ones;
        const uint32_t c = __reduce_add_sync(0xffffffffu, (uint32_t)__popc(zeros));
        if (m < c) {
            alive = zeros;
        } else {
            m -= c;
            prefix |= 1u << b;
            alive &= ones;
        }
    }
    return prefix;
}

template <int S>
__device__ __forceinline__ void warp_bitonic_sort(uint32_t (&v)[S]) {
    const unsigned lane = lane_id();
#pragma unroll
    for (int size = 2; size <= 32 * S; size <<= 1) {
#pragma unroll
        for (int stride = size >> 1; stride > 0; stride >>= 1) {
            if (stride < S) {
#pragma unroll
                for (int j = 0; j < S; j++) {
                    const int pj = j ^ stride;
                    if (pj > j) {
                        const unsigned i = lane * S + j;
                        const bool asc = (i & size) == 0;
                        uint32_t a = v[j], b = v[pj];
                        bool sw = asc ? (a > b) : (a < b);
                        v[j] = sw ? b : a;
                        v[pj] = sw ? a : b;
                    }
                }
            } else {
                const int ls = stride / S;
#pragma unroll
                for (int j = 0; j < S; j++) {
                    uint32_t o = __shfl_xor_sync(0xffffffffu, v[j], ls);
                    const unsigned i = lane * S + j;
                    const bool asc = (i & size) == 0;
                    const bool lower = (lane & ls) == 0;
                    uint32_t mn = min(v[j], o), mx = max(v[j], o);
                    v[j] = (lower == asc) ? mn : mx;
                }
            }
        }
    }
}

// element m of the sorted blocked sequence, broadcast to the warp
template <int S>
__device__ __forceinline__ uint32_t warp_elem(const uint32_t (&v)[S], uint32_t m) {
    uint32_t jj = m % S, x = v[0];
#pragma unroll
    for (int j = 1; j < S; j++)
        if ((uint32_t)j == jj) x = v[j];
    return __shfl_sync(0xffffffffu, x, (int)(m / S));
}

__device__ __forceinline__ void warp_sum_u128(uint64_t &hi, uint64_t &lo) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        uint64_t ohi = __shfl_xor_sync(0xffffffffu, hi, o);
        uint64_t olo = __shfl_xor_sync(0xffffffffu, lo, o);
        uint64_t nlo = lo + olo;
        hi = hi + ohi + (nlo < lo ? 1u : 0u);
        lo = nlo;
    }
}

// Statistics in the documented arithmetic: mean = (float)(sum / n);
// stdev = (float)sqrt((hi * 2^64 + lo) / (n * n)) with hi:lo = n*sumsq - sum^2.
__device__ __forceinline__ void finish_stats(uint32_t n, uint64_t sum, uint64_t sq_hi, uint64_t sq_lo,
                                             float *mean, float *stdev) {
    if (n == 0) {
        *mean = 0.0f;
        *stdev = 0.0f;
        return;
    }
    unsigned __int128 sq = ((unsigned __int128)sq_hi << 64) | sq_lo;
    unsigned __int128 num = (unsigned __int128)n * sq - (unsigned __int128)sum * sum;
    double dhi = (double)(uint64_t)(num >> 64), dlo = (double)(uint64_t)num;
    double dn = (double)n;
    double var = __ddiv_rn(__dadd_rn(__dmul_rn(dhi, 18446744073709551616.0), dlo), __dmul_rn(dn, dn));
    *mean = __double2float_rn(__ddiv_rn((double)sum, dn));
    *stdev = __double2float_rn(__dsqrt_rn(var));
}

// Block-wide bitonic sort of n2 (power of two) values in global scratch.
__device__ __forceinline__ void block_bitonic_sort(uint32_t *v, uint32_t n2) {
    for (uint32_t size = 2; size <= n2; size <<= 1) {
        for (uint32_t stride = size >> 1; stride > 0; stride >>= 1) {
            __syncthreads();
            for (uint32_t t = threadIdx.x; t < n2 / 2; t += blockDim.x) {
                uint32_t i = 2 * t - (t & (stride - 1));   // i has bit `stride` clear
                uint32_t p = i + stride;
                bool asc = (i & size) == 0;
                uint32_t a = v[i], b = v[p];
                if (asc ? (a > b) : (a < b)) {
                    v[i] = b;
                    v[p] = a;
                }
            }
        }
    }
    __syncthreads();
}

// Fills scratch[0, n2) with the read's per-window values (PAD for windows with
// a non-ACGT base and for the padding); g(valid, key) maps a window to its value.
template <bool CANON, typename G>
__device__ __forceinline__ void block_window_values(const uint8_t *__restrict__ seq, uint64_t start, uint32_t nwin,
                                                    uint32_t n2, int k, uint32_t *scratch, G &&g) {
    const uint64_t kmask = (1ULL << (2 * k)) - 1;
    const int shift = 2 * (k - 1);
    const uint32_t span = (nwin + blockDim.x - 1) / blockDim.x;
    const uint32_t w0 = threadIdx.x * span;
    uint64_t fw = 0, rc = 0;
    int run = 0;
    if (w0 < nwin) {
        const uint8_t *p = seq + start + w0;
        for (int i = 0; i < k - 1; i++) {
            uint32_t c = base_code(p[i]);
            if (c > 3) run = 0;
            else {
                fw = ((fw << 2) | c) & kmask;
                rc = (rc >> 2) | ((uint64_t)(3u - c) << shift);
                run++;
            }
        }
        for (uint32_t j = 0; j < span && w0 + j < nwin; j++) {
            uint32_t c = base_code(p[k - 1 + j]);
            if (c > 3) run = 0;
            else {
                fw = ((fw << 2) | c) & kmask;
                rc = (rc >> 2) | ((uint64_t)(3u - c) << shift);
                run++;
            }
            bool valid = run >= k;
            uint64_t key = (CANON && rc < fw) ? rc : fw;
            scratch[w0 + j] = valid ? g(key) : PAD_VAL;
        }
    }
    for (uint32_t i = nwin + threadIdx.x; i < n2; i += blockDim.x) scratch[i] = PAD_VAL;
    __syncthreads();
}

}  // namespace tk
