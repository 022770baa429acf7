// tk_norm.cu -- the normalization tail of util/insilico_read_normalization.pl
// on the GPU: what the script does with the coverage statistics once
// fastaToKmerCoverageStats has written them.
//
//   sort    each side's stats table by read name (`sort -k1,1`, LC_ALL=C;
//           insilico:865-892): rows by their first field bytewise, ties by
//           the whole line;
//   merge   util/support_scripts/nbkc_merge_left_right_stats.pl --sorted
//           (script lines 89-146): two cursors over the sorted tables; a row
//           when the accs agree without their "/digit" ending, else the cursor
//           whose acc is string-less moves on; the averages printed "%.1f";
//   select  util/support_scripts/nbkc_normalize.pl (script lines 68-117):
//           srand(12345); rows with median < min_cov, mean <= 0 or
//           stdev/mean > max_CV are dropped, every other row draws rand(1)
//           and is kept when the draw is <= max_cov / median;
//   extract make_normalized_reads_file (insilico:470-584): the records whose
//           core names were kept, in input order -- FASTQ records verbatim,
//           FASTA records as PerlLib/Fasta_reader.pm prints them; a side may
//           be several read sets (files or pieces), and every kept name must
//           be found in one of them.
//
// A side's reads may come from several read sets; names are addressed by
// their device address throughout the selection.
//
// No text table exists on the device.  Each read's "%g" fields are carried as
// (6 significant digits, decimal exponent), computed exactly from the float
// (rounded half to even on its binary value, as glibc prints), and the number
// Perl reads back from that text is the correctly rounded double of that
// decimal, D * 10^e with |e| <= 22 -- one IEEE multiplication or division of
// exact operands.  The "%.1f" averages are carried as integers N (text N/10)
// rounded the same way, and read back as N / 10.0.
//
// Sorting is an LSD radix sort of the names 8 bytes at a time (zero padded,
// big-endian), skipping the bits every name shares.  Two names whose padded
// bytes agree (equal names, or names differing only in trailing NUL bytes)
// make the order depend on the rest of the line; when any exist the sort is
// redone on the full key (suffix text, then name length, then name bytes).
//
// The merge is the scripts' sequential two-cursor walk, run speculatively in
// chunks of MG_CHUNK left rows: chunk k starts at (k*C, the number of right
// names below left name k*C) and walks until it stands exactly on the next
// chunk's start.  The walk is deterministic, so a chunk that starts on the
// true path and reaches the next start hands over to a chunk that is on the
// true path too; the first chunk that overshoots is walked again, from its
// (true) start to the end, by one thread.  For reads named <core>/1 and
// <core>/2 every chunk meets its successor.
//
// rand(1) is drand48 (X' = 0x5DEECE66D X + 11 mod 2^48 from X0 = seed << 16 |
// 0x330E, value X'/2^48); the row with the k-th draw jumps straight to it
// with the affine map for k steps composed from the maps for 2^i steps.
#include "tk_internal.cuh"

#include <algorithm>
#include <cstring>
#include <string>

namespace tk {

constexpr int NM_THREADS = 256;
constexpr uint32_t MG_CHUNK = 256;          // left rows per speculative merge chunk
constexpr int SFX_SLOT = 48;                // bytes per read of "\t%u\t%g\t%g" (full-key sort)

enum : uint32_t { NE_DOMAIN = 0, NE_DIV0 = 1, NE_HASH = 2, NE_WORDS = 4 };
enum : uint8_t { MG_REACHED = 0, MG_END = 1, MG_FAIL = 2 };

__constant__ uint64_t c_pow10[20] = {1ull, 10ull, 100ull, 1000ull, 10000ull, 100000ull, 1000000ull, 10000000ull,
                                     100000000ull, 1000000000ull, 10000000000ull, 100000000000ull,
                                     1000000000000ull, 10000000000000ull, 100000000000000ull,
                                     1000000000000000ull, 10000000000000000ull, 100000000000000000ull,
                                     1000000000000000000ull, 10000000000000000000ull};
__constant__ double c_pow10d[23] = {1e0,  1e1,  1e2,  1e3,  1e4,  1e5,  1e6,  1e7,  1e8,  1e9,  1e10, 1e11,
                                    1e12, 1e13, 1e14, 1e15, 1e16, 1e17, 1e18, 1e19, 1e20, 1e21, 1e22};
__constant__ uint64_t c_lcg_a[48], c_lcg_c[48];   // drand48 advanced 2^i steps: X -> a X + c

constexpr uint64_t LCG_MASK = (1ULL << 48) - 1;

typedef unsigned __int128 u128;

// ---------------------------------------------------------------- exact decimal

// a / 2^sh rounded half to even, 1 <= sh <= 127
__device__ __forceinline__ uint64_t shr_rne(u128 a, int sh) {
    const u128 q = a >> sh, r = a & ((((u128)1) << sh) - 1), h = ((u128)1) << (sh - 1);
    uint64_t v = (uint64_t)q;
    if (r > h || (r == h && (v & 1))) v++;
    return v;
}

// a / d rounded half to even
__device__ __forceinline__ uint64_t div_rne(uint64_t a, uint64_t d) {
    uint64_t q = a / d;
    const uint64_t r = a - q * d;
    if (r > d - r || (r == d - r && (q & 1))) q++;
    return q;
}

// m * 2^q * 10^s rounded half to even (m < 2^24; callers keep s in [-14, 22])
__device__ uint64_t scaled_rne(uint32_t m, int q, int s) {
    if (s >= 0) {
        u128 a = (u128)m * c_pow10[s > 19 ? 19 : s];
        if (s > 19) a *= c_pow10[s - 19];
        if (q >= 0) return (uint64_t)(a << q);
        return shr_rne(a, -q);
    }
    const int t = -s;
    if (q >= 0) return div_rne((uint64_t)m << q, c_pow10[t]);
    return div_rne(m, c_pow10[t] << (-q));
}

// printf("%g") of (double)f as 6 significant digits D and exponent X (value =
// D * 10^(X-5)); D = 0 for zero.  False outside 0 or [1e-17, 1.8e19).
__device__ bool g6(float f, uint32_t *D, int *X) {
    if (f == 0.0f) {
        *D = 0;
        *X = 0;
        return true;
    }
    if (!(f >= 1e-17f) || !(f < 1.8e19f)) return false;
    const uint32_t bits = __float_as_uint(f);
    const int be = (int)((bits >> 23) & 0xFF);
    const uint32_t m = (bits & 0x7FFFFFu) | 0x800000u;   // normal in this range
    const int q = be - 150;
    // floor(log10 f) to within one: the binade's exponent times log10(2) ~ 1233/4096
    int x = ((be - 127) * 1233) >> 12;
    for (int it = 0; it < 4; it++) {
        const uint64_t d = scaled_rne(m, q, 5 - x);
        if (d >= 1000000) { x++; continue; }
        if (d < 100000) { x--; continue; }
        *D = (uint32_t)d;
        *X = x;
        return true;
    }
    return false;
}

// the double Perl reads from the "%g" text of (D, X)
__device__ __forceinline__ double g6_value(uint32_t D, int X) {
    if (D == 0) return 0.0;
    const int e = X - 5;
    return e >= 0 ? __dmul_rn((double)D, c_pow10d[e]) : __ddiv_rn((double)D, c_pow10d[-e]);
}

// printf("%.1f") of y >= 0 as N (text N/10 "." N%10); false outside [0, 1e15)
__device__ bool fix1(double y, uint64_t *N) {
    if (y == 0.0) {
        *N = 0;
        return true;
    }
    if (!(y > 0.0) || !(y < 1e15)) return false;
    const uint64_t bits = (uint64_t)__double_as_longlong(y);
    const int be = (int)((bits >> 52) & 0x7FF);
    uint64_t M = bits & ((1ULL << 52) - 1);
    int Q;
    if (be == 0) Q = -1074;
    else { M |= 1ULL << 52; Q = be - 1075; }
    const uint64_t W = 10 * M;   // < 2^57; y < 2^50 so Q < 0
    const int sh = -Q;
    if (sh >= 64) { *N = 0; return true; }   // y * 10 < 2^-7
    uint64_t v = W >> sh;
    const uint64_t r = W & ((1ULL << sh) - 1), h = 1ULL << (sh - 1);
    if (r > h || (r == h && (v & 1))) v++;
    *N = v;
    return true;
}

__device__ __forceinline__ uint32_t dec_len(uint64_t v) {
    uint32_t n = 1;
    while (v >= 10) { v /= 10; n++; }
    return n;
}

__device__ __forceinline__ char *put_dec(char *o, uint64_t v) {
    const uint32_t n = dec_len(v);
    for (uint32_t i = 0; i < n; i++) {
        o[n - 1 - i] = (char)('0' + v % 10);
        v /= 10;
    }
    return o + n;
}

// significant digits of D left after dropping trailing zeros (1..6)
__device__ __forceinline__ int g6_sig(uint32_t D) {
    int nz = 6;
    while (nz > 1 && D % 10 == 0) { D /= 10; nz--; }
    return nz;
}

__device__ uint32_t g6_len(uint32_t D, int X) {
    if (D == 0) return 1;
    const int nz = g6_sig(D);
    if (X < -4 || X >= 6) {
        const int ax = X < 0 ? -X : X;
        return (uint32_t)(1 + (nz > 1 ? nz : 0) + 2 + (ax >= 100 ? 3 : 2));
    }
    if (X >= 0) return (uint32_t)(X + 1 + (nz > X + 1 ? 1 + nz - (X + 1) : 0));
    return (uint32_t)(2 + (-X - 1) + nz);
}

__device__ char *put_g6(char *o, uint32_t D, int X) {
    if (D == 0) {
        *o++ = '0';
        return o;
    }
    char d[6];
    uint32_t v = D;
    for (int i = 5; i >= 0; i--) { d[i] = (char)('0' + v % 10); v /= 10; }
    const int nz = g6_sig(D);
    if (X < -4 || X >= 6) {
        *o++ = d[0];
        if (nz > 1) {
            *o++ = '.';
            for (int i = 1; i < nz; i++) *o++ = d[i];
        }
        *o++ = 'e';
        *o++ = X < 0 ? '-' : '+';
        const int ax = X < 0 ? -X : X;
        if (ax < 10) *o++ = '0';
        return put_dec(o, (uint64_t)ax);
    }
    if (X >= 0) {
        for (int i = 0; i <= X; i++) *o++ = d[i];
        if (nz > X + 1) {
            *o++ = '.';
            for (int i = X + 1; i < nz; i++) *o++ = d[i];
        }
        return o;
    }
    *o++ = '0';
    *o++ = '.';
    for (int i = 0; i < -X - 1; i++) *o++ = '0';
    for (int i = 0; i < nz; i++) *o++ = d[i];
    return o;
}

__device__ __forceinline__ uint32_t fix1_len(uint64_t N) { return dec_len(N / 10) + 2; }

__device__ __forceinline__ char *put_fix1(char *o, uint64_t N) {
    o = put_dec(o, N / 10);
    *o++ = '.';
    *o++ = (char)('0' + N % 10);
    return o;
}

__device__ __forceinline__ void flag_err(uint32_t *err, uint32_t which) { atomicExch(&err[which], 1u); }

// ---------------------------------------------------------------- per read

__global__ void k_norm_vals(uint64_t n, const uint32_t *__restrict__ med, const float *__restrict__ mean,
                            const float *__restrict__ sd, NormVal *__restrict__ out, uint32_t *__restrict__ err) {
    const uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    NormVal v;
    uint32_t Dm = 0, Ds = 0;
    int Xm = 0, Xs = 0;
    if (!g6(mean[i], &Dm, &Xm) || !g6(sd[i], &Ds, &Xs)) {
        flag_err(err, NE_DOMAIN);
        Dm = Ds = 0;
        Xm = Xs = 0;
    }
    v.med = med[i];
    v.gmean = Dm;
    v.gsd = Ds;
    v.xmean = (int8_t)Xm;
    v.xsd = (int8_t)Xs;
    v.mean = g6_value(Dm, Xm);
    v.sd = g6_value(Ds, Xs);
    v.sfx_len = (uint8_t)(3 + dec_len(v.med) + g6_len(Dm, Xm) + g6_len(Ds, Xs));
    v.pad = 0;
    out[i] = v;
}

// ---------------------------------------------------------------- name sort

// A name is addressed by its device address (reads of one side may come
// from several read sets, each with its own text).
__device__ __forceinline__ const char *at(uint64_t a) { return reinterpret_cast<const char *>(a); }

// 8 name bytes from byte 8*ch, big-endian, zero past the name's end
__device__ __forceinline__ uint64_t name_chunk(const char *__restrict__ name, uint32_t len, uint32_t ch) {
    uint64_t k = 0;
    const uint32_t b0 = ch * 8;
#pragma unroll
    for (int i = 0; i < 8; i++) {
        const uint32_t p = b0 + i;
        k = (k << 8) | (p < len ? (uint64_t)(uint8_t)name[p] : 0ull);
    }
    return k;
}

// read set -> the side's name addresses and lengths (from index first on)
__global__ void k_name_addr(const char *__restrict__ text, const uint64_t *__restrict__ name_off,
                            const uint32_t *__restrict__ name_len, uint64_t n, uint64_t *__restrict__ addr,
                            uint32_t *__restrict__ len) {
    const uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    addr[i] = reinterpret_cast<uint64_t>(text + name_off[i]);
    len[i] = name_len[i];
}

__device__ __forceinline__ uint64_t slot_chunk(const uint8_t *__restrict__ slots, uint64_t r, uint32_t ch) {
    const uint8_t *s = slots + r * SFX_SLOT + ch * 8;
    uint64_t k = 0;
#pragma unroll
    for (int i = 0; i < 8; i++) k = (k << 8) | s[i];
    return k;
}

__global__ void k_name_maxlen(const uint32_t *__restrict__ len, uint64_t n, uint32_t *__restrict__ out) {
    __shared__ uint32_t sm[NM_THREADS / 32];
    uint32_t v = 0;
    for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (uint64_t)gridDim.x * blockDim.x)
        v = max(v, len[i]);
    v = __reduce_max_sync(0xffffffffu, v);
    if (lane_id() == 0) sm[threadIdx.x >> 5] = v;
    __syncthreads();
    if (threadIdx.x == 0) {
        for (int w = 1; w < NM_THREADS / 32; w++) v = max(v, sm[w]);
        if (v) atomicMax(out, v);
    }
}

__global__ void k_iota(uint32_t *__restrict__ p, uint64_t n) {
    const uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) p[i] = (uint32_t)i;
}

// keys[i] = the sort key of read perm[i] (mode 0: name chunk ch, 1: suffix
// chunk ch, 2: name length); orand[0] |= keys, orand[1] &= keys
__global__ void k_sort_keys(const uint64_t *__restrict__ name_addr, const uint32_t *__restrict__ name_len,
                            const uint8_t *__restrict__ slots,
                            const uint32_t *__restrict__ perm, uint64_t n, int mode, uint32_t ch,
                            uint64_t *__restrict__ keys, unsigned long long *__restrict__ orand) {
    const uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    uint64_t vo = 0, va = ~0ULL;
    if (i < n) {
        const uint32_t r = perm[i];
        uint64_t k;
        if (mode == 0) k = name_chunk(at(name_addr[r]), name_len[r], ch);
        else if (mode == 1) k = slot_chunk(slots, r, ch);
        else k = name_len[r];
        keys[i] = k;
        vo = va = k;
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        vo |= __shfl_xor_sync(0xffffffffu, vo, o);
        va &= __shfl_xor_sync(0xffffffffu, va, o);
    }
    __shared__ unsigned long long so[NM_THREADS / 32], sa[NM_THREADS / 32];
    if (lane_id() == 0) { so[threadIdx.x >> 5] = vo; sa[threadIdx.x >> 5] = va; }
    __syncthreads();
    if (threadIdx.x == 0) {
        for (int w = 1; w < (int)(blockDim.x >> 5); w++) { vo |= so[w]; va &= sa[w]; }
        atomicOr(&orand[0], vo);
        atomicAnd(&orand[1], va);
    }
}

// "\t%u\t%g\t%g" per read, zero padded to SFX_SLOT bytes
__global__ void k_sfx_slots(const NormVal *__restrict__ val, uint64_t n, uint8_t *__restrict__ slots) {
    const uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const NormVal v = val[i];
    char buf[SFX_SLOT];
    char *o = buf;
    *o++ = '\t';
    o = put_dec(o, v.med);
    *o++ = '\t';
    o = put_g6(o, v.gmean, v.xmean);
    *o++ = '\t';
    o = put_g6(o, v.gsd, v.xsd);
    while (o < buf + SFX_SLOT) *o++ = 0;
    for (int q = 0; q < SFX_SLOT; q++) slots[i * SFX_SLOT + q] = (uint8_t)buf[q];
}

// sorted-order name arrays; core = length without a final "/<digit>" (names
// are first header tokens, so they hold no whitespace)
__global__ void k_sorted_names(const uint64_t *__restrict__ name_addr, const uint32_t *__restrict__ name_len,
                               const uint32_t *__restrict__ perm, uint64_t n,
                               uint64_t *__restrict__ h0, uint64_t *__restrict__ h1, uint64_t *__restrict__ off,
                               uint32_t *__restrict__ len, uint32_t *__restrict__ core) {
    const uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const uint32_t r = perm[i];
    const uint64_t o = name_addr[r];
    const uint32_t l = name_len[r];
    const char *nm = at(o);
    h0[i] = name_chunk(nm, l, 0);
    h1[i] = name_chunk(nm, l, 1);
    off[i] = o;
    len[i] = l;
    uint32_t c = l;
    if (l >= 3 && nm[l - 2] == '/' && (uint32_t)((uint8_t)nm[l - 1] - '0') < 10u) c = l - 2;
    core[i] = c;
}

// set when a sorted neighbour has the same zero-padded name
__global__ void k_sort_ties(const uint64_t *__restrict__ h0,
                            const uint64_t *__restrict__ h1, const uint64_t *__restrict__ off,
                            const uint32_t *__restrict__ len, uint64_t n, uint32_t *__restrict__ flag) {
    const uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x + 1;
    if (i >= n) return;
    if (h0[i] != h0[i - 1] || h1[i] != h1[i - 1]) return;
    const uint32_t la = len[i - 1], lb = len[i], m = la > lb ? la : lb;
    for (uint32_t p = 16; p < m; p++) {
        const uint8_t x = p < la ? (uint8_t)at(off[i - 1])[p] : 0, y = p < lb ? (uint8_t)at(off[i])[p] : 0;
        if (x != y) return;
    }
    atomicExch(flag, 1u);
}

// ---------------------------------------------------------------- pair merge

struct SNames {
    const uint64_t *h0, *h1, *off;   // off: the name's device address
    const uint32_t *len, *core;
};

// bytewise comparison of two names, a shorter prefix first (Perl's lt/gt)
__device__ int sn_cmp(const SNames &A, uint64_t i, const SNames &B, uint64_t j) {
    const uint64_t a0 = A.h0[i], b0 = B.h0[j];
    if (a0 != b0) return a0 < b0 ? -1 : 1;
    const uint64_t a1 = A.h1[i], b1 = B.h1[j];
    if (a1 != b1) return a1 < b1 ? -1 : 1;
    const uint32_t la = A.len[i], lb = B.len[j], m = la < lb ? la : lb;
    if (m > 16) {
        const char *pa = at(A.off[i]), *pb = at(B.off[j]);
        for (uint32_t p = 16; p < m; p++) {
            const uint8_t x = (uint8_t)pa[p], y = (uint8_t)pb[p];
            if (x != y) return x < y ? -1 : 1;
        }
    }
    return la < lb ? -1 : (la > lb ? 1 : 0);
}

__device__ bool sn_core_eq(const SNames &A, uint64_t i, const SNames &B, uint64_t j) {
    const uint32_t c = A.core[i];
    if (c != B.core[j]) return false;
    if (c <= 8) {
        const uint64_t mask = c ? ~0ULL << (64 - 8 * c) : 0ULL;
        return ((A.h0[i] ^ B.h0[j]) & mask) == 0;
    }
    if (A.h0[i] != B.h0[j]) return false;
    if (c <= 16) {
        const uint64_t mask = ~0ULL << (64 - 8 * (c - 8));
        return ((A.h1[i] ^ B.h1[j]) & mask) == 0;
    }
    if (A.h1[i] != B.h1[j]) return false;
    const char *pa = at(A.off[i]), *pb = at(B.off[j]);
    for (uint32_t p = 16; p < c; p++)
        if (pa[p] != pb[p]) return false;
    return true;
}

// chunk k's start: (k*C, number of right names below left name k*C); chunk 0 at (0, 0)
__global__ void k_merge_starts(SNames L, uint64_t nL, SNames R, uint64_t nR, uint64_t nchunks,
                               uint64_t *__restrict__ jstart) {
    const uint64_t k = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= nchunks) return;
    if (k == 0) { jstart[0] = 0; return; }
    const uint64_t i = k * MG_CHUNK;
    uint64_t lo = 0, hi = nR;
    while (lo < hi) {
        const uint64_t mid = (lo + hi) >> 1;
        if (sn_cmp(R, mid, L, i) < 0) lo = mid + 1;
        else hi = mid;
    }
    jstart[k] = lo;
}

// One step of nbkc_merge_left_right_stats.pl's loop.  Returns true with a row.
__device__ __forceinline__ bool merge_step(const SNames &L, const SNames &R, uint64_t &i, uint64_t &j) {
    if (sn_core_eq(L, i, R, j)) { i++; j++; return true; }
    if (sn_cmp(L, i, R, j) < 0) i++;
    else j++;
    return false;
}

__global__ void k_merge_run(SNames L, uint64_t nL, SNames R, uint64_t nR, uint64_t nchunks,
                            const uint64_t *__restrict__ jstart, uint2 *__restrict__ slots,
                            uint32_t *__restrict__ cnt, uint8_t *__restrict__ status) {
    const uint64_t k = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= nchunks) return;
    const bool last = k + 1 == nchunks;
    const uint64_t ti = last ? nL : (k + 1) * MG_CHUNK, tj = last ? nR : jstart[k + 1];
    uint64_t i = k * MG_CHUNK, j = jstart[k];
    uint32_t c = 0;
    uint8_t st = MG_END;
    uint2 *out = slots + k * (MG_CHUNK + 1);
    while (i < nL && j < nR) {
        if (!last) {
            if (i == ti && j == tj) { st = MG_REACHED; break; }
            if (i > ti || j > tj) { st = MG_FAIL; break; }
        }
        const uint64_t i0 = i, j0 = j;
        if (merge_step(L, R, i, j)) {
            if (c <= MG_CHUNK) out[c] = make_uint2((uint32_t)i0, (uint32_t)j0);
            c++;
        }
    }
    if (c > MG_CHUNK + 1) st = MG_FAIL;
    cnt[k] = c;
    status[k] = st;
}

__global__ void k_merge_first(const uint8_t *__restrict__ status, uint64_t nchunks,
                              unsigned long long *__restrict__ first) {
    const uint64_t k = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (k < nchunks && status[k] != MG_REACHED) atomicMin(first, (unsigned long long)k);
}

// the sequential walk from (i, j) to the end, one thread
__global__ void k_merge_repair(SNames L, uint64_t nL, SNames R, uint64_t nR, uint64_t i, uint64_t j,
                               uint2 *__restrict__ out, unsigned long long *__restrict__ n_out) {
    if (blockIdx.x != 0 || threadIdx.x != 0) return;
    uint64_t c = 0;
    while (i < nL && j < nR) {
        const uint64_t i0 = i, j0 = j;
        if (merge_step(L, R, i, j)) out[c++] = make_uint2((uint32_t)i0, (uint32_t)j0);
    }
    *n_out = c;
}

__global__ void k_merge_compact(const uint2 *__restrict__ slots, const uint32_t *__restrict__ cnt,
                                const uint64_t *__restrict__ offs, uint64_t nvalid, uint32_t *__restrict__ row_l,
                                uint32_t *__restrict__ row_r) {
    const uint64_t t = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    const uint64_t k = t / (MG_CHUNK + 1), s = t % (MG_CHUNK + 1);
    if (k >= nvalid || s >= cnt[k]) return;
    const uint2 p = slots[k * (MG_CHUNK + 1) + s];
    row_l[offs[k] + s] = p.x;
    row_r[offs[k] + s] = p.y;
}

__global__ void k_merge_append(const uint2 *__restrict__ rep, uint64_t n, uint64_t base, uint32_t *__restrict__ row_l,
                               uint32_t *__restrict__ row_r) {
    const uint64_t t = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= n) return;
    row_l[base + t] = rep[t].x;
    row_r[base + t] = rep[t].y;
}

// ---------------------------------------------------------------- selection

struct RowArgs {
    const NormVal *vl, *vr;          // read order
    const uint32_t *perm_l, *perm_r;
    const uint32_t *row_l, *row_r;   // pairs: sorted positions per row
    uint64_t *row_n;                 // pairs: 3 per row
    uint64_t n_rows;
    bool pairs;
    int max_cov, min_cov, max_cv;
};

// median, mean and stdev nbkc_normalize.pl reads from row p
__device__ __forceinline__ void row_numbers(const RowArgs &a, uint64_t p, double *med, double *u, double *sd) {
    if (a.pairs) {
        const uint64_t *N = a.row_n + 3 * p;
        *med = __ddiv_rn((double)N[0], 10.0);
        *u = __ddiv_rn((double)N[1], 10.0);
        *sd = __ddiv_rn((double)N[2], 10.0);
    } else {
        const NormVal v = a.vl[a.perm_l[p]];
        *med = (double)v.med;
        *u = v.mean;
        *sd = v.sd;
    }
}

// the row's class: 0 draws, 1 below min_cov, 2 aberrant; pairs also get their averages
__global__ void k_norm_rows(RowArgs a, uint32_t *__restrict__ draws, double *__restrict__ ratio,
                            unsigned long long *__restrict__ tally, uint32_t *__restrict__ err) {
    const uint64_t p = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    uint32_t below = 0, aberrant = 0;
    if (p < a.n_rows) {
        if (a.pairs) {
            const NormVal l = a.vl[a.perm_l[a.row_l[p]]], r = a.vr[a.perm_r[a.row_r[p]]];
            uint64_t Nu = 0, Ns = 0;
            const bool ok = fix1(__dmul_rn(__dadd_rn(l.mean, r.mean), 0.5), &Nu) &&
                            fix1(__dmul_rn(__dadd_rn(l.sd, r.sd), 0.5), &Ns);
            if (!ok) flag_err(err, NE_DOMAIN);
            uint64_t *N = a.row_n + 3 * p;
            N[0] = 5 * ((uint64_t)l.med + r.med);
            N[1] = Nu;
            N[2] = Ns;
        }
        double med, u, sd;
        row_numbers(a, p, &med, &u, &sd);
        uint32_t d = 0;
        if (med < (double)a.min_cov) below = 1;
        else if (u <= 0.0 || __ddiv_rn(sd, u) > (double)a.max_cv) aberrant = 1;
        else {
            d = 1;
            if (med == 0.0) flag_err(err, NE_DIV0);
            else ratio[p] = __ddiv_rn((double)a.max_cov, med);
        }
        draws[p] = d;
    }
    below = __reduce_add_sync(0xffffffffu, below);
    aberrant = __reduce_add_sync(0xffffffffu, aberrant);
    if (lane_id() == 0) {
        if (below) atomicAdd(&tally[0], (unsigned long long)below);
        if (aberrant) atomicAdd(&tally[1], (unsigned long long)aberrant);
    }
}

// drand48 state after `steps` draws from X0
__device__ __forceinline__ uint64_t lcg_jump(uint64_t x0, uint64_t steps) {
    uint64_t A = 1, Cc = 0;
    for (int b = 0; b < 48 && steps; b++, steps >>= 1)
        if (steps & 1) {
            Cc = (c_lcg_a[b] * Cc + c_lcg_c[b]) & LCG_MASK;
            A = (c_lcg_a[b] * A) & LCG_MASK;
        }
    return (A * x0 + Cc) & LCG_MASK;
}

// the printed acc of row p: left name without "/<digit>" (pairs) then
// without a final "/1" or "/2"
__device__ __forceinline__ void row_acc(const RowArgs &a, const SNames &L, uint64_t p, uint64_t *off, uint32_t *len) {
    const uint64_t i = a.pairs ? a.row_l[p] : p;
    uint32_t n = a.pairs ? L.core[i] : L.len[i];
    const uint64_t o = L.off[i];
    if (n >= 2 && at(o)[n - 2] == '/' && (at(o)[n - 1] == '1' || at(o)[n - 1] == '2')) n -= 2;
    *off = o;
    *len = n;
}

__global__ void k_norm_pick(RowArgs a, SNames L, const uint32_t *__restrict__ draws, const double *__restrict__ ratio,
                            const uint64_t *__restrict__ rank, uint64_t x0, uint32_t *__restrict__ out_len,
                            unsigned long long *__restrict__ tally) {
    const uint64_t p = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    uint32_t keep = 0;
    if (p < a.n_rows) {
        uint32_t len = 0;
        if (draws[p]) {
            const uint64_t x = lcg_jump(x0, rank[p] + 1);
            const double r = __dmul_rn((double)x, 0x1p-48);   // X / 2^48, exact
            if (r <= ratio[p]) {
                uint64_t o;
                uint32_t n;
                row_acc(a, L, p, &o, &n);
                len = n + 1;
                keep = 1;
            }
        }
        out_len[p] = len;
    }
    keep = __reduce_add_sync(0xffffffffu, keep);
    if (lane_id() == 0 && keep) atomicAdd(&tally[2], (unsigned long long)keep);
}

__global__ void k_norm_accs(RowArgs a, SNames L, const uint64_t *__restrict__ acc_off, char *__restrict__ out) {
    const uint64_t p = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= a.n_rows || acc_off[p + 1] == acc_off[p]) return;
    uint64_t o;
    uint32_t n;
    row_acc(a, L, p, &o, &n);
    char *w = out + acc_off[p];
    for (uint32_t q = 0; q < n; q++) w[q] = at(o)[q];
    w[n] = '\n';
}

// ---------------------------------------------------------------- table text

__device__ char *put_stats_fields(char *o, const NormVal &v) {
    o = put_dec(o, v.med);
    *o++ = '\t';
    o = put_g6(o, v.gmean, v.xmean);
    *o++ = '\t';
    return put_g6(o, v.gsd, v.xsd);
}

__global__ void k_table_len(RowArgs a, SNames L, SNames R, uint32_t *__restrict__ out_len) {
    const uint64_t p = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= a.n_rows) return;
    if (!a.pairs) {
        out_len[p] = L.len[p] + a.vl[a.perm_l[p]].sfx_len + 1;
        return;
    }
    const uint64_t i = a.row_l[p], j = a.row_r[p];
    const NormVal l = a.vl[a.perm_l[i]], r = a.vr[a.perm_r[j]];
    const uint64_t *N = a.row_n + 3 * p;
    out_len[p] = L.core[i] + 1 + L.len[i] + l.sfx_len + 1 + R.len[j] + r.sfx_len + 3 + fix1_len(N[0]) +
                 fix1_len(N[1]) + fix1_len(N[2]) + 1;
}

__global__ void k_table_write(RowArgs a, SNames L, SNames R, const uint64_t *__restrict__ offs, char *__restrict__ out) {
    const uint64_t p = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= a.n_rows) return;
    char *o = out + offs[p];
    if (!a.pairs) {
        const uint64_t so = L.off[p];
        for (uint32_t q = 0; q < L.len[p]; q++) *o++ = at(so)[q];
        *o++ = '\t';
        o = put_stats_fields(o, a.vl[a.perm_l[p]]);
        *o = '\n';
        return;
    }
    const uint64_t i = a.row_l[p], j = a.row_r[p];
    const NormVal l = a.vl[a.perm_l[i]], r = a.vr[a.perm_r[j]];
    const uint64_t *N = a.row_n + 3 * p;
    const char *ln = at(L.off[i]), *rn = at(R.off[j]);
    for (uint32_t q = 0; q < L.core[i]; q++) *o++ = ln[q];
    *o++ = '\t';
    for (uint32_t q = 0; q < L.len[i]; q++) *o++ = ln[q];
    *o++ = '\t';
    o = put_stats_fields(o, l);
    *o++ = '\t';
    for (uint32_t q = 0; q < R.len[j]; q++) *o++ = rn[q];
    *o++ = '\t';
    o = put_stats_fields(o, r);
    for (int f = 0; f < 3; f++) {
        *o++ = '\t';
        o = put_fix1(o, N[f]);
    }
    *o = '\n';
}

// ---------------------------------------------------------------- extraction

__device__ __forceinline__ uint64_t fnv_step(uint64_t h, uint8_t c) { return (h ^ c) * 0x100000001b3ULL; }

// A name as up to three pieces of device text (the FASTQ core name after its
// "_forward" and "_reverse" were cut out).
struct Pieces {
    const char *p[3];
    uint32_t n[3];
    int k;
};

__device__ __forceinline__ uint32_t pieces_len(const Pieces &s) {
    uint32_t t = 0;
    for (int q = 0; q < s.k; q++) t += s.n[q];
    return t;
}

__device__ __forceinline__ char pieces_at(const Pieces &s, uint32_t i) {
    for (int q = 0; q < s.k; q++) {
        if (i < s.n[q]) return s.p[q][i];
        i -= s.n[q];
    }
    return 0;
}

// cuts the first occurrence of pat (8 bytes) out of s
__device__ void pieces_cut(Pieces &s, const char *pat) {
    const uint32_t n = pieces_len(s);
    for (uint32_t i = 0; i + 8 <= n; i++) {
        bool hit = true;
        for (uint32_t q = 0; q < 8 && hit; q++) hit = pieces_at(s, i + q) == pat[q];
        if (!hit) continue;
        // rebuild as [0, i) + [i + 8, n)
        Pieces t;
        t.k = 0;
        uint32_t pos = 0;
        for (int q = 0; q < s.k; q++) {
            const uint32_t a = pos, b = pos + s.n[q];   // piece covers [a, b)
            if (a < i) {
                const uint32_t e = b < i ? b : i;
                t.p[t.k] = s.p[q];
                t.n[t.k++] = e - a;
            }
            if (b > i + 8) {
                const uint32_t st = a > i + 8 ? a : i + 8;
                t.p[t.k] = s.p[q] + (st - a);
                t.n[t.k++] = b - st;
            }
            pos = b;
        }
        s = t;
        return;
    }
}

__device__ __forceinline__ uint64_t pieces_hash(const Pieces &s) {
    uint64_t h = 0xcbf29ce484222325ULL;
    for (int q = 0; q < s.k; q++)
        for (uint32_t i = 0; i < s.n[q]; i++) h = fnv_step(h, (uint8_t)s.p[q][i]);
    return mix64(h);
}

__device__ __forceinline__ bool pieces_eq(const Pieces &s, const char *b, uint32_t bn) {
    if (pieces_len(s) != bn) return false;
    uint32_t x = 0;
    for (int q = 0; q < s.k; q++)
        for (uint32_t i = 0; i < s.n[q]; i++)
            if (s.p[q][i] != b[x++]) return false;
    return true;
}

// the selection's names as the extraction looks them up: each accs line
// without a final "/" and word character (build_selected_index)
__device__ __forceinline__ uint32_t key_len(const char *t, uint64_t o, uint32_t n) {
    if (n >= 2 && t[o + n - 2] == '/') {
        const uint8_t c = (uint8_t)t[o + n - 1];
        if ((c - '0' < 10u) || ((c | 0x20) - 'a' < 26u) || c == '_') n -= 2;
    }
    return n;
}

__global__ void k_hash_insert(const char *__restrict__ accs, const uint64_t *__restrict__ acc_off, uint64_t n_rows,
                              uint32_t *__restrict__ slots, uint64_t mask, uint8_t *__restrict__ dup,
                              uint32_t *__restrict__ err) {
    const uint64_t p = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= n_rows) return;
    const uint64_t o = acc_off[p];
    if (acc_off[p + 1] == o) return;
    if (acc_off[p + 1] - o == 1) {   // an empty line names nothing (names hold no whitespace)
        dup[p] = 1;
        return;
    }
    const uint32_t n = key_len(accs, o, (uint32_t)(acc_off[p + 1] - o - 1));
    Pieces s;
    s.k = 1;
    s.p[0] = accs + o;
    s.n[0] = n;
    uint64_t h = pieces_hash(s) & mask;
    for (uint64_t probe = 0; probe <= mask; probe++) {
        const uint32_t cur = atomicCAS(&slots[h], ~0u, (uint32_t)p);
        if (cur == ~0u) return;
        const uint64_t co = acc_off[cur];
        const uint32_t cn = key_len(accs, co, (uint32_t)(acc_off[cur + 1] - co - 1));
        if (pieces_eq(s, accs + co, cn)) {
            dup[p] = 1;
            return;
        }
        h = (h + 1) & mask;
    }
    flag_err(err, NE_HASH);
}

// per FASTQ record: its core name looked up in the selection
__global__ void k_extract_find(const char *__restrict__ text, uint64_t text_len, const uint64_t *__restrict__ name_off,
                               const uint32_t *__restrict__ name_len, uint64_t n, const char *__restrict__ accs,
                               const uint64_t *__restrict__ acc_off, const uint32_t *__restrict__ slots, uint64_t mask,
                               uint8_t *__restrict__ found, uint32_t *__restrict__ rec_len) {
    const uint64_t r = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (r >= n) return;
    const uint64_t o = name_off[r];
    uint32_t l = name_len[r];
    if (l >= 3 && text[o + l - 2] == '/' && (text[o + l - 1] == '1' || text[o + l - 1] == '2')) l -= 2;
    Pieces s;
    s.k = 1;
    s.p[0] = text + o;
    s.n[0] = l;
    pieces_cut(s, "_forward");
    pieces_cut(s, "_reverse");
    uint64_t h = pieces_hash(s) & mask;
    bool hit = false;
    for (uint64_t probe = 0; probe <= mask; probe++) {
        const uint32_t cur = slots[h];
        if (cur == ~0u) break;
        const uint64_t co = acc_off[cur];
        const uint32_t cn = key_len(accs, co, (uint32_t)(acc_off[cur + 1] - co - 1));
        if (pieces_eq(s, accs + co, cn)) {
            found[cur] = 1;
            hit = true;
            break;
        }
        h = (h + 1) & mask;
    }
    uint32_t len = 0;
    if (hit) {
        // the record runs from its '@' through its fourth line's "\n"
        const uint64_t a = o - 1;
        uint64_t e;
        if (r + 1 < n) e = name_off[r + 1] - 1;
        else {
            e = a;
            int nl = 0;
            while (e < text_len && nl < 4)
                if (text[e++] == '\n') nl++;
        }
        len = (uint32_t)(e - a);
    }
    rec_len[r] = len;
}

// ---- FASTA records (Fasta_reader.pm:45-70, Sequence::get_FASTA_format with
// fasta_line_len => -1): control bytes other than tab and newline, and bytes
// 0x7F-0xFF, are deleted; header = the first line; sequence = the other lines
// joined without whitespace; accession = the header's first field; the record
// is written ">header\nsequence\n".  The extraction key is the accession
// without a final "/1" or "/2" (insilico:526-527).

constexpr int FA_ACC_MAX = 256;   // accession bytes kept for the lookup

__device__ __forceinline__ bool fa_hdr_keep(uint8_t c) { return c == '\t' || (c >= 32 && c < 127); }
__device__ __forceinline__ bool fa_seq_keep(uint8_t c) { return c > 32 && c < 127; }

// [a, e): record r ('>' at a); hl = end of its header line
__device__ __forceinline__ void fa_extent(const char *__restrict__ text, uint64_t text_len,
                                          const uint64_t *__restrict__ name_off, uint64_t n, uint64_t r, uint64_t *a,
                                          uint64_t *hl, uint64_t *e) {
    *a = name_off[r] - 1;
    *e = r + 1 < n ? name_off[r + 1] - 1 : text_len;
    uint64_t p = *a + 1;
    while (p < *e && text[p] != '\n') p++;
    *hl = p;
}

__global__ void k_extract_find_fa(const char *__restrict__ text, uint64_t text_len,
                                  const uint64_t *__restrict__ name_off, uint64_t n, const char *__restrict__ accs,
                                  const uint64_t *__restrict__ acc_off, const uint32_t *__restrict__ slots,
                                  uint64_t mask, uint8_t *__restrict__ found, uint32_t *__restrict__ rec_len,
                                  uint32_t *__restrict__ err) {
    const uint64_t r = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (r >= n) return;
    uint64_t a, hl, e;
    fa_extent(text, text_len, name_off, n, r, &a, &hl, &e);
    char acc[FA_ACC_MAX];
    uint32_t al = 0, hk = 0;
    bool in_acc = true;
    for (uint64_t p = a + 1; p < hl; p++) {
        const uint8_t c = (uint8_t)text[p];
        if (!fa_hdr_keep(c)) continue;
        hk++;
        if (c == ' ' || c == '\t') in_acc = false;
        if (in_acc) {
            if (al == FA_ACC_MAX) {
                flag_err(err, NE_DOMAIN);
                in_acc = false;
            } else {
                acc[al++] = (char)c;
            }
        }
    }
    if (al >= 2 && acc[al - 2] == '/' && (acc[al - 1] == '1' || acc[al - 1] == '2')) al -= 2;
    Pieces s;
    s.k = 1;
    s.p[0] = acc;
    s.n[0] = al;
    uint64_t h = pieces_hash(s) & mask;
    bool hit = false;
    for (uint64_t probe = 0; probe <= mask; probe++) {
        const uint32_t cur = slots[h];
        if (cur == ~0u) break;
        const uint64_t co = acc_off[cur];
        const uint32_t cn = key_len(accs, co, (uint32_t)(acc_off[cur + 1] - co - 1));
        if (pieces_eq(s, accs + co, cn)) {
            found[cur] = 1;
            hit = true;
            break;
        }
        h = (h + 1) & mask;
    }
    uint32_t len = 0;
    if (hit) {
        uint64_t sk = 0;
        for (uint64_t p = hl; p < e; p++) sk += fa_seq_keep((uint8_t)text[p]);
        len = (uint32_t)(1 + hk + 1 + sk + 1);
    }
    rec_len[r] = len;
}

__global__ void k_extract_write_fa(const char *__restrict__ text, uint64_t text_len,
                                   const uint64_t *__restrict__ name_off, uint64_t n,
                                   const uint64_t *__restrict__ out_off, uint64_t out_base, char *__restrict__ out) {
    const uint64_t r = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (r >= n || out_off[r + 1] == out_off[r]) return;
    uint64_t a, hl, e;
    fa_extent(text, text_len, name_off, n, r, &a, &hl, &e);
    char *o = out + out_base + out_off[r];
    *o++ = '>';
    for (uint64_t p = a + 1; p < hl; p++)
        if (fa_hdr_keep((uint8_t)text[p])) *o++ = text[p];
    *o++ = '\n';
    for (uint64_t p = hl; p < e; p++)
        if (fa_seq_keep((uint8_t)text[p])) *o++ = text[p];
    *o = '\n';
}

__global__ void k_extract_missing(const uint64_t *__restrict__ acc_off, uint64_t n_rows, const uint8_t *__restrict__ dup,
                                  const uint8_t *__restrict__ found, unsigned long long *__restrict__ missing) {
    const uint64_t p = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    uint32_t m = 0;
    if (p < n_rows && acc_off[p + 1] != acc_off[p] && !dup[p] && !found[p]) m = 1;
    m = __reduce_add_sync(0xffffffffu, m);
    if (lane_id() == 0 && m) atomicAdd(missing, (unsigned long long)m);
}

// A block per EX_RECS consecutive records: the block's output is one
// contiguous byte range, written in aligned 16-byte chunks by consecutive
// threads (coalesced); the record holding a chunk is found by a binary search
// over the block's record offsets in shared memory.  A chunk inside one
// record takes five aligned 4-byte source loads and four funnel shifts and
// leaves as one 16-byte store; a chunk across a record boundary, or shared
// with a neighbouring block, is written byte by byte (only the block's own
// bytes).
constexpr int EX_RECS = 256;

__global__ void __launch_bounds__(NM_THREADS) k_extract_copy(const char *__restrict__ text, uint64_t text_len, bool vec,
                                                             const uint64_t *__restrict__ name_off, uint64_t n,
                                                             const uint64_t *__restrict__ out_off, uint64_t out_base,
                                                             char *__restrict__ out) {
    __shared__ uint64_t s_off[EX_RECS + 1], s_src[EX_RECS];
    const uint64_t r0 = (uint64_t)blockIdx.x * EX_RECS;
    if (r0 >= n) return;
    const uint32_t m = (uint32_t)(n - r0 < EX_RECS ? n - r0 : EX_RECS);
    for (uint32_t i = threadIdx.x; i <= m; i += blockDim.x) {
        s_off[i] = out_base + out_off[r0 + i];            // out_off has n + 1 entries
        if (i < m) s_src[i] = name_off[r0 + i] - 1;       // the record's '@'
    }
    __syncthreads();
    const uint64_t O0 = s_off[0], O1 = s_off[m];
    if (O1 == O0) return;
    const uint64_t c0 = O0 >> 4, c1 = (O1 + 15) >> 4;
    for (uint64_t cidx = c0 + threadIdx.x; cidx < c1; cidx += blockDim.x) {
        const uint64_t b = 16 * cidx;   // the chunk's first output byte
        // the last record whose output starts at or before max(b, O0)
        const uint64_t key = b < O0 ? O0 : b;
        uint32_t lo = 0, hi = m;        // s_off[lo] <= key < s_off[hi]
        while (hi - lo > 1) {
            const uint32_t mid = (lo + hi) >> 1;
            if (s_off[mid] <= key) lo = mid;
            else hi = mid;
        }
        char *d = out + b;
        const uint64_t a = s_src[lo] + (b - s_off[lo]);   // source of byte b when b lies in record lo
        if (b >= O0 && b + 16 <= s_off[lo + 1] && vec && (a & ~3ULL) + 20 <= text_len) {
            const uint32_t *p = reinterpret_cast<const uint32_t *>(text + (a & ~3ULL));
            const uint32_t sh = 8u * (uint32_t)(a & 3);
            const uint32_t x0 = __ldg(p), x1 = __ldg(p + 1), x2 = __ldg(p + 2), x3 = __ldg(p + 3), x4 = __ldg(p + 4);
            uint4 v;
            v.x = __funnelshift_r(x0, x1, sh);
            v.y = __funnelshift_r(x1, x2, sh);
            v.z = __funnelshift_r(x2, x3, sh);
            v.w = __funnelshift_r(x3, x4, sh);
            *reinterpret_cast<uint4 *>(d) = v;
        } else {
            uint32_t r = lo;
            for (int i = 0; i < 16; i++) {
                const uint64_t q = b + i;
                if (q < O0 || q >= O1) continue;
                while (q >= s_off[r + 1]) r++;
                d[i] = text[s_src[r] + (q - s_off[r])];
            }
        }
    }
}

// ---------------------------------------------------------------- host side

static inline unsigned nm_grid(uint64_t n, int threads = NM_THREADS) {
    return (unsigned)std::max<uint64_t>(1, (n + threads - 1) / threads);
}

static void lcg_tables(uint64_t a[48], uint64_t c[48]) {
    a[0] = 0x5DEECE66DULL;
    c[0] = 0xB;
    for (int i = 1; i < 48; i++) {
        a[i] = (a[i - 1] * a[i - 1]) & LCG_MASK;
        c[i] = (a[i - 1] * c[i - 1] + c[i - 1]) & LCG_MASK;
    }
}

static void side_free(tk_ctx *c, NormSide &s) {
    void *p[] = {s.addr, s.nlen, s.val, s.perm, s.h0, s.h1, s.off, s.len, s.core};
    for (void *q : p)
        if (q) dfree(c, q);
    s = NormSide();
}

struct Scratch {
    tk_ctx *c;
    std::vector<void *> held;
    explicit Scratch(tk_ctx *cc) : c(cc) {}
    int get(void **p, size_t bytes, const char *what) {
        int e = dmalloc(c, p, bytes ? bytes : 16, what);
        if (!e) held.push_back(*p);
        return e;
    }
    ~Scratch() {
        for (void *p : held) dfree(c, p);
    }
};

static int read_err(tk_ctx *c, uint32_t *d_err, uint32_t h[NE_WORDS]) {
    TK_CUDA(c, cudaMemcpyAsync(h, d_err, NE_WORDS * 4, cudaMemcpyDeviceToHost, c->stream));
    TK_CUDA(c, cudaStreamSynchronize(c->stream));
    return TK_OK;
}

// One side's names into sorted order: the LSD radix passes of the name (and,
// when padded names tie, the full key).
static int sort_side(tk_ctx *c, NormSide &s) {
    const uint64_t n = s.n;
    TK_TRY(dmalloc(c, (void **)&s.perm, n * 4, "norm order"));
    TK_TRY(dmalloc(c, (void **)&s.h0, n * 8, "norm names"));
    TK_TRY(dmalloc(c, (void **)&s.h1, n * 8, "norm names"));
    TK_TRY(dmalloc(c, (void **)&s.off, n * 8, "norm names"));
    TK_TRY(dmalloc(c, (void **)&s.len, n * 4, "norm names"));
    TK_TRY(dmalloc(c, (void **)&s.core, n * 4, "norm names"));
    Scratch sc(c);
    uint64_t *keys = nullptr, *tkeys = nullptr;
    uint32_t *tperm = nullptr, *d_u32 = nullptr;
    unsigned long long *orand = nullptr;
    uint8_t *slots = nullptr;
    TK_TRY(sc.get((void **)&keys, n * 8, "sort keys"));
    TK_TRY(sc.get((void **)&tkeys, n * 8, "sort keys"));
    TK_TRY(sc.get((void **)&tperm, n * 4, "sort order"));
    TK_TRY(sc.get((void **)&d_u32, 16, "sort scalars"));
    TK_TRY(sc.get((void **)&orand, 16, "sort key bits"));
    TK_CUDA(c, cudaMemsetAsync(d_u32, 0, 16, c->stream));
    k_name_maxlen<<<(unsigned)std::min<uint64_t>(nm_grid(n), (uint64_t)c->sm_count * 8), NM_THREADS, 0, c->stream>>>(
        s.nlen, n, d_u32);
    c->launches++;
    uint32_t maxlen = 0;
    TK_CUDA(c, cudaMemcpyAsync(&maxlen, d_u32, 4, cudaMemcpyDeviceToHost, c->stream));
    TK_CUDA(c, cudaStreamSynchronize(c->stream));
    const uint32_t nch = std::max<uint32_t>(1, (maxlen + 7) / 8);
    uint32_t *perm = s.perm;
    auto pass = [&](int mode, uint32_t ch) -> int {
        TK_CUDA(c, cudaMemsetAsync(orand, 0, 8, c->stream));
        TK_CUDA(c, cudaMemsetAsync(orand + 1, 0xFF, 8, c->stream));
        k_sort_keys<<<nm_grid(n), NM_THREADS, 0, c->stream>>>(s.addr, s.nlen, slots, perm, n, mode, ch, keys, orand);
        c->launches++;
        TK_TRY(check_launch(c, "sort keys"));
        unsigned long long h[2];
        TK_CUDA(c, cudaMemcpyAsync(h, orand, 16, cudaMemcpyDeviceToHost, c->stream));
        TK_CUDA(c, cudaStreamSynchronize(c->stream));
        const uint64_t diff = h[0] ^ h[1];
        if (!diff) return TK_OK;   // every key alike: the order stands
        const int lo = __builtin_ctzll(diff), hi = 63 - __builtin_clzll(diff);
        bool in_tmp = false;
        TK_TRY(radix_sort_pairs(c, keys, perm, n, hi - lo + 1, tkeys, tperm, &in_tmp, lo));
        if (in_tmp) {
            std::swap(keys, tkeys);
            std::swap(perm, tperm);
        }
        return TK_OK;
    };
    auto iota = [&]() {
        k_iota<<<nm_grid(n), NM_THREADS, 0, c->stream>>>(perm, n);
        c->launches++;
    };
    iota();
    for (int ch = (int)nch - 1; ch >= 0; ch--) TK_TRY(pass(0, (uint32_t)ch));
    auto gather = [&]() -> int {
        k_sorted_names<<<nm_grid(n), NM_THREADS, 0, c->stream>>>(s.addr, s.nlen, perm, n, s.h0, s.h1, s.off, s.len,
                                                                  s.core);
        c->launches++;
        return check_launch(c, "sorted names");
    };
    TK_TRY(gather());
    TK_CUDA(c, cudaMemsetAsync(d_u32, 0, 4, c->stream));
    if (n > 1) {
        k_sort_ties<<<nm_grid(n - 1), NM_THREADS, 0, c->stream>>>(s.h0, s.h1, s.off, s.len, n, d_u32);
        c->launches++;
    }
    uint32_t ties = 0;
    TK_CUDA(c, cudaMemcpyAsync(&ties, d_u32, 4, cudaMemcpyDeviceToHost, c->stream));
    TK_CUDA(c, cudaStreamSynchronize(c->stream));
    if (ties) {
        // equal (padded) names: order by name, then by the rest of the line
        TK_TRY(sc.get((void **)&slots, n * SFX_SLOT, "sort line suffixes"));
        k_sfx_slots<<<nm_grid(n), NM_THREADS, 0, c->stream>>>(s.val, n, slots);
        c->launches++;
        iota();
        for (int ch = SFX_SLOT / 8 - 1; ch >= 0; ch--) TK_TRY(pass(1, (uint32_t)ch));
        TK_TRY(pass(2, 0));
        for (int ch = (int)nch - 1; ch >= 0; ch--) TK_TRY(pass(0, (uint32_t)ch));
        TK_TRY(gather());
    }
    if (perm != s.perm) {
        TK_CUDA(c, cudaMemcpyAsync(s.perm, perm, n * 4, cudaMemcpyDeviceToDevice, c->stream));
    }
    return TK_OK;
}

static SNames snames(const NormSide &s) {
    SNames v;
    v.h0 = s.h0;
    v.h1 = s.h1;
    v.off = s.off;
    v.len = s.len;
    v.core = s.core;
    return v;
}

// the merged rows of nbkc_merge_left_right_stats.pl --sorted
static int merge_sides(tk_norm *nm) {
    tk_ctx *c = nm->ctx;
    const NormSide &A = nm->side[0], &B = nm->side[1];
    const uint64_t nL = A.n, nR = B.n;
    nm->n_rows = 0;
    if (!nL || !nR) return TK_OK;
    const SNames L = snames(A), R = snames(B);
    const uint64_t nchunks = (nL + MG_CHUNK - 1) / MG_CHUNK;
    Scratch sc(c);
    uint64_t *jstart = nullptr, *offs = nullptr;
    uint2 *slots = nullptr, *rep = nullptr;
    uint32_t *cnt = nullptr;
    uint8_t *status = nullptr;
    unsigned long long *d_first = nullptr;
    TK_TRY(sc.get((void **)&jstart, (nchunks + 1) * 8, "merge starts"));
    TK_TRY(sc.get((void **)&slots, nchunks * (MG_CHUNK + 1) * sizeof(uint2), "merge rows"));
    TK_TRY(sc.get((void **)&cnt, nchunks * 4, "merge counts"));
    TK_TRY(sc.get((void **)&status, nchunks, "merge status"));
    TK_TRY(sc.get((void **)&d_first, 16, "merge first"));
    k_merge_starts<<<nm_grid(nchunks), NM_THREADS, 0, c->stream>>>(L, nL, R, nR, nchunks, jstart);
    c->launches++;
    k_merge_run<<<nm_grid(nchunks, 128), 128, 0, c->stream>>>(L, nL, R, nR, nchunks, jstart, slots, cnt, status);
    c->launches++;
    TK_TRY(check_launch(c, "merge"));
    const unsigned long long none = nchunks;
    TK_CUDA(c, cudaMemcpyAsync(d_first, &none, 8, cudaMemcpyHostToDevice, c->stream));
    k_merge_first<<<nm_grid(nchunks), NM_THREADS, 0, c->stream>>>(status, nchunks, d_first);
    c->launches++;
    unsigned long long first = 0;
    uint8_t st = 0;
    TK_CUDA(c, cudaMemcpyAsync(&first, d_first, 8, cudaMemcpyDeviceToHost, c->stream));
    TK_CUDA(c, cudaStreamSynchronize(c->stream));
    if (first >= nchunks) return set_err(c, TK_E_INVAL, "pair merge: no chunk ends the walk");   // the last one always does
    TK_CUDA(c, cudaMemcpyAsync(&st, status + first, 1, cudaMemcpyDeviceToHost, c->stream));
    uint64_t j_first = 0;
    TK_CUDA(c, cudaMemcpyAsync(&j_first, jstart + first, 8, cudaMemcpyDeviceToHost, c->stream));
    TK_CUDA(c, cudaStreamSynchronize(c->stream));
    const uint64_t nvalid = st == MG_END ? first + 1 : first;
    uint64_t n_main = 0;
    TK_TRY(sc.get((void **)&offs, (nvalid + 1) * 8, "merge offsets"));
    if (nvalid) TK_TRY(scan_excl_u32_to_u64(c, cnt, offs, nvalid, &n_main));
    unsigned long long n_rep = 0;
    if (st == MG_FAIL) {
        const uint64_t i0 = first * MG_CHUNK;
        const uint64_t cap = std::min(nL - i0, nR - std::min(nR, j_first)) + 1;
        unsigned long long *d_nrep = d_first + 1;
        TK_TRY(sc.get((void **)&rep, cap * sizeof(uint2), "merge repair rows"));
        k_merge_repair<<<1, 32, 0, c->stream>>>(L, nL, R, nR, i0, j_first, rep, d_nrep);
        c->launches++;
        TK_TRY(check_launch(c, "merge repair"));
        TK_CUDA(c, cudaMemcpyAsync(&n_rep, d_nrep, 8, cudaMemcpyDeviceToHost, c->stream));
        TK_CUDA(c, cudaStreamSynchronize(c->stream));
    }
    nm->n_rows = n_main + n_rep;
    TK_TRY(dmalloc(c, (void **)&nm->row_l, nm->n_rows * 4 + 4, "merged rows"));
    TK_TRY(dmalloc(c, (void **)&nm->row_r, nm->n_rows * 4 + 4, "merged rows"));
    if (nvalid) {
        k_merge_compact<<<nm_grid(nvalid * (MG_CHUNK + 1)), NM_THREADS, 0, c->stream>>>(slots, cnt, offs, nvalid,
                                                                                        nm->row_l, nm->row_r);
        c->launches++;
    }
    if (n_rep) {
        k_merge_append<<<nm_grid(n_rep), NM_THREADS, 0, c->stream>>>(rep, n_rep, n_main, nm->row_l, nm->row_r);
        c->launches++;
    }
    TK_TRY(check_launch(c, "merge rows"));
    return cuda_check(c, cudaStreamSynchronize(c->stream), "merge sync");
}

static RowArgs row_args(const tk_norm *nm) {
    RowArgs a;
    a.vl = nm->side[0].val;
    a.vr = nm->side[1].val;
    a.perm_l = nm->side[0].perm;
    a.perm_r = nm->side[1].perm;
    a.row_l = nm->row_l;
    a.row_r = nm->row_r;
    a.row_n = nm->row_n;
    a.n_rows = nm->n_rows;
    a.pairs = nm->pairs;
    a.max_cov = nm->max_cov;
    a.min_cov = nm->min_cov;
    a.max_cv = nm->max_cv;
    return a;
}

int norm_select(tk_norm *nm, const tk_reads *const *const sets[2], const uint32_t nsets[2],
                const uint32_t *const med[2], const float *const mean[2], const float *const sd[2], int where) {
    tk_ctx *c = nm->ctx;
    cudaEvent_t ev = nullptr;
    prof_begin(c, TK_KID_NORM, &ev);
    {
        uint64_t a[48], cc[48];
        lcg_tables(a, cc);
        TK_CUDA(c, cudaMemcpyToSymbolAsync(c_lcg_a, a, sizeof a, 0, cudaMemcpyHostToDevice, c->stream));
        TK_CUDA(c, cudaMemcpyToSymbolAsync(c_lcg_c, cc, sizeof cc, 0, cudaMemcpyHostToDevice, c->stream));
    }
    Scratch sc(c);
    uint32_t *d_err = nullptr;
    TK_TRY(sc.get((void **)&d_err, NE_WORDS * 4, "norm errors"));
    TK_CUDA(c, cudaMemsetAsync(d_err, 0, NE_WORDS * 4, c->stream));
    const int sides = nm->pairs ? 2 : 1;
    uint64_t units = 0;
    for (int sd_i = 0; sd_i < sides; sd_i++) {
        NormSide &s = nm->side[sd_i];
        s.n = 0;
        for (uint32_t q = 0; q < nsets[sd_i]; q++) s.n += sets[sd_i][q]->n_reads;
        units += s.n;
        TK_TRY(dmalloc(c, (void **)&s.val, (s.n ? s.n : 1) * sizeof(NormVal), "norm values"));
        if (!s.n) continue;
        TK_TRY(dmalloc(c, (void **)&s.addr, s.n * 8, "norm name addresses"));
        TK_TRY(dmalloc(c, (void **)&s.nlen, s.n * 4, "norm name lengths"));
        uint64_t first = 0;
        for (uint32_t q = 0; q < nsets[sd_i]; q++) {
            const tk_reads *r = sets[sd_i][q];
            if (r->n_reads) {
                k_name_addr<<<nm_grid(r->n_reads), NM_THREADS, 0, c->stream>>>(r->d_text, r->d_name_off, r->d_name_len,
                                                                               r->n_reads, s.addr + first, s.nlen + first);
                c->launches++;
            }
            first += r->n_reads;
        }
        const uint32_t *dm = med[sd_i];
        const float *dmean = mean[sd_i], *dsd = sd[sd_i];
        if (where == TK_HOST) {
            uint32_t *a = nullptr;
            float *b = nullptr, *d = nullptr;
            TK_TRY(sc.get((void **)&a, s.n * 4, "norm medians"));
            TK_TRY(sc.get((void **)&b, s.n * 4, "norm means"));
            TK_TRY(sc.get((void **)&d, s.n * 4, "norm stdevs"));
            TK_CUDA(c, cudaMemcpyAsync(a, dm, s.n * 4, cudaMemcpyHostToDevice, c->stream));
            TK_CUDA(c, cudaMemcpyAsync(b, dmean, s.n * 4, cudaMemcpyHostToDevice, c->stream));
            TK_CUDA(c, cudaMemcpyAsync(d, dsd, s.n * 4, cudaMemcpyHostToDevice, c->stream));
            dm = a;
            dmean = b;
            dsd = d;
        }
        k_norm_vals<<<nm_grid(s.n), NM_THREADS, 0, c->stream>>>(s.n, dm, dmean, dsd, s.val, d_err);
        c->launches++;
        TK_TRY(check_launch(c, "norm values"));
        TK_TRY(sort_side(c, s));
    }
    uint32_t herr[NE_WORDS];
    TK_TRY(read_err(c, d_err, herr));
    if (herr[NE_DOMAIN])
        return set_err(c, TK_E_INVAL, "normalization: a mean or stdev outside [1e-17, 1.8e19) (or not a number)");
    if (nm->pairs) TK_TRY(merge_sides(nm));
    else nm->n_rows = nm->side[0].n;
    const uint64_t P = nm->n_rows;
    if (nm->pairs) TK_TRY(dmalloc(c, (void **)&nm->row_n, (P ? P : 1) * 24, "merged averages"));
    TK_TRY(dmalloc(c, (void **)&nm->acc_off, (P + 1) * 8, "accs offsets"));
    uint32_t *draws = nullptr, *lens = nullptr;
    uint64_t *rank = nullptr;
    double *ratio = nullptr;
    unsigned long long *tally = nullptr;
    TK_TRY(sc.get((void **)&draws, P * 4, "norm draws"));
    TK_TRY(sc.get((void **)&ratio, P * 8, "norm ratios"));
    TK_TRY(sc.get((void **)&lens, P * 4, "accs lengths"));
    TK_TRY(sc.get((void **)&rank, (P + 1) * 8, "norm draw ranks"));
    TK_TRY(sc.get((void **)&tally, 32, "norm tallies"));
    TK_CUDA(c, cudaMemsetAsync(tally, 0, 32, c->stream));
    const RowArgs a = row_args(nm);
    const SNames L = snames(nm->side[0]);
    uint64_t n_draws = 0;
    if (P) {
        k_norm_rows<<<nm_grid(P), NM_THREADS, 0, c->stream>>>(a, draws, ratio, tally, d_err);
        c->launches++;
        TK_TRY(check_launch(c, "norm rows"));
        TK_TRY(scan_excl_u32_to_u64(c, draws, rank, P, &n_draws));
        TK_TRY(read_err(c, d_err, herr));
        if (herr[NE_DOMAIN]) return set_err(c, TK_E_INVAL, "normalization: an average outside [0, 1e15)");
        if (herr[NE_DIV0]) return set_err(c, TK_E_INVAL, "normalization: a selected row has median 0 (min_cov <= 0)");
        const uint64_t x0 = (12345ULL << 16) | 0x330EULL;
        k_norm_pick<<<nm_grid(P), NM_THREADS, 0, c->stream>>>(a, L, draws, ratio, rank, x0, lens, tally);
        c->launches++;
        TK_TRY(check_launch(c, "norm pick"));
        TK_TRY(scan_excl_u32_to_u64(c, lens, nm->acc_off, P, &nm->accs_len));
    } else {
        TK_CUDA(c, cudaMemsetAsync(nm->acc_off, 0, 8, c->stream));
        nm->accs_len = 0;
    }
    TK_CUDA(c, cudaMemcpyAsync(nm->acc_off + P, &nm->accs_len, 8, cudaMemcpyHostToDevice, c->stream));
    TK_TRY(dmalloc(c, (void **)&nm->d_accs, nm->accs_len ? nm->accs_len : 1, "accs text"));
    if (P && nm->accs_len) {
        k_norm_accs<<<nm_grid(P), NM_THREADS, 0, c->stream>>>(a, L, nm->acc_off, nm->d_accs);
        c->launches++;
        TK_TRY(check_launch(c, "accs text"));
    }
    unsigned long long t[3];
    TK_CUDA(c, cudaMemcpyAsync(t, tally, 24, cudaMemcpyDeviceToHost, c->stream));
    TK_CUDA(c, cudaStreamSynchronize(c->stream));
    nm->counts.rows = P;
    nm->counts.below_min = t[0];
    nm->counts.aberrant = t[1];
    nm->counts.selected = t[2];
    prof_end(c, TK_KID_NORM, ev, units);
    return TK_OK;
}

int norm_table(tk_norm *nm) {
    if (nm->d_table) return TK_OK;
    tk_ctx *c = nm->ctx;
    const uint64_t P = nm->n_rows;
    const char *hdr = nm->pairs ? "acc\tleft_acc\tleft_median_cov\tleft_mean_cov\tleft_stdev\tright_acc\t"
                                  "right_median_cov\tright_mean_cov\tright_stdev\tmedian_cov\tmean_cov\tstdev\n"
                                : "acc\tmedian_cov\tmean_cov\tstdev\n";
    const uint64_t hl = std::strlen(hdr);
    Scratch sc(c);
    uint32_t *lens = nullptr;
    uint64_t *offs = nullptr, body = 0;
    TK_TRY(sc.get((void **)&lens, P * 4, "table lengths"));
    TK_TRY(sc.get((void **)&offs, (P + 1) * 8, "table offsets"));
    const RowArgs a = row_args(nm);
    const SNames L = snames(nm->side[0]), R = snames(nm->side[1]);
    if (P) {
        k_table_len<<<nm_grid(P), NM_THREADS, 0, c->stream>>>(a, L, R, lens);
        c->launches++;
        TK_TRY(check_launch(c, "table lengths"));
        TK_TRY(scan_excl_u32_to_u64(c, lens, offs, P, &body));
    }
    char *d = nullptr;
    TK_TRY(dmalloc(c, (void **)&d, hl + body, "table text"));
    int e = cuda_check(c, cudaMemcpyAsync(d, hdr, hl, cudaMemcpyHostToDevice, c->stream), "table header");
    if (!e && P) {
        k_table_write<<<nm_grid(P), NM_THREADS, 0, c->stream>>>(a, L, R, offs, d + hl);
        c->launches++;
        e = check_launch(c, "table text");
    }
    if (!e) e = cuda_check(c, cudaStreamSynchronize(c->stream), "table sync");
    if (e) {
        dfree(c, d);
        return e;
    }
    nm->d_table = d;
    nm->table_len = hl + body;
    return TK_OK;
}

// The records of sets[0..nsets) (one side's files or pieces, in order) that
// the selection holds; every selected name must be found in one of them.
// Earlier extractions' device texts whose host copies have ended go back to
// the allocator; with `all`, every one, the context's stream first waiting
// for the copies still running (so a later user of a block is ordered after
// them).
static void ext_reap(tk_norm *nm, bool all) {
    tk_ctx *c = nm->ctx;
    auto &r = nm->ext_retired;
    size_t keep = 0;
    for (size_t i = 0; i < r.size(); i++) {
        if (all || cudaEventQuery(r[i].second) == cudaSuccess) {
            cudaStreamWaitEvent(c->stream, r[i].second, 0);
            dfree(c, r[i].first);
            cudaEventDestroy(r[i].second);
        } else {
            r[keep++] = r[i];
        }
    }
    r.resize(keep);
    cudaGetLastError();   // a query that reported a copy still running
}

int norm_extract(tk_norm *nm, const tk_reads *const *sets, uint32_t nsets) {
    tk_ctx *c = nm->ctx;
    // the previous text, if its host copy may still run, is retired with that
    // copy's event rather than waited for: this extraction runs while the
    // previous one downloads
    if (nm->d_ext) {
        if (nm->ext_copy_done) {
            nm->ext_retired.emplace_back(nm->d_ext, nm->ext_copy_done);
            nm->ext_copy_done = nullptr;
        } else {
            dfree(c, nm->d_ext);
        }
        nm->d_ext = nullptr;
        nm->ext_len = 0;
    }
    ext_reap(nm, false);
    cudaEvent_t ev = nullptr;
    prof_begin(c, TK_KID_EXTRACT, &ev);
    const uint64_t P = nm->n_rows;
    uint64_t n_all = 0;
    for (uint32_t q = 0; q < nsets; q++) n_all += sets[q]->n_reads;
    Scratch sc(c);
    uint32_t *d_err = nullptr, *rec_len = nullptr;
    uint8_t *found = nullptr;
    uint64_t *offs = nullptr;
    unsigned long long *d_missing = nullptr;
    TK_TRY(sc.get((void **)&d_err, NE_WORDS * 4, "extract errors"));
    TK_TRY(sc.get((void **)&found, P, "extract found"));
    TK_TRY(sc.get((void **)&d_missing, 8, "extract missing"));
    TK_CUDA(c, cudaMemsetAsync(d_err, 0, NE_WORDS * 4, c->stream));
    TK_CUDA(c, cudaMemsetAsync(found, 0, P ? P : 1, c->stream));
    TK_CUDA(c, cudaMemsetAsync(d_missing, 0, 8, c->stream));
    if (!nm->d_hash) {
        // the selection's names, once: one slot per distinct name, the rows
        // that repeat a name (or name nothing) marked in d_keydup
        uint64_t cap = 1024;
        while (cap < 2 * nm->counts.selected) cap <<= 1;
        TK_TRY(dmalloc(c, (void **)&nm->d_keydup, P ? P : 1, "selected name repeats"));
        TK_TRY(dmalloc(c, (void **)&nm->d_hash, cap * 4, "selected names"));
        nm->hash_mask = cap - 1;
        TK_CUDA(c, cudaMemsetAsync(nm->d_hash, 0xFF, cap * 4, c->stream));
        TK_CUDA(c, cudaMemsetAsync(nm->d_keydup, 0, P ? P : 1, c->stream));
        if (P) {
            k_hash_insert<<<nm_grid(P), NM_THREADS, 0, c->stream>>>(nm->d_accs, nm->acc_off, P, nm->d_hash,
                                                                     nm->hash_mask, nm->d_keydup, d_err);
            c->launches++;
            TK_TRY(check_launch(c, "selected names"));
        }
    }
    const uint8_t *dup = nm->d_keydup;
    // per set: look its records up (marking the names found), then size them
    TK_TRY(sc.get((void **)&rec_len, n_all * 4, "extract lengths"));
    TK_TRY(sc.get((void **)&offs, (n_all + nsets) * 8, "extract offsets"));
    std::vector<uint64_t> base(nsets + 1, 0);
    uint64_t first = 0;
    for (uint32_t q = 0; q < nsets; q++) {
        const tk_reads *fq = sets[q];
        const uint64_t n = fq->n_reads;
        uint64_t total = 0;
        if (n) {
            uint32_t *rl = rec_len + first;
            if (fq->format == TK_FMT_FASTA)
                k_extract_find_fa<<<nm_grid(n), NM_THREADS, 0, c->stream>>>(fq->d_text, fq->text_len, fq->d_name_off,
                                                                             n, nm->d_accs, nm->acc_off, nm->d_hash,
                                                                             nm->hash_mask, found, rl, d_err);
            else
                k_extract_find<<<nm_grid(n), NM_THREADS, 0, c->stream>>>(fq->d_text, fq->text_len, fq->d_name_off,
                                                                          fq->d_name_len, n, nm->d_accs, nm->acc_off,
                                                                          nm->d_hash, nm->hash_mask, found, rl);
            c->launches++;
            TK_TRY(check_launch(c, "extract find"));
            TK_TRY(scan_excl_u32_to_u64(c, rl, offs + first + q, n, &total));
        }
        base[q + 1] = base[q] + total;
        first += n;
    }
    if (P) {
        k_extract_missing<<<nm_grid(P), NM_THREADS, 0, c->stream>>>(nm->acc_off, P, dup, found, d_missing);
        c->launches++;
    }
    uint32_t herr[NE_WORDS];
    unsigned long long missing = 0;
    TK_CUDA(c, cudaMemcpyAsync(&missing, d_missing, 8, cudaMemcpyDeviceToHost, c->stream));
    TK_TRY(read_err(c, d_err, herr));
    if (herr[NE_HASH]) return set_err(c, TK_E_INVAL, "extract: selected-name table full");
    if (herr[NE_DOMAIN])
        return set_err(c, TK_E_RANGE, "extract: a FASTA accession longer than " + std::to_string(FA_ACC_MAX) + " bytes");
    if (missing)
        return set_err(c, TK_E_PARSE, "extract: not all selected records were found (missing " +
                                          std::to_string(missing) + ")");
    const uint64_t total = base[nsets];
    TK_TRY(dmalloc(c, (void **)&nm->d_ext, total ? total : 1, "extracted reads"));
    first = 0;
    for (uint32_t q = 0; q < nsets; q++) {
        const tk_reads *fq = sets[q];
        const uint64_t n = fq->n_reads;
        const uint64_t len = base[q + 1] - base[q];
        if (n && len) {
            uint64_t *o = offs + first + q;   // n + 1 offsets of this set
            const uint64_t tail = len;
            TK_CUDA(c, cudaMemcpyAsync(o + n, &tail, 8, cudaMemcpyHostToDevice, c->stream));
            // offsets relative to this set's part, which starts at base[q] of d_ext
            if (fq->format == TK_FMT_FASTA) {
                k_extract_write_fa<<<nm_grid(n), NM_THREADS, 0, c->stream>>>(fq->d_text, fq->text_len,
                                                                              fq->d_name_off, n, o, base[q], nm->d_ext);
            } else {
                const bool vec = ((uintptr_t)fq->d_text & 3) == 0;
                k_extract_copy<<<(unsigned)((n + EX_RECS - 1) / EX_RECS), NM_THREADS, 0, c->stream>>>(
                    fq->d_text, fq->text_len, vec, fq->d_name_off, n, o, base[q], nm->d_ext);
            }
            c->launches++;
            TK_TRY(check_launch(c, "extract copy"));
        }
        first += n;
    }
    TK_CUDA(c, cudaStreamSynchronize(c->stream));
    nm->ext_len = total;
    prof_end(c, TK_KID_EXTRACT, ev, n_all);
    return TK_OK;
}

void norm_release(tk_norm *nm) {
    tk_ctx *c = nm->ctx;
    if (nm->ext_copy_done) {
        cudaStreamWaitEvent(c->stream, nm->ext_copy_done, 0);
        cudaEventDestroy(nm->ext_copy_done);
        nm->ext_copy_done = nullptr;
    }
    ext_reap(nm, true);
    side_free(c, nm->side[0]);
    side_free(c, nm->side[1]);
    void *p[] = {nm->row_l, nm->row_r, nm->row_n, nm->acc_off, nm->d_accs, nm->d_table, nm->d_ext, nm->d_hash,
                 nm->d_keydup};
    for (void *q : p)
        if (q) dfree(c, q);
}

}  // namespace tk
