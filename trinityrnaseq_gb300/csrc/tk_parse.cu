// tk_parse.cu -- K1: FASTA/FASTQ text -> device read set.
//
// The text is split into lines and records entirely on the GPU with tiled,
// coalesced passes (each thread owns 32 consecutive bytes, read as two 16-byte
// vectors; a block owns an 8 KB tile):
//   A1  newlines per tile                 -> scan -> first line of every tile
//   A2  newline positions (line ends)
//   L   line kinds: FASTA '>' header / sequence; FASTQ line index mod 4,
//       with the '@' and '+' checks of a 4-line record; header lines are
//       scanned into a record index per line
//   B1  emitted bases per tile (sequence-line bytes that are not whitespace)
//   B2  emit: base -> seq[emit_prefix + record] upper-cased; a header's first
//       byte records its read's start
//   N   accession (first header token) and read length per record
// Semantics follow PerlLib/Fasta_reader.pm:45-73 (records start at '>' lines,
// sequence = following lines with whitespace removed), Sequence->new at
// PerlLib/Fasta_reader.pm:107-118 (accession = first whitespace token), and the
// 4-line record checks of util/support_scripts/fastQ_to_fastA.pl:80-92.
#include "tk_internal.cuh"

namespace tk {

constexpr int PT_THREADS = 256;
constexpr int PT_BYTES = 32;
constexpr uint64_t PT_TILE = (uint64_t)PT_THREADS * PT_BYTES;

enum LineKind : uint8_t { LK_SKIP = 0, LK_HDR = 1, LK_SEQ = 2 };

// ' ', '\t', '\n', '\v', '\f', '\r' (9..13)
__device__ __forceinline__ bool is_ws(uint32_t c) { return c == ' ' || c - 9u < 5u; }

struct Bytes32 {
    uint32_t w[8];
    __device__ __forceinline__ uint32_t get(int i) const { return (w[i >> 2] >> ((i & 3) * 8)) & 0xFFu; }
};

// 32 bytes at p (p is 16-byte aligned relative to an aligned base when `vec`)
__device__ __forceinline__ Bytes32 load32(const char *__restrict__ text, uint64_t len, uint64_t p, bool vec) {
    Bytes32 b;
    if (vec && p + 32 <= len) {
        uint4 a = __ldg(reinterpret_cast<const uint4 *>(text + p));
        uint4 c = __ldg(reinterpret_cast<const uint4 *>(text + p + 16));
        b.w[0] = a.x; b.w[1] = a.y; b.w[2] = a.z; b.w[3] = a.w;
        b.w[4] = c.x; b.w[5] = c.y; b.w[6] = c.z; b.w[7] = c.w;
    } else {
#pragma unroll
        for (int i = 0; i < 8; i++) {
            uint32_t v = 0;
#pragma unroll
            for (int j = 0; j < 4; j++) {
                uint64_t q = p + (uint64_t)(i * 4 + j);
                uint32_t by = q < len ? (uint32_t)(uint8_t)text[q] : 0u;
                v |= by << (8 * j);
            }
            b.w[i] = v;
        }
    }
    return b;
}

struct ParseGeom {
    const char *text;
    uint64_t len;
    uint64_t S, E;        // parsed byte range (leading/trailing whitespace trimmed)
    uint64_t A;           // first tile start (S rounded down to 16)
    bool vec;
};

// ---- bounds: first non-whitespace byte and one past the last one
__global__ void k_bounds(const char *__restrict__ text, uint64_t len, unsigned long long *out) {
    __shared__ unsigned long long found;
    if (threadIdx.x == 0) found = ~0ULL;
    __syncthreads();
    for (uint64_t base = 0; base < len; base += blockDim.x) {
        uint64_t p = base + threadIdx.x;
        if (p < len && !is_ws((uint8_t)text[p])) atomicMin(&found, (unsigned long long)p);
        __syncthreads();
        if (found != ~0ULL) break;
        __syncthreads();
    }
    unsigned long long S = found;
    __syncthreads();
    if (threadIdx.x == 0) found = 0;
    __syncthreads();
    if (S != ~0ULL) {
        for (uint64_t base = 0; base < len; base += blockDim.x) {
            uint64_t q = base + threadIdx.x;
            if (q < len) {
                uint64_t p = len - 1 - q;
                if (!is_ws((uint8_t)text[p])) atomicMax(&found, (unsigned long long)(p + 1));
            }
            __syncthreads();
            if (found != 0) break;
            __syncthreads();
        }
    }
    if (threadIdx.x == 0) {
        out[0] = S == ~0ULL ? len : S;
        out[1] = S == ~0ULL ? len : found;
        out[2] = S == ~0ULL ? 0 : (uint8_t)text[S];
    }
}

// Bit i set when byte p+i (p = this thread's first byte) is a '\n' inside
// [S, E).  Per 4-byte word the equal bytes are found with the exact
// zero-byte test and their top bits gathered by one multiply.
__device__ __forceinline__ uint32_t newline_bits(const ParseGeom &g, const Bytes32 &b, uint64_t p) {
    uint32_t m = 0;
#pragma unroll
    for (int q = 0; q < 8; q++) {
        const uint32_t v = b.w[q] ^ 0x0A0A0A0Au;
        const uint32_t z = ~((((v & 0x7F7F7F7Fu) + 0x7F7F7F7Fu) | v)) & 0x80808080u;   // bit 7 of each '\n' byte
        m |= ((((z >> 7) * 0x00204081u) >> 21) & 0xFu) << (4 * q);                     // byte b -> bit b
    }
    if (p < g.S) m &= g.S - p >= 32 ? 0u : ~0u << (g.S - p);
    if (p + 32 > g.E) m &= g.E <= p ? 0u : (g.E - p >= 32 ? ~0u : (1u << (g.E - p)) - 1u);
    return m;
}

// ---- A1: newlines per tile, and each thread's newline bits for A2
__global__ void k_tile_newlines(ParseGeom g, uint32_t *__restrict__ tile_nl, uint32_t *__restrict__ nl_bits) {
    __shared__ uint32_t sm[PT_THREADS / 32 + 1];
    uint64_t p = g.A + (uint64_t)blockIdx.x * PT_TILE + (uint64_t)threadIdx.x * PT_BYTES;
    Bytes32 b = load32(g.text, g.len, p, g.vec);
    const uint32_t m = newline_bits(g, b, p);
    nl_bits[(uint64_t)blockIdx.x * PT_THREADS + threadIdx.x] = m;
    uint32_t tot;
    block_excl_scan<uint32_t>(__popc(m), sm, &tot);
    if (threadIdx.x == 0) tile_nl[blockIdx.x] = tot;
}

// ---- A2: line ends, from the newline bits (1/8 of the text's bytes)
__global__ void k_line_ends(ParseGeom g, const uint32_t *__restrict__ nl_bits, const uint64_t *__restrict__ tile_line0,
                            uint64_t *__restrict__ line_end) {
    __shared__ uint32_t sm[PT_THREADS / 32 + 1];
    const uint64_t p = g.A + (uint64_t)blockIdx.x * PT_TILE + (uint64_t)threadIdx.x * PT_BYTES;
    uint32_t m = nl_bits[(uint64_t)blockIdx.x * PT_THREADS + threadIdx.x];
    uint32_t tot;
    uint64_t line = tile_line0[blockIdx.x] + block_excl_scan<uint32_t>(__popc(m), sm, &tot);
    while (m) {
        line_end[line++] = p + (uint32_t)(__ffs(m) - 1);
        m &= m - 1;
    }
}

// ---- L: line kinds.  FASTQ errors record the first offending line.
__global__ void k_line_kinds(ParseGeom g, const uint64_t *__restrict__ line_end, uint64_t n_lines, int fastq,
                             uint8_t *__restrict__ kind, uint32_t *__restrict__ is_hdr, uint32_t *__restrict__ len,
                             uint32_t *__restrict__ err) {
    uint64_t j = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= n_lines) return;
    uint64_t ls = j == 0 ? g.S : line_end[j - 1] + 1;
    uint64_t le = line_end[j];
    uint32_t first = le > ls ? (uint8_t)g.text[ls] : 0u;
    uint8_t kd;
    uint32_t h = 0;
    if (!fastq) {
        h = first == '>';
        kd = h ? LK_HDR : LK_SEQ;
    } else {
        uint32_t m = (uint32_t)(j & 3);
        if (m == 0) {
            h = 1;
            kd = LK_HDR;
            if (first != '@') { atomicExch(&err[DE_PARSE], 1u); atomicMin(&err[DE_PARSE + 1], (uint32_t)(j + 1)); }
        } else if (m == 1) {
            kd = LK_SEQ;
        } else {
            kd = LK_SKIP;
            if (m == 2 && first != '+') { atomicExch(&err[DE_PARSE], 1u); atomicMin(&err[DE_PARSE + 1], (uint32_t)(j + 1)); }
        }
    }
    kind[j] = kd;
    is_hdr[j] = h;
    // fast path: bytes the line emits if sequence lines hold no whitespace
    // besides their newline (checked while copying); k_line_records clears
    // lines that precede the first record
    len[j] = kd == LK_SEQ ? (uint32_t)(le - ls) : 0u;
}

// record index per line (~0 before the first header) and header line per record
__global__ void k_line_records(const uint32_t *__restrict__ is_hdr, uint64_t *__restrict__ line_rec_io, uint64_t n_lines,
                               uint64_t *__restrict__ hdr_line, uint32_t *__restrict__ len) {
    uint64_t j = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= n_lines) return;
    uint64_t incl = line_rec_io[j] + is_hdr[j];   // exclusive scan + own flag
    if (is_hdr[j]) hdr_line[incl - 1] = j;
    line_rec_io[j] = incl == 0 ? ~0ULL : incl - 1;
    if (incl == 0) len[j] = 0u;
}

// FASTQ: line j belongs to record j >> 2, whose header is line 4r
__global__ void k_fastq_records(uint64_t *__restrict__ line_rec, uint64_t n_lines, uint64_t *__restrict__ hdr_line) {
    const uint64_t j = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= n_lines) return;
    line_rec[j] = j >> 2;
    if ((j & 3) == 0) hdr_line[j >> 2] = j;
}

// ---- fast path, copy.  A warp takes 32 consecutive lines (or records): lane l
// loads line l's metadata (coalesced), header lines record their read's start,
// and then the warp copies the group's sequence lines in aligned 16-byte
// output words (copy_group), upper-casing into seq.  A sequence line holding
// whitespace sets *ws_seen and the byte-wise path redoes the emit.
// Byte mask of the bytes [a, b) of a 4-byte word (0 <= a, b <= 4).
__device__ __forceinline__ uint32_t byte_mask(int a, int b) {
    return b > a ? (0xFFFFFFFFu >> (32 - 8 * (b - a))) << (8 * a) : 0u;
}

// The 16 bytes at offset so of a line of n bytes starting at text position
// S, as four words, and per word the mask of its bytes inside the line
// (bytes outside it read as 'A').  Five aligned 4-byte loads and funnel
// shifts when the text is aligned and they lie inside it, byte loads
// otherwise.
__device__ __forceinline__ void line_word16(const ParseGeom &g, uint64_t S, int64_t so, uint32_t n, uint32_t (&x)[4],
                                            uint32_t (&in)[4]) {
    const int64_t rest = (int64_t)n - so;                    // bytes [lo, hi) are in the line
    const int lo = so < 0 ? (so < -16 ? 16 : (int)-so) : 0;
    const int hi = rest < 16 ? (rest < 0 ? 0 : (int)rest) : 16;
#pragma unroll
    for (int q = 0; q < 4; q++) in[q] = byte_mask(min(max(lo - 4 * q, 0), 4), min(max(hi - 4 * q, 0), 4));
    const int64_t a = (int64_t)S + so;
    if (g.vec && a >= 0 && (uint64_t)((a & ~3LL) + 20) <= g.len) {
        const uint32_t *p = reinterpret_cast<const uint32_t *>(g.text + (a & ~3LL));
        const uint32_t sh = 8u * (uint32_t)(a & 3);
        uint32_t w[5];
#pragma unroll
        for (int i = 0; i < 5; i++) w[i] = __ldg(p + i);
#pragma unroll
        for (int q = 0; q < 4; q++) x[q] = (__funnelshift_r(w[q], w[q + 1], sh) & in[q]) | (0x41414141u & ~in[q]);
        return;
    }
#pragma unroll
    for (int q = 0; q < 4; q++) {
        x[q] = 0;
        for (int i = 0; i < 4; i++) {
            const int64_t o = so + 4 * q + i;
            const uint32_t c = (o >= 0 && o < (int64_t)n) ? (uint8_t)g.text[S + o] : 0x41u;
            x[q] |= c << (8 * i);
        }
    }
}

// Upper-cases a word of bases; notes whether it held whitespace (' ' or 9..13).
__device__ __forceinline__ uint32_t upcase_word(uint32_t x, bool &ws) {
    const uint32_t t = x & 0x7F7F7F7Fu;
    // bit 7 of each byte that is a-z, then of each byte that is ' ' or 9..13
    const uint32_t lower = (t + 0x1F1F1F1Fu) & ~(t + 0x05050505u) & ~x & 0x80808080u;
    const uint32_t sp = x ^ 0x20202020u;
    const uint32_t zsp = ~(((sp & 0x7F7F7F7Fu) + 0x7F7F7F7Fu) | sp) & 0x80808080u;
    const uint32_t rng = (t + 0x77777777u) & ~(t + 0x72727272u) & ~x & 0x80808080u;
    ws |= (zsp | rng) != 0u;
    return x ^ (lower >> 2);
}

// The warp copies the lines its lanes hold (lane l: text[src, src + len) to
// seq + dst; len 0 = none), upper-casing, and notes whether a line held
// whitespace.  The output is cut into the aligned 16-byte words the lines
// touch; the warp numbers the words of its 32 lines one after another (a scan
// of each line's word count) and each lane takes every 32nd, so the lanes stay
// busy whatever the line lengths; a lane finds its word's line by a binary
// search over the lanes' first word numbers.  A word wholly inside its line
// is one 16-byte store; the first and last word of a line (shared with the
// separator and the neighbouring line) are stored byte by byte.  seq is
// 16-byte aligned.
__device__ __forceinline__ void copy_group(const ParseGeom &g, uint64_t src, uint64_t dst, uint32_t len,
                                           uint8_t *__restrict__ seq, bool &ws) {
    const unsigned lane = lane_id();
    const uint32_t nw = len ? (uint32_t)(((dst + len + 15) >> 4) - (dst >> 4)) : 0u;
    uint32_t incl = nw;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const uint32_t t = __shfl_up_sync(0xffffffffu, incl, o);
        if (lane >= (unsigned)o) incl += t;
    }
    const uint32_t total = __shfl_sync(0xffffffffu, incl, 31);
    const uint32_t first = incl - nw;   // this lane's line's first word number
    for (uint32_t base = 0; base < total; base += 32) {
        const uint32_t t = base + lane;
        // the last lane whose first word number is <= t: its line holds word t
        // (a line without words shares its first number with the next line)
        int i = 0;
#pragma unroll
        for (int step = 16; step >= 1; step >>= 1) {
            const uint32_t f = __shfl_sync(0xffffffffu, first, (i + step) & 31);
            if (i + step < 32 && f <= t) i += step;
        }
        const uint64_t s_i = __shfl_sync(0xffffffffu, src, i);
        const uint64_t d_i = __shfl_sync(0xffffffffu, dst, i);
        const uint32_t n_i = __shfl_sync(0xffffffffu, len, i);
        const uint32_t f_i = __shfl_sync(0xffffffffu, first, i);
        if (t >= total) continue;
        const uint64_t out = (d_i & ~15ULL) + 16ull * (t - f_i);   // the word's first output byte
        const int64_t so = (int64_t)out - (int64_t)d_i;            // its offset in the line
        uint32_t x[4], in[4];
        line_word16(g, s_i, so, n_i, x, in);
#pragma unroll
        for (int q = 0; q < 4; q++) x[q] = upcase_word(x[q], ws);
        uint8_t *o = seq + out;
        if (so >= 0 && so + 16 <= (int64_t)n_i) {
            *reinterpret_cast<uint4 *>(o) = make_uint4(x[0], x[1], x[2], x[3]);
        } else {
            // a line's first or last word: whole 4-byte pieces inside the
            // line as words, the piece cut by a line end byte by byte
#pragma unroll
            for (int q = 0; q < 4; q++) {
                if (in[q] == 0xFFFFFFFFu) {
                    reinterpret_cast<uint32_t *>(o)[q] = x[q];
                } else if (in[q]) {
#pragma unroll
                    for (int i = 0; i < 4; i++)
                        if ((in[q] >> (8 * i)) & 0xFFu) o[4 * q + i] = (uint8_t)(x[q] >> (8 * i));
                }
            }
        }
    }
}

__global__ void k_copy_lines(ParseGeom g, const uint64_t *__restrict__ line_end, const uint8_t *__restrict__ kind,
                             const uint64_t *__restrict__ line_rec, const uint64_t *__restrict__ line_out,
                             uint64_t n_lines, uint8_t *__restrict__ seq, uint64_t *__restrict__ rd_off,
                             uint32_t *__restrict__ ws_seen) {
    const unsigned lane = lane_id();
    const uint64_t warps = (uint64_t)gridDim.x * (blockDim.x >> 5);
    bool ws = false;
    for (uint64_t j0 = ((uint64_t)blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5)) * 32; j0 < n_lines; j0 += warps * 32) {
        const uint64_t j = j0 + lane;
        uint64_t src = 0, dst = 0;
        uint32_t len = 0;
        if (j < n_lines) {
            const uint8_t kd = kind[j];
            const uint64_t rec = line_rec[j];
            if (rec != ~0ULL) {
                const uint64_t out = line_out[j] + rec;
                if (kd == LK_HDR) rd_off[rec] = out;
                else if (kd == LK_SEQ) {
                    src = j == 0 ? g.S : line_end[j - 1] + 1;
                    len = (uint32_t)(line_end[j] - src);
                    dst = out;
                }
            }
        }
        copy_group(g, src, dst, len, seq, ws);
    }
    if (__any_sync(0xffffffffu, ws) && lane == 0) atomicExch(ws_seen, 1u);
}

// ---- FASTQ: records of four lines, handled per record (no per-line arrays).
// Check: the header line starts with '@' and the third with '+' (the first
// offending line is recorded, as k_line_kinds does); seq_len = the sequence
// line's length.
__global__ void k_fq_check(ParseGeom g, const uint64_t *__restrict__ line_end, uint64_t n_reads,
                           uint32_t *__restrict__ seq_len, uint32_t *__restrict__ err) {
    const uint64_t r = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (r >= n_reads) return;
    const uint64_t j = 4 * r;
    const uint64_t h0 = j == 0 ? g.S : line_end[j - 1] + 1, h1 = line_end[j];
    const uint64_t p0 = line_end[j + 1] + 1, p1 = line_end[j + 2];
    const uint32_t fh = h1 > h0 ? (uint8_t)g.text[h0] : 0u, fp = p1 > p0 ? (uint8_t)g.text[p0] : 0u;
    if (fh != '@') { atomicExch(&err[DE_PARSE], 1u); atomicMin(&err[DE_PARSE + 1], (uint32_t)(j + 1)); }
    if (fp != '+') { atomicExch(&err[DE_PARSE], 1u); atomicMin(&err[DE_PARSE + 1], (uint32_t)(j + 3)); }
    seq_len[r] = (uint32_t)(line_end[j + 1] - (h1 + 1));
}

// A warp takes 32 consecutive records: lane l records read r0 + l's start and
// holds its sequence line, then the warp copies them as k_copy_lines does.
__global__ void k_fq_copy(ParseGeom g, const uint64_t *__restrict__ line_end, const uint64_t *__restrict__ seq_off,
                          uint64_t n_reads, uint8_t *__restrict__ seq, uint64_t *__restrict__ rd_off,
                          uint32_t *__restrict__ ws_seen) {
    const unsigned lane = lane_id();
    const uint64_t warps = (uint64_t)gridDim.x * (blockDim.x >> 5);
    bool ws = false;
    for (uint64_t r0 = ((uint64_t)blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5)) * 32; r0 < n_reads; r0 += warps * 32) {
        const uint64_t r = r0 + lane;
        uint64_t src = 0, dst = 0;
        uint32_t len = 0;
        if (r < n_reads) {
            src = line_end[4 * r] + 1;
            len = (uint32_t)(line_end[4 * r + 1] - src);
            dst = seq_off[r] + r;
            rd_off[r] = dst;
        }
        copy_group(g, src, dst, len, seq, ws);
    }
    if (__any_sync(0xffffffffu, ws) && lane == 0) atomicExch(ws_seen, 1u);
}

// per-thread walk over its 32 bytes with the line each byte belongs to
struct LineWalk {
    uint64_t line;
    uint8_t kind;
    uint64_t rec;
};

__device__ __forceinline__ void line_info(const uint8_t *__restrict__ kind, const uint64_t *__restrict__ line_rec,
                                          uint64_t line, uint64_t n_lines, LineWalk &w) {
    w.line = line;
    if (line < n_lines) {
        w.kind = kind[line];
        w.rec = line_rec[line];
    } else {
        w.kind = LK_SKIP;
        w.rec = ~0ULL;
    }
}

// ---- B1: emitted bytes per tile
__global__ void k_tile_emits(ParseGeom g, const uint64_t *__restrict__ tile_line0, const uint8_t *__restrict__ kind,
                             const uint64_t *__restrict__ line_rec, uint64_t n_lines, uint32_t *__restrict__ tile_emit) {
    __shared__ uint32_t sm[PT_THREADS / 32 + 1];
    uint64_t p = g.A + (uint64_t)blockIdx.x * PT_TILE + (uint64_t)threadIdx.x * PT_BYTES;
    Bytes32 b = load32(g.text, g.len, p, g.vec);
    uint32_t nl = 0;
#pragma unroll
    for (int i = 0; i < PT_BYTES; i++) {
        uint64_t q = p + i;
        nl += (q >= g.S && q < g.E && b.get(i) == '\n');
    }
    uint32_t tot;
    uint64_t line = tile_line0[blockIdx.x] + block_excl_scan<uint32_t>(nl, sm, &tot);
    LineWalk w;
    line_info(kind, line_rec, line, n_lines, w);
    uint32_t em = 0;
    for (int i = 0; i < PT_BYTES; i++) {
        uint64_t q = p + i;
        if (q < g.S || q >= g.E) continue;
        uint32_t c = b.get(i);
        if (c == '\n') {
            line_info(kind, line_rec, w.line + 1, n_lines, w);
            continue;
        }
        em += (w.kind == LK_SEQ && w.rec != ~0ULL && !is_ws(c));
    }
    block_excl_scan<uint32_t>(em, sm, &tot);
    if (threadIdx.x == 0) tile_emit[blockIdx.x] = tot;
}

// ---- B2: write upper-cased bases and read starts
__global__ void k_emit(ParseGeom g, const uint64_t *__restrict__ tile_line0, const uint64_t *__restrict__ tile_emit0,
                       const uint8_t *__restrict__ kind, const uint64_t *__restrict__ line_rec, uint64_t n_lines,
                       uint8_t *__restrict__ seq, uint64_t *__restrict__ rd_off) {
    __shared__ uint32_t sm[PT_THREADS / 32 + 1];
    uint64_t p = g.A + (uint64_t)blockIdx.x * PT_TILE + (uint64_t)threadIdx.x * PT_BYTES;
    Bytes32 b = load32(g.text, g.len, p, g.vec);
    uint32_t nl = 0;
#pragma unroll
    for (int i = 0; i < PT_BYTES; i++) {
        uint64_t q = p + i;
        nl += (q >= g.S && q < g.E && b.get(i) == '\n');
    }
    uint32_t tot;
    uint64_t line = tile_line0[blockIdx.x] + block_excl_scan<uint32_t>(nl, sm, &tot);
    LineWalk w;
    line_info(kind, line_rec, line, n_lines, w);
    uint32_t em = 0;
    for (int i = 0; i < PT_BYTES; i++) {
        uint64_t q = p + i;
        if (q < g.S || q >= g.E) continue;
        uint32_t c = b.get(i);
        if (c == '\n') { line_info(kind, line_rec, w.line + 1, n_lines, w); continue; }
        em += (w.kind == LK_SEQ && w.rec != ~0ULL && !is_ws(c));
    }
    uint64_t pos = tile_emit0[blockIdx.x] + block_excl_scan<uint32_t>(em, sm, &tot);
    line_info(kind, line_rec, line, n_lines, w);
    bool nl_before = p > g.S && p - 1 < g.E && g.text[p - 1] == '\n';
    for (int i = 0; i < PT_BYTES; i++) {
        uint64_t q = p + i;
        if (q < g.S || q >= g.E) continue;
        uint32_t c = b.get(i);
        bool line_start = q == g.S || nl_before;
        nl_before = c == '\n';
        if (c == '\n') {
            line_info(kind, line_rec, w.line + 1, n_lines, w);
            continue;
        }
        if (line_start && w.kind == LK_HDR) rd_off[w.rec] = pos + w.rec;
        if (w.kind == LK_SEQ && w.rec != ~0ULL && !is_ws(c)) {
            uint32_t u = (c >= 'a' && c <= 'z') ? c - 32u : c;
            seq[pos + w.rec] = (uint8_t)u;
            pos++;
        }
    }
}

// ---- N: accession and read length per record
__global__ void k_names(ParseGeom g, const uint64_t *__restrict__ hdr_line, int fastq,
                        const uint64_t *__restrict__ line_end, uint64_t n_reads, const uint64_t *__restrict__ rd_off,
                        uint64_t *__restrict__ name_off, uint32_t *__restrict__ name_len, uint32_t *__restrict__ max_len) {
    const uint64_t r = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    uint32_t L32 = 0;
    if (r < n_reads) {
        const uint64_t j = fastq ? 4 * r : hdr_line[r];   // FASTQ: the header is line 4r
        const uint64_t ls = j == 0 ? g.S : line_end[j - 1] + 1;
        const uint64_t le = line_end[j];
        uint64_t s = ls + 1, q = s;
        // byte by byte: a thread's header bytes share sectors, and 16-byte
        // word loads of unrelated headers per lane were slower
        while (q < le && !is_ws((uint8_t)g.text[q])) q++;
        name_off[r] = s;
        name_len[r] = (uint32_t)(q - s);
        const uint64_t L = rd_off[r + 1] - rd_off[r] - 1;
        L32 = (uint32_t)(L > 0xFFFFFFFFull ? 0xFFFFFFFFull : L);
    }
    // one atomic per warp (the longest read of its 32)
    L32 = __reduce_max_sync(0xffffffffu, L32);
    if (lane_id() == 0 && L32) atomicMax(max_len, L32);
}

// The packed read array as 2-bit codes and invalid-position bits: thread j
// converts positions 32j .. 32j+31 (j = -1 .. n_words-1; the 64 '\n' bytes
// around `seq` make word -1 all invalid).  Per 4-byte group: the code of
// A/C/G/T is ((c >> 1) & 3) ^ (its bit 1 moved to bit 0); the group is valid
// where its bytes equal the letters those codes name.
__global__ void k_pack_codes(const uint8_t *__restrict__ seq, int64_t n_words, uint64_t *__restrict__ codes,
                             uint32_t *__restrict__ inv) {
    const int64_t j = (int64_t)blockIdx.x * blockDim.x + threadIdx.x - 1;
    if (j >= n_words) return;
    const uint4 *v = reinterpret_cast<const uint4 *>(seq + 32 * j);
    const uint4 a = v[0], b = v[1];
    const uint32_t w[8] = {a.x, a.y, a.z, a.w, b.x, b.y, b.z, b.w};
    uint64_t code = 0;
    uint32_t bad = 0;
#pragma unroll
    for (int q = 0; q < 8; q++) {
        uint32_t x = (w[q] >> 1) & 0x03030303u;
        x ^= (x >> 1) & 0x01010101u;   // byte b: code of position 4q+b
        // the letter each code names, compared with the byte itself
        const uint32_t sel = (x & 3u) | ((x >> 4) & 0x30u) | ((x >> 8) & 0x300u) | ((x >> 12) & 0x3000u);
        const uint32_t d = w[q] ^ __byte_perm(0x54474341u, 0u, sel);
        const uint32_t nz = (d | ((d & 0x7F7F7F7Fu) + 0x7F7F7F7Fu)) & 0x80808080u;   // bit 7 of each differing byte
        const uint32_t nib = (((nz >> 7) * 0x08040201u) >> 24) & 0xFu;                  // position 4q at bit 3
        const uint32_t byte = ((x << 6) & 0xC0u) | ((x >> 4) & 0x30u) | ((x >> 14) & 0x0Cu) | ((x >> 24) & 0x03u);
        code = (code << 8) | byte;
        bad = (bad << 4) | nib;
    }
    codes[j] = code;
    inv[j] = bad;
}

static inline unsigned grid_for(uint64_t n, int threads) { return (unsigned)((n + threads - 1) / threads); }

// Builds r->d_codes / r->d_inv from r->d_seq (after the last write to seq).
static int pack_reads(tk_ctx *c, tk_reads *r) {
    const int64_t n_words = (int64_t)((r->seq_len + 31) / 32) + 1;
    const uint64_t code_words = (uint64_t)n_words + 1;          // incl. word -1
    const uint64_t inv_words = ((uint64_t)n_words + 1 + 1) & ~1ULL;
    TK_TRY(dmalloc(c, (void **)&r->d_pack_alloc, code_words * 8 + inv_words * 4, "2-bit codes"));
    uint64_t *codes = r->d_pack_alloc + 1;
    uint32_t *inv = reinterpret_cast<uint32_t *>(r->d_pack_alloc + code_words) + 1;
    k_pack_codes<<<grid_for((uint64_t)n_words + 1, 256), 256, 0, c->stream>>>(r->d_seq, n_words, codes, inv);
    c->launches++;
    r->d_codes = codes;
    r->d_inv = inv;
    return check_launch(c, "2-bit codes");
}

int parse_reads(tk_ctx *c, tk_reads *r) {
    const char *text = r->d_text;
    uint64_t len = r->text_len;
    unsigned long long *d_bounds = nullptr;
    unsigned long long hb[3] = {0, 0, 0};
    cudaEvent_t ev;
    prof_begin(c, TK_KID_PARSE, &ev);
    TK_TRY(dmalloc(c, (void **)&d_bounds, 3 * sizeof(unsigned long long), "parse bounds"));
    k_bounds<<<1, 256, 0, c->stream>>>(text, len, d_bounds);
    c->launches++;
    int e = cuda_check(c, cudaMemcpyAsync(hb, d_bounds, sizeof(hb), cudaMemcpyDeviceToHost, c->stream), "bounds d2h");
    if (!e) e = cuda_check(c, cudaStreamSynchronize(c->stream), "bounds sync");
    dfree(c, d_bounds);
    if (e) return e;
    ParseGeom g;
    g.text = text;
    g.len = len;
    g.S = hb[0];
    g.E = hb[1];
    g.vec = ((uintptr_t)text & 15u) == 0;
    g.A = g.vec ? (g.S & ~15ULL) : g.S;
    r->format = g.S >= g.E ? TK_FMT_NONE : (hb[2] == '@' ? TK_FMT_FASTQ : TK_FMT_FASTA);
    const int fastq = r->format == TK_FMT_FASTQ;

    uint64_t n_tiles = g.S >= g.E ? 0 : (g.E - g.A + PT_TILE - 1) / PT_TILE;
    uint32_t *tile_nl = nullptr, *tile_em = nullptr, *is_hdr = nullptr, *nl_bits = nullptr;
    uint64_t *tile_line0 = nullptr, *tile_emit0 = nullptr, *line_end = nullptr, *line_rec = nullptr, *hdr_line = nullptr;
    uint32_t *line_len = nullptr;
    uint64_t *line_out = nullptr;
    uint8_t *kind = nullptr;
    uint32_t *d_maxlen = nullptr;
    uint64_t n_nl = 0, n_lines = 0, n_reads = 0, n_emit = 0;
    std::vector<void *> tmp;
    auto alloc = [&](void **p, size_t bytes, const char *what) {
        int ee = dmalloc(c, p, bytes ? bytes : 16, what);
        if (!ee) tmp.push_back(*p);
        return ee;
    };
    do {
        if (n_tiles == 0) break;
        if ((e = alloc((void **)&tile_nl, n_tiles * 4, "tile newlines"))) break;
        if ((e = alloc((void **)&tile_line0, (n_tiles + 1) * 8, "tile lines"))) break;
        if ((e = alloc((void **)&nl_bits, n_tiles * PT_THREADS * 4, "newline bits"))) break;
        k_tile_newlines<<<(unsigned)n_tiles, PT_THREADS, 0, c->stream>>>(g, tile_nl, nl_bits);
        c->launches++;
        if ((e = scan_excl_u32_to_u64(c, tile_nl, tile_line0, n_tiles, &n_nl))) break;
        n_lines = n_nl + 1;
        if ((e = alloc((void **)&line_end, n_lines * 8, "line ends"))) break;
        k_line_ends<<<(unsigned)n_tiles, PT_THREADS, 0, c->stream>>>(g, nl_bits, tile_line0, line_end);
        c->launches++;
        if ((e = cuda_check(c, cudaMemcpyAsync(line_end + n_nl, &g.E, 8, cudaMemcpyHostToDevice, c->stream), "line end"))) break;
        if (fastq && (n_lines & 3) != 0) {
            e = set_err(c, TK_E_PARSE, "FASTQ input: " + std::to_string(n_lines) + " lines is not a multiple of 4");
            break;
        }
        if ((e = cuda_check(c, cudaMemsetAsync(c->d_err, 0, DE_COUNT * 4, c->stream), "err reset"))) break;
        uint32_t big = 0xFFFFFFFFu;
        cudaMemcpyAsync(c->d_err + DE_PARSE + 1, &big, 4, cudaMemcpyHostToDevice, c->stream);
        uint32_t herr[2] = {0, 0};
        if (fastq) {
            // 4-line records, handled per record: checks and sequence lengths,
            // their scan gives every read's place in seq
            n_reads = n_lines / 4;
            if ((e = alloc((void **)&line_len, n_reads * 4, "sequence lengths"))) break;
            k_fq_check<<<grid_for(n_reads, 256), 256, 0, c->stream>>>(g, line_end, n_reads, line_len, c->d_err);
            c->launches++;
            if ((e = cuda_check(c, cudaMemcpyAsync(herr, c->d_err + DE_PARSE, 8, cudaMemcpyDeviceToHost, c->stream), "err d2h"))) break;
            if ((e = alloc((void **)&line_out, (n_reads + 1) * 8, "sequence offsets"))) break;
            if ((e = scan_excl_u32_to_u64(c, line_len, line_out, n_reads, &n_emit))) break;   // syncs
            if (herr[0]) {
                e = set_err(c, TK_E_PARSE, "FASTQ input: malformed record at line " + std::to_string(herr[1]));
                break;
            }
            break;
        }
        if ((e = alloc((void **)&kind, n_lines, "line kinds"))) break;
        if ((e = alloc((void **)&is_hdr, n_lines * 4, "header flags"))) break;
        if ((e = alloc((void **)&line_rec, n_lines * 8, "line records"))) break;
        if ((e = alloc((void **)&line_len, n_lines * 4, "line lengths"))) break;
        k_line_kinds<<<grid_for(n_lines, 256), 256, 0, c->stream>>>(g, line_end, n_lines, fastq, kind, is_hdr, line_len,
                                                                     c->d_err);
        c->launches++;
        if ((e = cuda_check(c, cudaMemcpyAsync(herr, c->d_err + DE_PARSE, 8, cudaMemcpyDeviceToHost, c->stream), "err d2h"))) break;
        {
            if ((e = scan_excl_u32_to_u64(c, is_hdr, line_rec, n_lines, &n_reads))) break;  // syncs
            if ((e = alloc((void **)&hdr_line, (n_reads + 1) * 8, "header lines"))) break;
            k_line_records<<<grid_for(n_lines, 256), 256, 0, c->stream>>>(is_hdr, line_rec, n_lines, hdr_line, line_len);
            c->launches++;
        }
        if ((e = alloc((void **)&line_out, (n_lines + 1) * 8, "line outputs"))) break;
        if ((e = scan_excl_u32_to_u64(c, line_len, line_out, n_lines, &n_emit))) break;   // syncs
        if (herr[0]) {
            e = set_err(c, TK_E_PARSE, "FASTQ input: malformed record at line " + std::to_string(herr[1]));
            break;
        }
    } while (0);
    if (e) {
        for (void *p : tmp) dfree(c, p);
        return e;
    }
    r->n_reads = n_reads;
    r->n_bases = n_emit;
    r->seq_len = n_emit + n_reads;
    uint64_t seq_alloc = ((r->seq_len + 2 * SEQ_PAD + 15) / 16) * 16 + 16;
    e = dmalloc(c, (void **)&r->d_seq_alloc, seq_alloc, "packed reads");
    if (!e) e = dmalloc(c, (void **)&r->d_rd_off, (n_reads + 1) * 8, "read offsets");
    if (!e) e = dmalloc(c, (void **)&r->d_name_off, (n_reads ? n_reads : 1) * 8, "name offsets");
    if (!e) e = dmalloc(c, (void **)&r->d_name_len, (n_reads ? n_reads : 1) * 4, "name lengths");
    if (!e) e = dmalloc(c, (void **)&d_maxlen, 4, "max length");
    if (!e) {
        r->d_seq = r->d_seq_alloc + SEQ_PAD;
        cudaMemsetAsync(r->d_seq_alloc, '\n', seq_alloc, c->stream);
        cudaMemsetAsync(d_maxlen, 0, 4, c->stream);
        uint64_t tail = r->seq_len;
        cudaMemcpyAsync(r->d_rd_off + n_reads, &tail, 8, cudaMemcpyHostToDevice, c->stream);
        uint32_t ws_seen = 0;
        if (n_tiles && n_reads) {
            cudaMemsetAsync(c->d_err + DE_WS, 0, 4, c->stream);
            if (fastq) {
                const unsigned grid = (unsigned)std::max<uint64_t>(1, std::min<uint64_t>((n_reads + 255) / 256,
                                                                                       (uint64_t)c->sm_count * 32));
                k_fq_copy<<<grid, 256, 0, c->stream>>>(g, line_end, line_out, n_reads, r->d_seq, r->d_rd_off,
                                                       c->d_err + DE_WS);
            } else {
                const unsigned grid = (unsigned)std::max<uint64_t>(1, std::min<uint64_t>((n_lines + 7) / 8,
                                                                                       (uint64_t)c->sm_count * 32));
                k_copy_lines<<<grid, 256, 0, c->stream>>>(g, line_end, kind, line_rec, line_out, n_lines, r->d_seq,
                                                          r->d_rd_off, c->d_err + DE_WS);
            }
            c->launches++;
            e = cuda_check(c, cudaMemcpyAsync(&ws_seen, c->d_err + DE_WS, 4, cudaMemcpyDeviceToHost, c->stream), "ws flag");
            if (!e) e = cuda_check(c, cudaStreamSynchronize(c->stream), "copy sync");
        }
        if (!e && ws_seen) {
            // some sequence line holds spaces, tabs or CRs: redo the emit byte by byte
            do {
                if (fastq) {
                    // the byte-wise emit works from the per-line arrays
                    if ((e = alloc((void **)&kind, n_lines, "line kinds"))) break;
                    if ((e = alloc((void **)&is_hdr, n_lines * 4, "header flags"))) break;
                    if ((e = alloc((void **)&line_rec, n_lines * 8, "line records"))) break;
                    uint32_t *ll = nullptr;
                    uint64_t *hl = nullptr;
                    if ((e = alloc((void **)&ll, n_lines * 4, "line lengths"))) break;
                    if ((e = alloc((void **)&hl, (n_reads + 1) * 8, "header lines"))) break;
                    k_line_kinds<<<grid_for(n_lines, 256), 256, 0, c->stream>>>(g, line_end, n_lines, fastq, kind, is_hdr,
                                                                                 ll, c->d_err);
                    k_fastq_records<<<grid_for(n_lines, 256), 256, 0, c->stream>>>(line_rec, n_lines, hl);
                    c->launches += 2;
                }
                if ((e = alloc((void **)&tile_em, n_tiles * 4, "tile emits"))) break;
                if ((e = alloc((void **)&tile_emit0, (n_tiles + 1) * 8, "tile emit offsets"))) break;
                k_tile_emits<<<(unsigned)n_tiles, PT_THREADS, 0, c->stream>>>(g, tile_line0, kind, line_rec, n_lines, tile_em);
                c->launches++;
                if ((e = scan_excl_u32_to_u64(c, tile_em, tile_emit0, n_tiles, &n_emit))) break;
                r->n_bases = n_emit;
                r->seq_len = n_emit + n_reads;
                tail = r->seq_len;
                cudaMemsetAsync(r->d_seq_alloc, '\n', seq_alloc, c->stream);
                cudaMemcpyAsync(r->d_rd_off + n_reads, &tail, 8, cudaMemcpyHostToDevice, c->stream);
                k_emit<<<(unsigned)n_tiles, PT_THREADS, 0, c->stream>>>(g, tile_line0, tile_emit0, kind, line_rec, n_lines,
                                                                       r->d_seq, r->d_rd_off);
                c->launches++;
            } while (0);
        }
        if (!e && n_tiles && n_reads) {
            k_names<<<grid_for(n_reads, 256), 256, 0, c->stream>>>(g, hdr_line, fastq, line_end, n_reads, r->d_rd_off,
                                                                   r->d_name_off, r->d_name_len, d_maxlen);
            c->launches++;
        }
        if (!e) e = pack_reads(c, r);
        if (!e) e = cuda_check(c, cudaMemcpyAsync(&r->max_len, d_maxlen, 4, cudaMemcpyDeviceToHost, c->stream), "maxlen d2h");
        if (!e) e = cuda_check(c, cudaStreamSynchronize(c->stream), "parse sync");
    }
    for (void *p : tmp) dfree(c, p);
    if (d_maxlen) dfree(c, d_maxlen);
    prof_end(c, TK_KID_PARSE, ev, r->text_len);
    return e;
}

}  // namespace tk
