// tk_internal.cuh -- shared definitions of the GB300 k-mer library.
//
// Device data layout (all in HBM, owned by the library):
//  * read batch   : `seq`  = every read's bases upper-cased, each read followed
//                   by one '\n' separator, 64 bytes of '\n' padding on both
//                   sides; `rd_off[r]` = first base of read r (n+1 entries);
//                   `name_off/name_len` = accession (first header token) in
//                   the device copy of the input text.  The same positions
//                   as 2-bit codes: `codes[j]` holds positions 32j..32j+31
//                   (A0 C1 G2 T3, first position in the top bits) and bit
//                   31-i of `inv[j]` is set when position 32j+i is not
//                   A/C/G/T; word -1 exists (all positions invalid).
//  * k-mer table  : open addressing, linear probing, 16-byte slots
//                   {u64 key; u32 value; u32 pad} so a probe touches one
//                   32-byte DRAM sector; capacity a power of two; empty key
//                   = ~0 (k <= 31 keeps every real key below it).
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>
#include <atomic>
#include <string>
#include <unordered_map>
#include <utility>
#include <vector>

#include "../../include/trinkmer.h"

namespace tk {

constexpr uint64_t EMPTY_KEY = ~0ULL;
constexpr uint32_t PAD_VAL = 0xFFFFFFFFu;
constexpr int SEQ_PAD = 64;          // '\n' bytes before and after `seq`
constexpr int MAX_K = 31;

struct __align__(16) Slot {
    unsigned long long key;
    unsigned int val;
    unsigned int pad;
};

// Capacity = 2^(pbits + lbits) slots in 2^pbits partitions of 2^lbits slots.
// A key's partition is the top pbits of its hash and its home slot inside the
// partition the low lbits; probing wraps inside the partition.  With
// partitions of at most 32 MB, the counting pass that inserts keys in
// partition order works on an L2-resident slice at a time.
struct DevTable {
    Slot *slots;
    uint64_t lmask;     // 2^lbits - 1
    int lbits;
    int pbits;
};

constexpr int MAX_LBITS = 21;        // 2M slots = 32 MB per partition
constexpr int BUCKET_BITS = 10;      // hash buckets of the partitioned count (>= pbits)

// device-side error words (set by kernels, read by the host after a launch)
enum DevErr : uint32_t {
    DE_PARSE = 0,       // [0] parse error flag, [1] first bad line (low 32 bits)
    DE_OVERFLOW = 2,    // [2] overflow list overrun
    DE_WS = 3,          // [3] parser: whitespace seen inside a sequence line
    DE_COUNT = 8
};

__host__ __device__ inline uint64_t mix64(uint64_t x) {
    x ^= x >> 33; x *= 0xff51afd7ed558ccdULL;
    x ^= x >> 33; x *= 0xc4ceb9fe1a85ec53ULL;
    x ^= x >> 33; return x;
}

// A/C/G/T -> 0..3 for upper-case input (`seq` is upper-cased by the parser);
// anything else -> 4.  ((c>>1)&3) maps A,C,G,T to 0,1,3,2; the xor swaps G,T.
__device__ __forceinline__ uint32_t base_code(uint32_t c) {
    uint32_t d = c - 0x41u;
    bool ok = d < 20u && ((0x80045u >> d) & 1u);
    uint32_t b = (c >> 1) & 3u;
    b ^= b >> 1;
    return ok ? b : 4u;
}

__device__ __forceinline__ unsigned lane_id() { return threadIdx.x & 31u; }

// ------------------------------------------------------------------ table ops

__host__ __device__ __forceinline__ uint64_t tbl_home(const DevTable &t, uint64_t h) {
    uint64_t part = t.pbits ? (h >> (64 - t.pbits)) : 0;
    return (part << t.lbits) | (h & t.lmask);
}

__host__ __device__ __forceinline__ uint64_t tbl_next(const DevTable &t, uint64_t s) {
    return (s & ~t.lmask) | ((s + 1) & t.lmask);
}

// The probe is an atomicCAS(EMPTY -> key) on the slot's key: it claims an empty
// slot and returns the resident key otherwise.  On GB300 a CAS probe followed
// by red.add runs ~1.3x faster than a load probe followed by red.add on an
// L2-resident table, and 2-8x faster when the table is not L2-resident (the
// load + red pair to one line thrashes).
__device__ __forceinline__ unsigned long long tbl_claim(Slot *slot, uint64_t key) {
    unsigned long long cur = atomicCAS(&slot->key, EMPTY_KEY, (unsigned long long)key);
    return cur == EMPTY_KEY ? (unsigned long long)key : cur;
}

// Adds `inc` to key's value, inserting the key if absent.  Returns false after
// max_probes slots without finding the key or a free slot.
__device__ __forceinline__ bool tbl_add(DevTable t, uint64_t key, uint32_t inc, int max_probes) {
    uint64_t s = tbl_home(t, mix64(key));
    for (int i = 0; i < max_probes; i++) {
        if (tbl_claim(&t.slots[s], key) == key) {
            atomicAdd(&t.slots[s].val, inc);
            return true;
        }
        s = tbl_next(t, s);
    }
    return false;
}

// Keeps the minimum value per key (ReadsToTranscripts ownership).
__device__ __forceinline__ bool tbl_min(DevTable t, uint64_t key, uint32_t v, int max_probes) {
    uint64_t s = tbl_home(t, mix64(key));
    for (int i = 0; i < max_probes; i++) {
        unsigned long long cur = tbl_claim(&t.slots[s], key);
        if (cur == key) {
            atomicMin(&t.slots[s].val, v);
            return true;
        }
        s = tbl_next(t, s);
    }
    return false;
}

__device__ __forceinline__ uint32_t tbl_get(DevTable t, uint64_t key, uint32_t miss) {
    uint64_t s = tbl_home(t, mix64(key));
    for (uint64_t i = 0; i <= t.lmask; i++) {
        ulonglong2 v = __ldcg(reinterpret_cast<const ulonglong2 *>(&t.slots[s]));
        if (v.x == key) return (uint32_t)v.y;
        if (v.x == EMPTY_KEY) return miss;
        s = tbl_next(t, s);
    }
    return miss;
}

// one-slot-pair table every lookup misses in (an empty catalogue)
__host__ __device__ __forceinline__ DevTable tbl_empty(Slot *two_slots) {
    DevTable t;
    t.slots = two_slots;
    t.lmask = 1;
    t.lbits = 1;
    t.pbits = 0;
    return t;
}

// ------------------------------------------------------------------ warp scans

template <typename T>
__device__ __forceinline__ T warp_incl_scan(T v) {
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        T n = __shfl_up_sync(0xffffffffu, v, o);
        if ((int)lane_id() >= o) v += n;
    }
    return v;
}

template <typename T>
__device__ __forceinline__ T warp_sum(T v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}

// Block-wide exclusive scan; `sm` needs blockDim.x/32 + 1 entries.  Returns the
// thread's exclusive prefix; *total receives the block total.
template <typename T>
__device__ __forceinline__ T block_excl_scan(T v, T *sm, T *total) {
    const unsigned lane = lane_id(), warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
    T inc = warp_incl_scan(v);
    if (lane == 31) sm[warp] = inc;
    __syncthreads();
    if (warp == 0) {
        T w = lane < nw ? sm[lane] : T(0);
        T wi = warp_incl_scan(w);
        if (lane < nw) sm[lane] = wi - w;
        if (lane == nw - 1) sm[nw] = wi;
    }
    __syncthreads();
    T r = sm[warp] + inc - v;
    *total = sm[nw];
    __syncthreads();
    return r;
}

}  // namespace tk

// ------------------------------------------------------------------ host side

struct tk_prof_rec {
    cudaEvent_t a, b;
    int kid;
    uint64_t units;
    uint64_t launches;   // kernels launched between the two events
};

struct tk_ctx {
    int device = 0;
    cudaStream_t stream = nullptr;
    bool own_stream = false;
    // host <-> device copies that overlap the work on `stream` (created on
    // first use; tk_ctx_synchronize waits for both streams)
    cudaStream_t copy_stream = nullptr;
    uint32_t *d_err = nullptr;             // tk::DE_COUNT words
    std::string last_error;
    // profiling (CUDA events on `stream` around the hot kernels)
    bool prof = false;
    std::vector<tk_prof_rec> pending;
    std::vector<cudaEvent_t> free_events;
    double prof_ms[TK_KID_NUM] = {0};
    uint64_t prof_launches[TK_KID_NUM] = {0};
    uint64_t prof_units[TK_KID_NUM] = {0};
    uint64_t launches = 0;                  // every kernel launched by the library
    uint64_t prof_open[TK_KID_NUM] = {0};   // `launches` when each class's bracket opened
    // blocks of >= 256 MB: cudaMalloc'd once and kept for reuse (see dmalloc)
    std::vector<std::pair<void *, size_t>> big_free;
    std::unordered_map<void *, size_t> big_used;
    int max_probes = 4096;
    int sm_count = 152;
    // the batched-bins fill + count graph, updated in place for each batch
    // (tk_bins.cu) and instantiated again only when an update is refused
    cudaGraphExec_t bins_exec = nullptr;
    // read sets, tables and bundles alive on this context; tk_ctx_destroy
    // defers the release until the last of them is freed
    std::atomic<int> live{0};
    std::atomic<bool> closing{false};
};

struct tk_reads {
    tk_ctx *ctx = nullptr;
    int format = 0;                         // TK_FMT_FASTA / TK_FMT_FASTQ
    uint64_t n_reads = 0;
    uint64_t n_bases = 0;                   // bases over all reads
    uint64_t seq_len = 0;                   // bytes of seq incl. separators
    uint32_t max_len = 0;
    char *d_text = nullptr;                 // device copy of the input text
    uint64_t text_len = 0;
    bool own_text = false;
    uint8_t *d_seq_alloc = nullptr;
    uint8_t *d_seq = nullptr;               // = d_seq_alloc + SEQ_PAD
    uint64_t *d_rd_off = nullptr;           // n_reads + 1
    uint64_t *d_name_off = nullptr;         // n_reads
    uint32_t *d_name_len = nullptr;         // n_reads
    char *d_fasta = nullptr;                // last FASTA conversion (tk_reads_to_fasta)
    uint64_t fasta_len = 0;
    int fasta_append = 0, fasta_flags = -1;
    uint64_t *d_pack_alloc = nullptr;       // codes and inv, one allocation
    const uint64_t *d_codes = nullptr;      // word 0 of the 2-bit codes (word -1 exists)
    const uint32_t *d_inv = nullptr;        // word 0 of the invalid-position bits (word -1 exists)
};

struct tk_table {
    tk_ctx *ctx = nullptr;
    int k = 25;
    int canonical = 1;
    tk::DevTable t{nullptr, 0};
    uint64_t capacity = 0;
    uint64_t distinct = 0;                  // valid after tk_table_finalize-type queries
    uint64_t total = 0;                     // k-mer occurrences added
    bool distinct_valid = true;
    uint64_t *d_ovf = nullptr;              // overflow key list
    uint64_t ovf_cap = 0;
    unsigned long long *d_counters = nullptr;  // [0] overflow n, [1] windows added
    uint32_t *d_hll = nullptr;              // HLL registers
    double max_load = 0.6;
    bool fresh = false;                     // slots not yet written (see table_alloc_geom)
    // last formatted dump (valid until the table changes)
    char *d_dump = nullptr;
    cudaEvent_t dump_copy_done = nullptr;   // an asynchronous host copy of d_dump in flight
    uint64_t dump_len = 0;
    uint32_t dump_min = 0;
    bool dump_valid = false;
    // coverage cache (tk_cov.cu): the k-mers with the highest counts in an
    // L2-sized table, built on the first coverage pass after a change
    uint64_t *d_hot = nullptr;
    uint64_t hot_bytes = 0;
    bool hot_valid = false;
};

struct tk_r2t {
    tk_ctx *ctx = nullptr;
    int k = 25;
    int strand = 0;
    tk_table *table = nullptr;              // key -> bundle record index
    uint64_t n_records = 0;
    std::vector<uint64_t> comp_id;          // per bundle record
};

// per-record de Bruijn k-mer graphs of a bundle (tk_dbg.cu)
struct tk_dbg {
    tk_ctx *ctx = nullptr;
    int k = 24;                             // -K: node lines are (k+1)-mers
    int strand = 0;
    char *d_text = nullptr;
    uint64_t text_len = 0;
    uint64_t n_records = 0, n_components = 0, n_nodes = 0, n_windows = 0;
};

namespace tk {
// One read's coverage statistics as the stats tables carry them: the median,
// mean and stdev printed "%u", "%g", "%g", and the numbers Perl reads back.
struct NormVal {
    double mean, sd;        // the values of the "%g" texts
    uint32_t med;
    uint32_t gmean, gsd;    // their 6 significant digits (0 for a zero)
    int8_t xmean, xsd;      // their decimal exponents
    uint8_t sfx_len;        // length of "\t%u\t%g\t%g"
    uint8_t pad;
};

// One side's reads (from one or more read sets) in the order of its sorted
// stats table.
struct NormSide {
    uint64_t n = 0;
    uint64_t *addr = nullptr;       // read order: device address of each name
    uint32_t *nlen = nullptr;       // read order: name length
    NormVal *val = nullptr;         // read order
    uint32_t *perm = nullptr;       // sorted position -> read
    uint64_t *h0 = nullptr, *h1 = nullptr, *off = nullptr;   // sorted: first 16 name bytes, name offset
    uint32_t *len = nullptr, *core = nullptr;                 // sorted: name length, without "/<digit>"
};
}  // namespace tk

struct tk_norm {
    tk_ctx *ctx = nullptr;
    bool pairs = false;
    int max_cov = 0, min_cov = 0, max_cv = 0;
    tk::NormSide side[2];
    uint64_t n_rows = 0;
    uint32_t *row_l = nullptr, *row_r = nullptr;   // pairs: sorted positions of each merged row
    uint64_t *row_n = nullptr;                     // pairs: 10 x the three "%.1f" averages per row
    uint64_t *acc_off = nullptr;                   // n_rows + 1: each row's line in d_accs (empty if not kept)
    char *d_accs = nullptr;
    uint64_t accs_len = 0;
    tk_norm_counts counts{};
    char *d_table = nullptr;
    uint64_t table_len = 0;
    char *d_ext = nullptr;                         // last extraction
    uint64_t ext_len = 0;
    cudaEvent_t ext_copy_done = nullptr;           // an asynchronous host copy of d_ext in flight
    std::vector<std::pair<char *, cudaEvent_t>> ext_retired;   // earlier extractions whose host copy may still run
    uint32_t *d_hash = nullptr;                    // selected names: row index per slot, ~0 empty
    uint8_t *d_keydup = nullptr;                   // per row: its name is another row's, or empty
    uint64_t hash_mask = 0;
    uint64_t n_keys = 0;
};

// host helpers shared by the translation units
namespace tk {
int set_err(tk_ctx *c, int code, const std::string &msg);
int cuda_check(tk_ctx *c, cudaError_t e, const char *what);
int dmalloc(tk_ctx *c, void **p, size_t bytes, const char *what);
uint64_t ctx_cached_bytes(const tk_ctx *c);   // freed blocks the context keeps for reuse
void dfree(tk_ctx *c, void *p);
void prof_begin(tk_ctx *c, int kid, cudaEvent_t *ev);
void prof_end(tk_ctx *c, int kid, cudaEvent_t ev, uint64_t units);
void prof_add_units(tk_ctx *c, int kid, uint64_t units);
int check_launch(tk_ctx *c, const char *what);
int scan_excl_u64(tk_ctx *c, const uint64_t *in, uint64_t *out, uint64_t n, uint64_t *total_host);
int scan_excl_u32_to_u64(tk_ctx *c, const uint32_t *in, uint64_t *out, uint64_t n, uint64_t *total_host);
// K4 formatting of sorted (key, count) pairs (tk_table.cu)
int format_dump(tk_ctx *c, const uint64_t *keys, const uint32_t *cnt, uint64_t n, int k, char **text, uint64_t *len,
                uint64_t **offs_out = nullptr);
int radix_sort_pairs(tk_ctx *c, uint64_t *keys, uint32_t *vals, uint64_t n, int bits,
                     uint64_t *tmp_keys, uint32_t *tmp_vals, bool *result_in_tmp, int first_bit = 0);
int table_alloc(tk_table *t, uint64_t capacity);
int table_alloc_init(tk_table *t, uint64_t capacity, uint32_t init_val);
int table_rehash(tk_table *t, uint64_t new_capacity);
int table_count_seq(tk_table *t, const tk_reads *r);
int reads_fasta(tk_reads *r, int append, int flags, char **d_text, uint64_t *text_len);
int table_count_many(tk_table *t, const tk_reads *const *sets, int nsets);
// One read set's k-mers after counting pass 1: bucket-major over the set's
// own columns (one per block of its grid); region (bucket, column) starts at
// offs[bucket * cols + column] and is padded to whole 32-byte sectors.
struct BucketKeys {
    uint64_t *keys = nullptr;   // nullptr: the set has no windows
    uint64_t *offs = nullptr;   // NBUCKETS * cols + 1
    uint64_t cols = 0;
};
// Counting in two steps (tk_table.cu): table_count_begin, then pass 1 per
// read set as each becomes ready (at most 64 sets), then pass 2 over all of
// them (which frees their key buffers).
int table_count_begin(tk_table *t);
int table_bucket_pass(tk_table *t, const tk_reads *r, BucketKeys *out);
void table_bucket_free(tk_table *t, BucketKeys *bk);
int table_count_buckets(tk_table *t, std::vector<BucketKeys> &bk);
constexpr uint32_t COUNT_MAX_SETS = 64;
int norm_select(tk_norm *nm, const tk_reads *const *const sets[2], const uint32_t nsets[2],
                const uint32_t *const med[2], const float *const mean[2], const float *const sd[2], int where);
int norm_table(tk_norm *nm);
int norm_extract(tk_norm *nm, const tk_reads *const *sets, uint32_t nsets);
void norm_release(tk_norm *nm);
int dbg_build(tk_dbg *g, const tk_reads *b, const std::vector<uint64_t> &comp_id);
}  // namespace tk

#define TK_TRY(x) do { int _e = (x); if (_e) return _e; } while (0)
#define TK_CUDA(c, x) do { cudaError_t _e = (x); if (_e != cudaSuccess) return tk::cuda_check((c), _e, #x); } while (0)
