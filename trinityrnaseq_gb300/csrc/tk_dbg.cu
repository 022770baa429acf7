// tk_dbg.cu -- per-record de Bruijn k-mer graphs of the Inchworm bundle
// (Inchworm FastaToDeBruijn --fasta bundled_iworm_contigs.fasta -K 24
// --graph_per_record, called at Trinity:2298-2302; its output is cut into one
// file per component by util/support_scripts/partition_chrysalis_graphs_n_reads.pl).
//
// Per bundle record (one component: its Inchworm contigs joined by 'X'), the
// distinct (K+1)-mers in order of first occurrence, each with the node of the
// window just before its first occurrence (-1 at a contig start or a break)
// and its number of occurrences in the record (a k-mer and its reverse
// complement are one node unless strand-specific).  Text: "Component <id>"
// then "<node>\t<prev>\t<count>\t<kmer>" per node; a record without any
// window is left out.
//
// GPU plan, all over the record-concatenated bundle read set:
//  1. one thread per position: the window starting there, cut from the 2-bit
//     codes with its validity; the valid ones compacted (key, position);
//  2. stable radix sorts by key, then by record: equal (record, key) runs
//     with ascending positions, so a run's head is the node's first occurrence
//     and its length the count; every window position is mapped to its node;
//  3. nodes radix-sorted by first position = record order, then order of first
//     occurrence; node id = rank - the record's first rank; prev through the
//     position map of the window before;
//  4. line lengths, a scan, and one thread per line writing it.
#include "tk_internal.cuh"

#include <algorithm>
#include <vector>

namespace tk {

constexpr uint32_t NO_NODE = 0xFFFFFFFFu;

__device__ __forceinline__ uint32_t dbg_dec_len(uint64_t v) {
    uint32_t n = 1;
    while (v >= 10) {
        v /= 10;
        n++;
    }
    return n;
}

__device__ __forceinline__ char *dbg_put_dec(char *o, uint64_t v) {
    const uint32_t n = dbg_dec_len(v);
    for (uint32_t i = n; i > 0; i--) {
        o[i - 1] = (char)('0' + v % 10);
        v /= 10;
    }
    return o + n;
}

// record holding position p: the largest r with rd_off[r] <= p
__device__ __forceinline__ uint32_t dbg_record_of(const uint64_t *__restrict__ rd_off, uint64_t n_rec, uint64_t p) {
    uint64_t lo = 0, hi = n_rec;
    while (hi - lo > 1) {
        const uint64_t mid = (lo + hi) >> 1;
        if (__ldg(rd_off + mid) <= p) lo = mid;
        else hi = mid;
    }
    return (uint32_t)lo;
}

// 1. window starting at p (positions p .. p+k1-1) from the code pair holding its end
template <bool CANON>
__global__ void k_dbg_windows(const uint64_t *__restrict__ codes, const uint32_t *__restrict__ inv, uint64_t n_pos,
                              int k1, uint32_t *__restrict__ valid, uint64_t *__restrict__ keys) {
    const uint64_t p = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= n_pos) return;
    const uint64_t e = p + (uint64_t)k1 - 1;
    const int64_t q = (int64_t)(e >> 5);
    const int i = (int)(e & 31);
    const uint64_t hi = __ldg(codes + q - 1), lo = __ldg(codes + q);
    const uint64_t m = ((uint64_t)__ldg(inv + q - 1) << 32) | __ldg(inv + q);
    const bool ok = ((m >> (31 - i)) & ((1ULL << k1) - 1)) == 0;
    const int s = 62 - 2 * i;
    const uint64_t fw = (s ? ((lo >> s) | (hi << (64 - s))) : lo) & ((1ULL << (2 * k1)) - 1);
    uint64_t key = fw;
    if (CANON) {
        uint64_t x = __brevll(~fw);
        x = ((x >> 1) & 0x5555555555555555ULL) | ((x & 0x5555555555555555ULL) << 1);
        const uint64_t rc = x >> (64 - 2 * k1);
        key = rc < fw ? rc : fw;
    }
    valid[p] = ok ? 1u : 0u;
    keys[p] = key;
}

__global__ void k_dbg_compact(const uint32_t *__restrict__ valid, const uint64_t *__restrict__ keys,
                              const uint64_t *__restrict__ off, uint64_t n_pos, uint64_t *__restrict__ okeys,
                              uint32_t *__restrict__ opos) {
    const uint64_t p = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= n_pos || !valid[p]) return;
    okeys[off[p]] = keys[p];
    opos[off[p]] = (uint32_t)p;
}

// record of every (key-sorted) window, as the key of the second sort; the value
// is the window's index in the key order
__global__ void k_dbg_rec_keys(const uint32_t *__restrict__ pos, uint64_t n, const uint64_t *__restrict__ rd_off,
                               uint64_t n_rec, uint64_t *__restrict__ rec, uint32_t *__restrict__ idx) {
    const uint64_t j = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= n) return;
    rec[j] = dbg_record_of(rd_off, n_rec, pos[j]);
    idx[j] = (uint32_t)j;
}

// 2. windows in (record, key, position) order: run heads, and the position map
__global__ void k_dbg_heads(const uint64_t *__restrict__ rec, const uint32_t *__restrict__ idx,
                            const uint64_t *__restrict__ keys, uint64_t n, uint32_t *__restrict__ head) {
    const uint64_t j = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= n) return;
    head[j] = (j == 0 || rec[j] != rec[j - 1] || keys[idx[j]] != keys[idx[j - 1]]) ? 1u : 0u;
}

__global__ void k_dbg_nodes(const uint32_t *__restrict__ head, const uint64_t *__restrict__ hoff,
                            const uint32_t *__restrict__ idx, const uint32_t *__restrict__ pos, uint64_t n,
                            uint64_t n_nodes, uint32_t *__restrict__ node_start, uint64_t *__restrict__ node_first,
                            uint32_t *__restrict__ node_g, uint32_t *__restrict__ pos_node) {
    const uint64_t j = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (j > n) return;
    if (j == n) {
        node_start[n_nodes] = (uint32_t)n;
        return;
    }
    const uint32_t g = (uint32_t)(hoff[j] + head[j] - 1);
    const uint32_t p = pos[idx[j]];
    if (head[j]) {
        node_start[g] = (uint32_t)j;
        node_first[g] = p;
        node_g[g] = g;
    }
    pos_node[p] = g;
}

// 3. per rank (nodes in first-position order): the rank of each node, and the
// first rank of each record that has nodes
__global__ void k_dbg_ranks(const uint64_t *__restrict__ first, const uint32_t *__restrict__ g_of, uint64_t n_nodes,
                            const uint64_t *__restrict__ rd_off, uint64_t n_rec, uint32_t *__restrict__ rank_of,
                            uint32_t *__restrict__ rec_first, unsigned long long *__restrict__ n_comp) {
    const uint64_t j = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= n_nodes) return;
    rank_of[g_of[j]] = (uint32_t)j;
    const uint32_t r = dbg_record_of(rd_off, n_rec, first[j]);
    if (j == 0 || dbg_record_of(rd_off, n_rec, first[j - 1]) != r) {
        rec_first[r] = (uint32_t)j;
        atomicAdd(n_comp, 1ULL);
    }
}

struct DbgLine {
    uint32_t id;       // node id in its record
    int32_t prev;      // -1: none
    uint32_t count;
    uint32_t rec;      // record index; header line before the record's first node
};

__global__ void k_dbg_lines(const uint64_t *__restrict__ first, const uint32_t *__restrict__ g_of, uint64_t n_nodes,
                            const uint64_t *__restrict__ rd_off, uint64_t n_rec,
                            const uint32_t *__restrict__ rank_of, const uint32_t *__restrict__ rec_first,
                            const uint32_t *__restrict__ node_start, const uint32_t *__restrict__ pos_node,
                            const uint64_t *__restrict__ comp, int k1, DbgLine *__restrict__ line,
                            uint64_t *__restrict__ len) {
    const uint64_t j = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= n_nodes) return;
    const uint64_t p = first[j];
    const uint32_t g = g_of[j];
    const uint32_t r = dbg_record_of(rd_off, n_rec, p);
    const uint32_t r0 = rec_first[r];
    DbgLine L;
    L.id = (uint32_t)j - r0;
    L.count = node_start[g + 1] - node_start[g];
    L.rec = r;
    // the window just before the first occurrence, when it is a valid window
    // (it then lies in the same contig of the same record)
    const uint32_t pn = p > 0 ? pos_node[p - 1] : NO_NODE;
    L.prev = pn == NO_NODE ? -1 : (int32_t)(rank_of[pn] - r0);
    line[j] = L;
    uint64_t n = dbg_dec_len(L.id) + 1 + (L.prev < 0 ? 2 : dbg_dec_len((uint32_t)L.prev)) + 1 + dbg_dec_len(L.count) + 1 +
                 (uint64_t)k1 + 1;
    if (L.id == 0) n += 10 + dbg_dec_len(comp[r]) + 1;   // "Component " id "\n"
    len[j] = n;
}

// 4. one thread per node line
__global__ void k_dbg_write(const DbgLine *__restrict__ line, const uint64_t *__restrict__ first,
                            const uint64_t *__restrict__ off, uint64_t n_nodes, const uint64_t *__restrict__ comp,
                            const uint8_t *__restrict__ seq, int k1, char *__restrict__ out) {
    const uint64_t j = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= n_nodes) return;
    const DbgLine L = line[j];
    char *o = out + off[j];
    if (L.id == 0) {
        const char hdr[] = "Component ";
        for (int i = 0; i < 10; i++) o[i] = hdr[i];
        o = dbg_put_dec(o + 10, comp[L.rec]);
        *o++ = '\n';
    }
    o = dbg_put_dec(o, L.id);
    *o++ = '\t';
    if (L.prev < 0) {
        *o++ = '-';
        *o++ = '1';
    } else {
        o = dbg_put_dec(o, (uint32_t)L.prev);
    }
    *o++ = '\t';
    o = dbg_put_dec(o, L.count);
    *o++ = '\t';
    const uint8_t *s = seq + first[j];
    for (int i = 0; i < k1; i++) o[i] = (char)s[i];
    o[k1] = '\n';
}

static unsigned dbg_grid(uint64_t n, int threads) { return (unsigned)std::max<uint64_t>(1, (n + threads - 1) / threads); }

// Device allocations released on every path out of dbg_build.
struct DbgScratch {
    tk_ctx *c;
    std::vector<void *> p;
    explicit DbgScratch(tk_ctx *ctx) : c(ctx) {}
    int get(void **out, uint64_t bytes, const char *what) {
        int e = dmalloc(c, out, bytes ? bytes : 8, what);
        if (!e) p.push_back(*out);
        return e;
    }
    ~DbgScratch() {
        for (void *q : p) dfree(c, q);
    }
};

int dbg_build(tk_dbg *g, const tk_reads *b, const std::vector<uint64_t> &comp_id) {
    tk_ctx *c = g->ctx;
    const int k1 = g->k + 1;
    const uint64_t n_rec = b->n_reads, n_pos = b->seq_len;
    g->n_nodes = 0;
    g->n_components = 0;
    g->text_len = 0;
    if (n_rec == 0 || n_pos < (uint64_t)k1) return TK_OK;
    DbgScratch sc(c);
    cudaEvent_t ev;
    prof_begin(c, TK_KID_DBG, &ev);
    // 1. windows, compacted
    uint32_t *valid = nullptr;
    uint64_t *keys = nullptr, *off = nullptr;
    TK_TRY(sc.get((void **)&valid, n_pos * 4, "window flags"));
    TK_TRY(sc.get((void **)&keys, n_pos * 8, "window keys"));
    TK_TRY(sc.get((void **)&off, (n_pos + 1) * 8, "window offsets"));
    const uint64_t n_win_pos = n_pos - (uint64_t)k1 + 1;   // window starts whose window ends inside the set
    if (g->strand)
        k_dbg_windows<false><<<dbg_grid(n_win_pos, 256), 256, 0, c->stream>>>(b->d_codes, b->d_inv, n_win_pos, k1,
                                                                             valid, keys);
    else
        k_dbg_windows<true><<<dbg_grid(n_win_pos, 256), 256, 0, c->stream>>>(b->d_codes, b->d_inv, n_win_pos, k1,
                                                                            valid, keys);
    c->launches++;
    TK_TRY(check_launch(c, "de Bruijn windows"));
    uint64_t M = 0;
    TK_TRY(scan_excl_u32_to_u64(c, valid, off, n_win_pos, &M));
    if (M == 0) {
        prof_end(c, TK_KID_DBG, ev, 0);
        return TK_OK;
    }
    if (M >= NO_NODE) return set_err(c, TK_E_RANGE, "FastaToDeBruijn: more than 2^32 - 1 windows in one bundle");
    uint64_t *wk = nullptr, *wk2 = nullptr;
    uint32_t *wp = nullptr, *wp2 = nullptr;
    TK_TRY(sc.get((void **)&wk, M * 8, "windows"));
    TK_TRY(sc.get((void **)&wk2, M * 8, "windows (sort)"));
    TK_TRY(sc.get((void **)&wp, M * 4, "window positions"));
    TK_TRY(sc.get((void **)&wp2, M * 4, "window positions (sort)"));
    k_dbg_compact<<<dbg_grid(n_win_pos, 256), 256, 0, c->stream>>>(valid, keys, off, n_win_pos, wk, wp);
    c->launches++;
    TK_TRY(check_launch(c, "de Bruijn compact"));
    // 2. by key, then by record (both stable: positions stay ascending)
    bool in_tmp = false;
    TK_TRY(radix_sort_pairs(c, wk, wp, M, 2 * k1, wk2, wp2, &in_tmp));
    uint64_t *sk = in_tmp ? wk2 : wk;
    uint32_t *sp = in_tmp ? wp2 : wp;
    uint64_t *rec = keys, *rec2 = off;   // reuse: n_pos >= M
    uint32_t *idx = valid, *idx2 = in_tmp ? wp : wp2;
    k_dbg_rec_keys<<<dbg_grid(M, 256), 256, 0, c->stream>>>(sp, M, b->d_rd_off, n_rec, rec, idx);
    c->launches++;
    TK_TRY(check_launch(c, "de Bruijn records"));
    int rbits = 1;
    while ((1ULL << rbits) < n_rec) rbits++;
    TK_TRY(radix_sort_pairs(c, rec, idx, M, rbits, rec2, idx2, &in_tmp));
    const uint64_t *srec = in_tmp ? rec2 : rec;
    const uint32_t *sidx = in_tmp ? idx2 : idx;
    uint32_t *head = nullptr;
    uint64_t *hoff = nullptr;
    TK_TRY(sc.get((void **)&head, M * 4, "node heads"));
    TK_TRY(sc.get((void **)&hoff, (M + 1) * 8, "node offsets"));
    k_dbg_heads<<<dbg_grid(M, 256), 256, 0, c->stream>>>(srec, sidx, sk, M, head);
    c->launches++;
    TK_TRY(check_launch(c, "de Bruijn heads"));
    uint64_t G = 0;
    TK_TRY(scan_excl_u32_to_u64(c, head, hoff, M, &G));
    uint32_t *node_start = nullptr, *node_g = nullptr, *node_g2 = nullptr, *pos_node = nullptr;
    uint64_t *node_first = nullptr, *node_first2 = nullptr;
    TK_TRY(sc.get((void **)&node_start, (G + 1) * 4, "node starts"));
    TK_TRY(sc.get((void **)&node_first, G * 8, "node first positions"));
    TK_TRY(sc.get((void **)&node_first2, G * 8, "node first positions (sort)"));
    TK_TRY(sc.get((void **)&node_g, G * 4, "node ids"));
    TK_TRY(sc.get((void **)&node_g2, G * 4, "node ids (sort)"));
    TK_TRY(sc.get((void **)&pos_node, n_pos * 4, "position map"));
    TK_CUDA(c, cudaMemsetAsync(pos_node, 0xFF, n_pos * 4, c->stream));
    k_dbg_nodes<<<dbg_grid(M + 1, 256), 256, 0, c->stream>>>(head, hoff, sidx, sp, M, G, node_start, node_first, node_g,
                                                            pos_node);
    c->launches++;
    TK_TRY(check_launch(c, "de Bruijn nodes"));
    // 3. nodes in first-position order
    int pbits = 1;
    while ((1ULL << pbits) < n_pos) pbits++;
    TK_TRY(radix_sort_pairs(c, node_first, node_g, G, pbits, node_first2, node_g2, &in_tmp));
    const uint64_t *ofirst = in_tmp ? node_first2 : node_first;
    const uint32_t *og = in_tmp ? node_g2 : node_g;
    uint32_t *rank_of = nullptr, *rec_first = nullptr;
    uint64_t *d_comp = nullptr, *len = nullptr, *loff = nullptr;
    unsigned long long *d_ncomp = nullptr;
    DbgLine *line = nullptr;
    TK_TRY(sc.get((void **)&d_ncomp, 8, "component count"));
    TK_CUDA(c, cudaMemsetAsync(d_ncomp, 0, 8, c->stream));
    TK_TRY(sc.get((void **)&rank_of, G * 4, "node ranks"));
    TK_TRY(sc.get((void **)&rec_first, n_rec * 4, "record first ranks"));
    TK_TRY(sc.get((void **)&d_comp, n_rec * 8, "component ids"));
    TK_TRY(sc.get((void **)&line, G * sizeof(DbgLine), "node lines"));
    TK_TRY(sc.get((void **)&len, G * 8, "line lengths"));
    TK_TRY(sc.get((void **)&loff, (G + 1) * 8, "line offsets"));
    TK_CUDA(c, cudaMemcpyAsync(d_comp, comp_id.data(), n_rec * 8, cudaMemcpyHostToDevice, c->stream));
    k_dbg_ranks<<<dbg_grid(G, 256), 256, 0, c->stream>>>(ofirst, og, G, b->d_rd_off, n_rec, rank_of, rec_first,
                                                         d_ncomp);
    c->launches++;
    TK_TRY(check_launch(c, "de Bruijn ranks"));
    k_dbg_lines<<<dbg_grid(G, 256), 256, 0, c->stream>>>(ofirst, og, G, b->d_rd_off, n_rec, rank_of, rec_first,
                                                         node_start, pos_node, d_comp, k1, line, len);
    c->launches++;
    TK_TRY(check_launch(c, "de Bruijn lines"));
    uint64_t total = 0;
    TK_TRY(scan_excl_u64(c, len, loff, G, &total));
    char *text = nullptr;
    TK_TRY(dmalloc(c, (void **)&text, total + 1, "de Bruijn text"));
    k_dbg_write<<<dbg_grid(G, 256), 256, 0, c->stream>>>(line, ofirst, loff, G, d_comp, b->d_seq, k1, text);
    c->launches++;
    int e = check_launch(c, "de Bruijn text");
    if (e) {
        dfree(c, text);
        return e;
    }
    unsigned long long n_comp = 0;
    e = cuda_check(c, cudaMemcpyAsync(&n_comp, d_ncomp, 8, cudaMemcpyDeviceToHost, c->stream), "component count");
    if (!e) e = cuda_check(c, cudaStreamSynchronize(c->stream), "de Bruijn sync");
    if (e) {
        dfree(c, text);
        return e;
    }
    prof_end(c, TK_KID_DBG, ev, M);
    g->d_text = text;
    g->text_len = total;
    g->n_nodes = G;
    g->n_windows = M;
    g->n_components = n_comp;
    return TK_OK;
}

}  // namespace tk
