/*
 * oracle.c -- CPU restatement of Trinity's k-mer hot path (TEST INFRASTRUCTURE).
 *
 * Only the test suite, __graft_entry__.smoke() and bench.py's CPU-baseline /
 * reference arm load this file's library, and only as the checker or the
 * timed CPU reference.  The shipped GPU library never touches it.
 *
 * What it restates (reference file:line of each behaviour):
 *  - record parsing: PerlLib/Fasta_reader.pm:45-73 (records split at '>' lines,
 *    sequence = lines joined with all whitespace removed) and Sequence->new,
 *    PerlLib/Fasta_reader.pm:107-118 (accession = first whitespace token);
 *    FASTQ 4-line records as util/support_scripts/fastQ_to_fastA.pl:80-106.
 *  - k-mer windows: every length-k substring, util/misc/print_kmers.pl:19-27;
 *    a window holding a base other than A/C/G/T (any case) is not a k-mer
 *    (jellyfish 2.3.0, called at Trinity:2612-2619).
 *  - canonical counting: util/misc/kmer_counter.pl:26-37 counts a window and
 *    its reverse complement in DS mode; jellyfish --canonical keeps one key, the
 *    lexicographically smaller strand (A<C<G<T), which is the same count for
 *    odd k.
 *  - dump ">COUNT\nKMER\n" with -L: Trinity:2625, util/insilico_read_normalization.pl:641.
 *  - histo "<count> <n>" lines, overflow bin high+1:
 *    util/misc/insilico_norm_kmer_hists/kmer_histo.all.txt:1-10001.
 *  - coverage stats: util/insilico_read_normalization.pl:837-846 (tool call),
 *    Changelog.txt:536-538 (a k-mer missing from the -L 2 catalogue counts 1,
 *    unsigned counters), Changelog.txt:423-424 (an empty read is a row, not EOF);
 *    columns acc/median_cov/mean_cov/stdev consumed by name at
 *    util/support_scripts/nbkc_normalize.pl:85-97 and
 *    nbkc_merge_left_right_stats.pl:95-103, acc first for `sort -k1,1`
 *    (util/insilico_read_normalization.pl:874).
 *  - ReadsToTranscripts: Trinity:2237-2251 (tool call), Changelog.txt:467
 *    (reads upper-cased), Changelog.txt:870-873 (-p min percent of a read's
 *    k-mers), bundle format util/support_scripts/add_LR_reads_to_iworm_bundle.pl:19-47,
 *    output columns Trinity:2474 and partition_chrysalis_graphs_n_reads.pl:103.
 *
 * Documented decisions (not pinned by any file of the reference tree):
 *  D1 median of n values = the element at index n/2 of the ascending sort.
 *  D2 mean = (float)((double)sum / n); stdev = population standard deviation,
 *     (float)sqrt(((double)hi * 2^64 + (double)lo) / ((double)n * n)) where
 *     hi:lo = n*sum(v^2) - sum(v)^2 computed exactly in 128-bit integers.
 *     Both printed with C's %g (the default precision of a C++ ostream).
 *  D3 windows holding a non-ACGT base are skipped by the statistics; a read with
 *     no valid window prints median 0, mean 0, stdev 0.
 *  D4 ReadsToTranscripts: a k-mer found in several bundle records belongs to the
 *     first record holding it; a read votes once per valid window for the record
 *     owning that window's k-mer; the winner is the record with most votes,
 *     ties to the earlier record; pct = floor(100 * votes / (L - k + 1)); a read
 *     with no vote, shorter than k, or pct < -p is not written.
 *  D5 the component id is the integer after "s_" in the bundle header; a header
 *     without it takes its record ordinal.
 *  D8 FastaToDeBruijn --graph_per_record -K K (Trinity:2298-2302): per bundle
 *     record with at least one window of K+1 A/C/G/T bases, a line
 *     "Component <id>" (id as D5) and then one line per distinct (K+1)-mer of
 *     the record (canonical unless --SS), in order of first occurrence:
 *     "<node>\t<prev>\t<count>\t<kmer>" -- node = 0, 1, ... in that order,
 *     prev = the node of the window just before the first occurrence (-1 when
 *     that window is not a valid (K+1)-mer: a record or contig start, an 'X'
 *     join or another non-ACGT byte), count = occurrences in the record (both
 *     strands unless --SS), kmer = the first occurrence as written, upper case.
 *     Pinned: the "Component <id>" line starting each record and one line per
 *     k-mer (partition_chrysalis_graphs_n_reads.pl:197-223 counts the lines
 *     after each header as the component's k-mers, num_kmers + 24 vs the
 *     minimum contig length at :76); a component without k-mers is left out
 *     because that reader stops at the first empty one.  The node line's
 *     columns are this restatement's choice (the consumers QuantifyGraph and
 *     Butterfly are not in the reference checkout).
 */
#include "oracle.h"

#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <math.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#define ORC_E_INVAL (-1)
#define ORC_E_OOM (-3)
#define ORC_E_PARSE (-4)
#define ORC_E_FULL (-5)

static const uint64_t EMPTY = ~0ULL;

/* ---------------------------------------------------------------- parsing */

typedef struct {
    size_t n, cap;
    size_t *acc_off;   /* accession start in the input text */
    uint32_t *acc_len;
    size_t *seq_off;   /* sequence start in seqbuf */
    uint32_t *seq_len;
    char *seqbuf;
    size_t seqlen, seqcap;
} recs_t;

static int is_ws(unsigned char c) {
    return c == ' ' || c == '\t' || c == '\n' || c == '\r' || c == '\f' || c == '\v';
}

static void recs_free(recs_t *r) {
    free(r->acc_off); free(r->acc_len); free(r->seq_off); free(r->seq_len);
    free(r->seqbuf);
    memset(r, 0, sizeof(*r));
}

static int recs_push(recs_t *r, size_t acc_off, uint32_t acc_len) {
    if (r->n == r->cap) {
        size_t nc = r->cap ? r->cap * 2 : 1024;
        size_t *a = realloc(r->acc_off, nc * sizeof(size_t));
        uint32_t *b = realloc(r->acc_len, nc * sizeof(uint32_t));
        size_t *c = realloc(r->seq_off, nc * sizeof(size_t));
        uint32_t *d = realloc(r->seq_len, nc * sizeof(uint32_t));
        if (!a || !b || !c || !d) return ORC_E_OOM;
        r->acc_off = a; r->acc_len = b; r->seq_off = c; r->seq_len = d;
        r->cap = nc;
    }
    r->acc_off[r->n] = acc_off;
    r->acc_len[r->n] = acc_len;
    r->seq_off[r->n] = r->seqlen;
    r->seq_len[r->n] = 0;
    r->n++;
    return 0;
}

static int recs_append(recs_t *r, const char *p, size_t len) {
    if (r->seqlen + len + 1 > r->seqcap) {
        size_t nc = r->seqcap ? r->seqcap : 1 << 20;
        while (nc < r->seqlen + len + 1) nc *= 2;
        char *b = realloc(r->seqbuf, nc);
        if (!b) return ORC_E_OOM;
        r->seqbuf = b; r->seqcap = nc;
    }
    for (size_t i = 0; i < len; i++) {
        unsigned char c = (unsigned char)p[i];
        if (!is_ws(c)) r->seqbuf[r->seqlen++] = (char)c;
    }
    r->seq_len[r->n - 1] = (uint32_t)(r->seqlen - r->seq_off[r->n - 1]);
    return 0;
}

/* first whitespace-delimited token of the header line starting at h */
static uint32_t token_len(const char *h, const char *end) {
    const char *q = h;
    while (q < end && !is_ws((unsigned char)*q)) q++;
    return (uint32_t)(q - h);
}

static int parse_records(const char *text, size_t len, recs_t *r) {
    memset(r, 0, sizeof(*r));
    size_t i = 0;
    while (i < len && is_ws((unsigned char)text[i])) i++;
    if (i == len) return 0;
    const char *end = text + len;
    if (text[i] == '@') {
        /* FASTQ: header, sequence, '+' line, quality */
        size_t line = 0;
        size_t pos = i;
        while (pos < len) {
            const char *ls = text + pos;
            const char *nl = memchr(ls, '\n', (size_t)(end - ls));
            const char *le = nl ? nl : end;
            size_t ll = (size_t)(le - ls);
            int kind = (int)(line & 3);
            if (kind == 0) {
                if (ll == 0) {  /* trailing blank lines end the file */
                    size_t q = pos;
                    while (q < len && is_ws((unsigned char)text[q])) q++;
                    if (q == len) break;
                    recs_free(r); return ORC_E_PARSE;
                }
                if (ls[0] != '@') { recs_free(r); return ORC_E_PARSE; }
                int e = recs_push(r, (size_t)(ls + 1 - text), token_len(ls + 1, le));
                if (e) { recs_free(r); return e; }
            } else if (kind == 1) {
                int e = recs_append(r, ls, ll);
                if (e) { recs_free(r); return e; }
            } else if (kind == 2) {
                if (ll == 0 || ls[0] != '+') { recs_free(r); return ORC_E_PARSE; }
            }
            line++;
            pos = (size_t)(le - text) + 1;
        }
        if ((line & 3) != 0) { recs_free(r); return ORC_E_PARSE; }
        return 0;
    }
    /* FASTA */
    size_t pos = i;
    int in_rec = 0;
    while (pos < len) {
        const char *ls = text + pos;
        const char *nl = memchr(ls, '\n', (size_t)(end - ls));
        const char *le = nl ? nl : end;
        if (le > ls && ls[0] == '>') {
            int e = recs_push(r, (size_t)(ls + 1 - text), token_len(ls + 1, le));
            if (e) { recs_free(r); return e; }
            in_rec = 1;
        } else if (in_rec) {
            int e = recs_append(r, ls, (size_t)(le - ls));
            if (e) { recs_free(r); return e; }
        }
        pos = (size_t)(le - text) + 1;
    }
    return 0;
}

/* ---------------------------------------------------------------- k-mers */

static inline int base_code(unsigned char c) {
    switch (c) {
    case 'A': case 'a': return 0;
    case 'C': case 'c': return 1;
    case 'G': case 'g': return 2;
    case 'T': case 't': return 3;
    default: return -1;
    }
}

static inline uint64_t mix64(uint64_t x) {
    x ^= x >> 33; x *= 0xff51afd7ed558ccdULL;
    x ^= x >> 33; x *= 0xc4ceb9fe1a85ec53ULL;
    x ^= x >> 33; return x;
}

/* Calls fn(key, window_index) for each valid window of seq. */
#define FOR_EACH_KMER(seq, L, k, canonical, KEY, WIN, ...)                    \
    do {                                                                       \
        uint64_t _mask = (k) == 32 ? ~0ULL : ((1ULL << (2 * (k))) - 1);       \
        int _shift = 2 * ((k) - 1);                                            \
        uint64_t _fw = 0, _rc = 0;                                             \
        int _run = 0;                                                          \
        for (size_t _p = 0; _p < (size_t)(L); _p++) {                          \
            int _c = base_code((unsigned char)(seq)[_p]);                      \
            if (_c < 0) { _run = 0; continue; }                                \
            _fw = ((_fw << 2) | (uint64_t)_c) & _mask;                         \
            _rc = (_rc >> 2) | ((uint64_t)(3 - _c) << _shift);                 \
            if (++_run >= (k)) {                                               \
                uint64_t KEY = (canonical) && _rc < _fw ? _rc : _fw;           \
                size_t WIN = _p + 1 - (size_t)(k);                             \
                (void)WIN;                                                     \
                __VA_ARGS__                                                    \
            }                                                                  \
        }                                                                      \
    } while (0)

/* Lock-free open-addressing table (keys + u32 values), CPU side. */
typedef struct {
    uint64_t *keys;
    uint32_t *vals;
    uint64_t mask;
} ctab_t;

static int ctab_init(ctab_t *t, uint64_t want, uint32_t init_val) {
    uint64_t cap = 1024;
    while (cap < want) cap <<= 1;
    t->keys = malloc(cap * sizeof(uint64_t));
    t->vals = malloc(cap * sizeof(uint32_t));
    if (!t->keys || !t->vals) { free(t->keys); free(t->vals); return ORC_E_OOM; }
    t->mask = cap - 1;
#pragma omp parallel for schedule(static)
    for (int64_t i = 0; i < (int64_t)cap; i++) { t->keys[i] = EMPTY; t->vals[i] = init_val; }
    return 0;
}

static void ctab_free(ctab_t *t) { free(t->keys); free(t->vals); t->keys = NULL; t->vals = NULL; }

/* The key's slot, claimed if new; CTAB_FULL when every slot holds another key. */
#define CTAB_FULL (~0ULL)
static uint64_t ctab_slot(ctab_t *t, uint64_t key) {
    uint64_t s = mix64(key) & t->mask;
    for (uint64_t probe = 0; probe <= t->mask; probe++) {
        uint64_t cur = __atomic_load_n(&t->keys[s], __ATOMIC_ACQUIRE);
        if (cur == key) return s;
        if (cur == EMPTY) {
            uint64_t exp = EMPTY;
            if (__atomic_compare_exchange_n(&t->keys[s], &exp, key, 0,
                                            __ATOMIC_ACQ_REL, __ATOMIC_ACQUIRE))
                return s;
            if (exp == key) return s;
        }
        s = (s + 1) & t->mask;
    }
    return CTAB_FULL;
}

static int ctab_find(const ctab_t *t, uint64_t key, uint32_t *val) {
    uint64_t s = mix64(key) & t->mask;
    for (;;) {
        uint64_t cur = t->keys[s];
        if (cur == key) { *val = t->vals[s]; return 1; }
        if (cur == EMPTY) return 0;
        s = (s + 1) & t->mask;
    }
}

static int set_threads(int threads) {
#ifdef _OPENMP
    if (threads > 0) omp_set_num_threads(threads);
    return omp_get_max_threads();
#else
    (void)threads;
    return 1;
#endif
}

typedef struct { uint64_t k; uint32_t c; } kc_t;

static int cmp_kc(const void *a, const void *b) {
    uint64_t x = ((const kc_t *)a)->k, y = ((const kc_t *)b)->k;
    return x < y ? -1 : x > y;
}

static int extract_table(ctab_t *t, int sorted, uint64_t **keys, uint32_t **counts, uint64_t *n) {
    uint64_t cap = t->mask + 1, m = 0;
    for (uint64_t i = 0; i < cap; i++) m += t->keys[i] != EMPTY;
    kc_t *kc = malloc((m ? m : 1) * sizeof(kc_t));
    uint64_t *ko = malloc((m ? m : 1) * sizeof(uint64_t));
    uint32_t *co = malloc((m ? m : 1) * sizeof(uint32_t));
    if (!kc || !ko || !co) { free(kc); free(ko); free(co); return ORC_E_OOM; }
    uint64_t j = 0;
    for (uint64_t i = 0; i < cap; i++)
        if (t->keys[i] != EMPTY) { kc[j].k = t->keys[i]; kc[j].c = t->vals[i]; j++; }
    if (sorted) qsort(kc, m, sizeof(kc_t), cmp_kc);
    for (uint64_t i = 0; i < m; i++) { ko[i] = kc[i].k; co[i] = kc[i].c; }
    free(kc);
    *keys = ko; *counts = co; *n = m;
    return 0;
}

int orc_count(const char *text, size_t len, int k, int canonical, int threads,
              int sorted, uint64_t **keys, uint32_t **counts, uint64_t *n) {
    return orc_count_sized(text, len, k, canonical, threads, sorted, 0, keys, counts, n);
}

int orc_count_sized(const char *text, size_t len, int k, int canonical, int threads, int sorted,
                    uint64_t distinct_hint, uint64_t **keys, uint32_t **counts, uint64_t *n) {
    if (k < 1 || k > 31 || !keys || !counts || !n) return ORC_E_INVAL;
    set_threads(threads);
    recs_t r;
    int e = parse_records(text, len, &r);
    if (e) return e;
    uint64_t windows = 0;
    for (size_t i = 0; i < r.n; i++)
        if (r.seq_len[i] >= (uint32_t)k) windows += r.seq_len[i] - k + 1;
    ctab_t t;
    e = ctab_init(&t, distinct_hint ? 2 * distinct_hint + 16 : windows + windows / 2 + 16, 0);
    if (e) { recs_free(&r); return e; }
    int full = 0;
#pragma omp parallel for schedule(dynamic, 256)
    for (int64_t i = 0; i < (int64_t)r.n; i++) {
        const char *s = r.seqbuf + r.seq_off[i];
        FOR_EACH_KMER(s, r.seq_len[i], k, canonical, key, w, {
            uint64_t slot = ctab_slot(&t, key);
            if (slot == CTAB_FULL) __atomic_store_n(&full, 1, __ATOMIC_RELAXED);
            else __atomic_fetch_add(&t.vals[slot], 1u, __ATOMIC_RELAXED);
        });
    }
    recs_free(&r);
    if (full) { ctab_free(&t); return ORC_E_FULL; }
    e = extract_table(&t, sorted, keys, counts, n);
    ctab_free(&t);
    return e;
}

void orc_histo(const uint32_t *counts, uint64_t n, uint64_t low, uint64_t high, uint64_t *hist) {
    uint64_t nb = high - low + 3;
    memset(hist, 0, nb * sizeof(uint64_t));
    for (uint64_t i = 0; i < n; i++) {
        uint64_t c = counts[i];
        if (c < low) hist[0]++;
        else if (c > high) hist[nb - 1]++;
        else hist[1 + c - low]++;
    }
}

static const char BASES[4] = {'A', 'C', 'G', 'T'};

int orc_dump(const uint64_t *keys, const uint32_t *counts, uint64_t n, int k,
             uint32_t min_count, char **out, size_t *out_len) {
    size_t cap = 1024, m = 0;
    for (uint64_t i = 0; i < n; i++) if (counts[i] >= min_count) cap += (size_t)k + 14;
    char *b = malloc(cap);
    if (!b) return ORC_E_OOM;
    for (uint64_t i = 0; i < n; i++) {
        if (counts[i] < min_count) continue;
        m += (size_t)sprintf(b + m, ">%u\n", counts[i]);
        for (int j = 0; j < k; j++) b[m++] = BASES[(keys[i] >> (2 * (k - 1 - j))) & 3];
        b[m++] = '\n';
    }
    *out = b; *out_len = m;
    return 0;
}

static uint64_t revcomp(uint64_t fw, int k) {
    uint64_t rc = 0;
    for (int i = 0; i < k; i++) { rc = (rc << 2) | (3 - (fw & 3)); fw >>= 2; }
    return rc;
}

int orc_load_dump(const char *text, size_t len, int k, int canonical,
                  uint64_t **keys, uint32_t **counts, uint64_t *n) {
    if (k < 1 || k > 31) return ORC_E_INVAL;
    recs_t r;
    int e = parse_records(text, len, &r);
    if (e) return e;
    kc_t *kc = malloc((r.n ? r.n : 1) * sizeof(kc_t));
    if (!kc) { recs_free(&r); return ORC_E_OOM; }
    for (size_t i = 0; i < r.n; i++) {
        const char *h = text + r.acc_off[i];
        uint64_t c = 0;
        if (r.acc_len[i] == 0) { free(kc); recs_free(&r); return ORC_E_PARSE; }
        for (uint32_t j = 0; j < r.acc_len[i]; j++) {
            if (h[j] < '0' || h[j] > '9') { free(kc); recs_free(&r); return ORC_E_PARSE; }
            c = c * 10 + (uint64_t)(h[j] - '0');
        }
        if (r.seq_len[i] != (uint32_t)k) { free(kc); recs_free(&r); return ORC_E_PARSE; }
        uint64_t fw = 0;
        for (int j = 0; j < k; j++) {
            int b = base_code((unsigned char)r.seqbuf[r.seq_off[i] + j]);
            if (b < 0) { free(kc); recs_free(&r); return ORC_E_PARSE; }
            fw = (fw << 2) | (uint64_t)b;
        }
        if (canonical) { uint64_t rc = revcomp(fw, k); if (rc < fw) fw = rc; }
        kc[i].k = fw;
        kc[i].c = c > 0xFFFFFFFFull ? 0xFFFFFFFFu : (uint32_t)c;
    }
    size_t m = r.n;
    recs_free(&r);
    qsort(kc, m, sizeof(kc_t), cmp_kc);
    /* duplicates (possible when a non-canonical dump is loaded canonically) add */
    size_t j = 0;
    for (size_t i = 0; i < m; i++) {
        if (j && kc[j - 1].k == kc[i].k) {
            uint64_t s = (uint64_t)kc[j - 1].c + kc[i].c;
            kc[j - 1].c = s > 0xFFFFFFFFull ? 0xFFFFFFFFu : (uint32_t)s;
        } else kc[j++] = kc[i];
    }
    uint64_t *ko = malloc((j ? j : 1) * sizeof(uint64_t));
    uint32_t *co = malloc((j ? j : 1) * sizeof(uint32_t));
    if (!ko || !co) { free(ko); free(co); free(kc); return ORC_E_OOM; }
    for (size_t i = 0; i < j; i++) { ko[i] = kc[i].k; co[i] = kc[i].c; }
    free(kc);
    *keys = ko; *counts = co; *n = j;
    return 0;
}

/* ---------------------------------------------------------------- stats */

static int cmp_u32(const void *a, const void *b) {
    uint32_t x = *(const uint32_t *)a, y = *(const uint32_t *)b;
    return x < y ? -1 : x > y;
}

static int build_lookup(ctab_t *t, const uint64_t *keys, const uint32_t *counts, uint64_t n) {
    int e = ctab_init(t, 2 * n + 16, 0);
    if (e) return e;
#pragma omp parallel for schedule(static)
    for (int64_t i = 0; i < (int64_t)n; i++) {
        uint64_t s = ctab_slot(t, keys[i]);
        t->vals[s] = counts[i];
    }
    return 0;
}

/* Per-read statistics of one read (decisions D1-D3). */
static void read_stats(const ctab_t *t, const char *s, uint32_t L, int k, int ds,
                       uint32_t *vals, uint32_t *nv, uint32_t *median, float *mean, float *stdev) {
    uint32_t m = 0;
    FOR_EACH_KMER(s, L, k, ds, key, w, {
        uint32_t c = 1;
        uint32_t got;
        if (ctab_find(t, key, &got)) c = got;
        vals[m++] = c;
    });
    *nv = m;
    if (m == 0) { *median = 0; *mean = 0.0f; *stdev = 0.0f; return; }
    uint64_t sum = 0;
    unsigned __int128 sumsq = 0;
    for (uint32_t i = 0; i < m; i++) {
        sum += vals[i];
        sumsq += (unsigned __int128)vals[i] * vals[i];
    }
    uint32_t *tmp = vals + m;
    memcpy(tmp, vals, m * sizeof(uint32_t));
    qsort(tmp, m, sizeof(uint32_t), cmp_u32);
    *median = tmp[m / 2];
    *mean = (float)((double)sum / (double)m);
    unsigned __int128 num = (unsigned __int128)m * sumsq - (unsigned __int128)sum * sum;
    double hi = (double)(uint64_t)(num >> 64), lo = (double)(uint64_t)num;
    double var = (hi * 18446744073709551616.0 + lo) / ((double)m * (double)m);
    *stdev = (float)sqrt(var);
}

typedef struct { char *b; size_t n, cap; } sbuf_t;

static int sb_reserve(sbuf_t *s, size_t extra) {
    if (s->n + extra <= s->cap) return 0;
    size_t nc = s->cap ? s->cap : 4096;
    while (nc < s->n + extra) nc *= 2;
    char *b = realloc(s->b, nc);
    if (!b) return ORC_E_OOM;
    s->b = b; s->cap = nc;
    return 0;
}

static int concat_chunks(sbuf_t *chunks, int nchunks, const char *head, char **out, size_t *out_len) {
    size_t total = strlen(head);
    for (int c = 0; c < nchunks; c++) total += chunks[c].n;
    char *o = malloc(total + 1);
    if (!o) return ORC_E_OOM;
    size_t m = strlen(head);
    memcpy(o, head, m);
    for (int c = 0; c < nchunks; c++) { memcpy(o + m, chunks[c].b, chunks[c].n); m += chunks[c].n; }
    o[m] = 0;
    *out = o; *out_len = m;
    return 0;
}

#define CHUNK_READS 4096

int orc_cov_stats(const char *reads, size_t len, const uint64_t *keys,
                  const uint32_t *counts, uint64_t n, int k, int ds,
                  int capture, int threads, char **out, size_t *out_len) {
    if (k < 1 || k > 31) return ORC_E_INVAL;
    set_threads(threads);
    recs_t r;
    int e = parse_records(reads, len, &r);
    if (e) return e;
    ctab_t t;
    e = build_lookup(&t, keys, counts, n);
    if (e) { recs_free(&r); return e; }
    uint32_t maxlen = 0;
    for (size_t i = 0; i < r.n; i++) if (r.seq_len[i] > maxlen) maxlen = r.seq_len[i];
    int nchunks = (int)((r.n + CHUNK_READS - 1) / CHUNK_READS);
    sbuf_t *chunks = calloc((size_t)(nchunks ? nchunks : 1), sizeof(sbuf_t));
    int err = 0;
#pragma omp parallel
    {
        uint32_t *vals = malloc(2 * ((size_t)maxlen + 1) * sizeof(uint32_t));
#pragma omp for schedule(dynamic, 1)
        for (int c = 0; c < nchunks; c++) {
            sbuf_t *sb = &chunks[c];
            size_t lo = (size_t)c * CHUNK_READS, hi = lo + CHUNK_READS;
            if (hi > r.n) hi = r.n;
            for (size_t i = lo; i < hi; i++) {
                uint32_t med, nv; float mean, sd;
                read_stats(&t, r.seqbuf + r.seq_off[i], r.seq_len[i], k, ds, vals, &nv, &med, &mean, &sd);
                if (sb_reserve(sb, r.acc_len[i] + 64 + (capture ? (size_t)nv * 11 : 0))) { err = ORC_E_OOM; continue; }
                sb->n += (size_t)sprintf(sb->b + sb->n, "%.*s\t%u\t%g\t%g", (int)r.acc_len[i],
                                         reads + r.acc_off[i], med, (double)mean, (double)sd);
                if (capture) {
                    sb->b[sb->n++] = '\t';
                    for (uint32_t j = 0; j < nv; j++)
                        sb->n += (size_t)sprintf(sb->b + sb->n, j ? ",%u" : "%u", vals[j]);
                }
                sb->b[sb->n++] = '\n';
            }
        }
        free(vals);
    }
    ctab_free(&t);
    recs_free(&r);
    if (!err)
        err = concat_chunks(chunks, nchunks,
                            capture ? "acc\tmedian_cov\tmean_cov\tstdev\tkmer_coverage\n"
                                    : "acc\tmedian_cov\tmean_cov\tstdev\n",
                            out, out_len);
    for (int c = 0; c < nchunks; c++) free(chunks[c].b);
    free(chunks);
    return err;
}

int orc_cov_values(const char *reads, size_t len, const uint64_t *keys,
                   const uint32_t *counts, uint64_t n, int k, int ds,
                   int threads, uint64_t *n_reads, uint32_t **median,
                   float **mean, float **stdev) {
    if (k < 1 || k > 31) return ORC_E_INVAL;
    set_threads(threads);
    recs_t r;
    int e = parse_records(reads, len, &r);
    if (e) return e;
    ctab_t t;
    e = build_lookup(&t, keys, counts, n);
    if (e) { recs_free(&r); return e; }
    uint32_t maxlen = 0;
    for (size_t i = 0; i < r.n; i++) if (r.seq_len[i] > maxlen) maxlen = r.seq_len[i];
    uint32_t *md = malloc((r.n ? r.n : 1) * sizeof(uint32_t));
    float *mn = malloc((r.n ? r.n : 1) * sizeof(float));
    float *sd = malloc((r.n ? r.n : 1) * sizeof(float));
#pragma omp parallel
    {
        uint32_t *vals = malloc(2 * ((size_t)maxlen + 1) * sizeof(uint32_t));
#pragma omp for schedule(dynamic, 1024)
        for (int64_t i = 0; i < (int64_t)r.n; i++) {
            uint32_t nv;
            read_stats(&t, r.seqbuf + r.seq_off[i], r.seq_len[i], k, ds, vals, &nv, &md[i], &mn[i], &sd[i]);
        }
        free(vals);
    }
    *n_reads = r.n;
    *median = md; *mean = mn; *stdev = sd;
    ctab_free(&t);
    recs_free(&r);
    return 0;
}

/* ---------------------------------------------------------------- R2T */

typedef struct {
    ctab_t t;
    uint64_t nrec;
    uint64_t *comp_id;
} r2t_t;

static int r2t_build(r2t_t *z, const char *bundle, size_t blen, int k, int strand) {
    recs_t b;
    int e = parse_records(bundle, blen, &b);
    if (e) return e;
    uint64_t windows = 0;
    for (size_t i = 0; i < b.n; i++)
        if (b.seq_len[i] >= (uint32_t)k) windows += b.seq_len[i] - k + 1;
    e = ctab_init(&z->t, 2 * windows + 16, 0xFFFFFFFFu);
    if (e) { recs_free(&b); return e; }
    z->nrec = b.n;
    z->comp_id = malloc((b.n ? b.n : 1) * sizeof(uint64_t));
    for (size_t i = 0; i < b.n; i++) {
        const char *h = bundle + b.acc_off[i];
        uint32_t hl = b.acc_len[i];
        uint64_t id = i;
        if (hl > 2 && h[0] == 's' && h[1] == '_' && h[2] >= '0' && h[2] <= '9') {
            id = 0;
            for (uint32_t j = 2; j < hl && h[j] >= '0' && h[j] <= '9'; j++) id = id * 10 + (uint64_t)(h[j] - '0');
        }
        z->comp_id[i] = id;
    }
    /* serial in record order: the first record holding a k-mer owns it (D4) */
    for (size_t i = 0; i < b.n; i++) {
        const char *s = b.seqbuf + b.seq_off[i];
        FOR_EACH_KMER(s, b.seq_len[i], k, !strand, key, w, {
            uint64_t slot = ctab_slot(&z->t, key);
            if (z->t.vals[slot] > (uint32_t)i) z->t.vals[slot] = (uint32_t)i;
        });
    }
    recs_free(&b);
    return 0;
}

static void r2t_read(const r2t_t *z, const char *s, uint32_t L, int k, int strand,
                     uint32_t *buf, int32_t *rec, uint32_t *hits, uint32_t *nwin) {
    *rec = -1; *hits = 0; *nwin = L >= (uint32_t)k ? L - k + 1 : 0;
    uint32_t m = 0;
    FOR_EACH_KMER(s, L, k, !strand, key, w, {
        uint32_t v;
        if (ctab_find(&z->t, key, &v)) buf[m++] = v;
    });
    if (!m) return;
    qsort(buf, m, sizeof(uint32_t), cmp_u32);
    uint32_t best = 0, bestv = 0;
    for (uint32_t i = 0; i < m;) {
        uint32_t j = i;
        while (j < m && buf[j] == buf[i]) j++;
        if (j - i > best) { best = j - i; bestv = buf[i]; }
        i = j;
    }
    *rec = (int32_t)bestv; *hits = best;
}

int orc_r2t_values(const char *reads, size_t rlen, const char *bundle,
                   size_t blen, int k, int strand, int threads,
                   uint64_t *n_reads, int32_t **rec, uint32_t **hits,
                   uint32_t **nwin) {
    if (k < 1 || k > 31) return ORC_E_INVAL;
    set_threads(threads);
    r2t_t z;
    int e = r2t_build(&z, bundle, blen, k, strand);
    if (e) return e;
    recs_t r;
    e = parse_records(reads, rlen, &r);
    if (e) { ctab_free(&z.t); free(z.comp_id); return e; }
    uint32_t maxlen = 0;
    for (size_t i = 0; i < r.n; i++) if (r.seq_len[i] > maxlen) maxlen = r.seq_len[i];
    int32_t *rc = malloc((r.n ? r.n : 1) * sizeof(int32_t));
    uint32_t *h = malloc((r.n ? r.n : 1) * sizeof(uint32_t));
    uint32_t *nw = malloc((r.n ? r.n : 1) * sizeof(uint32_t));
#pragma omp parallel
    {
        uint32_t *buf = malloc(((size_t)maxlen + 1) * sizeof(uint32_t));
#pragma omp for schedule(dynamic, 1024)
        for (int64_t i = 0; i < (int64_t)r.n; i++)
            r2t_read(&z, r.seqbuf + r.seq_off[i], r.seq_len[i], k, strand, buf, &rc[i], &h[i], &nw[i]);
        free(buf);
    }
    *n_reads = r.n; *rec = rc; *hits = h; *nwin = nw;
    recs_free(&r);
    ctab_free(&z.t);
    free(z.comp_id);
    return 0;
}

int orc_r2t(const char *reads, size_t rlen, const char *bundle, size_t blen,
            int k, int strand, int min_pct, int threads, char **out,
            size_t *out_len) {
    if (k < 1 || k > 31) return ORC_E_INVAL;
    set_threads(threads);
    r2t_t z;
    int e = r2t_build(&z, bundle, blen, k, strand);
    if (e) return e;
    recs_t r;
    e = parse_records(reads, rlen, &r);
    if (e) { ctab_free(&z.t); free(z.comp_id); return e; }
    uint32_t maxlen = 0;
    for (size_t i = 0; i < r.n; i++) if (r.seq_len[i] > maxlen) maxlen = r.seq_len[i];
    int nchunks = (int)((r.n + CHUNK_READS - 1) / CHUNK_READS);
    sbuf_t *chunks = calloc((size_t)(nchunks ? nchunks : 1), sizeof(sbuf_t));
    int err = 0;
#pragma omp parallel
    {
        uint32_t *buf = malloc(((size_t)maxlen + 1) * sizeof(uint32_t));
#pragma omp for schedule(dynamic, 1)
        for (int c = 0; c < nchunks; c++) {
            sbuf_t *sb = &chunks[c];
            size_t lo = (size_t)c * CHUNK_READS, hi = lo + CHUNK_READS;
            if (hi > r.n) hi = r.n;
            for (size_t i = lo; i < hi; i++) {
                int32_t rec; uint32_t hits, nw;
                const char *s = r.seqbuf + r.seq_off[i];
                r2t_read(&z, s, r.seq_len[i], k, strand, buf, &rec, &hits, &nw);
                if (rec < 0) continue;
                uint32_t pct = (uint32_t)((100ull * hits) / nw);
                if (min_pct > 0 && pct < (uint32_t)min_pct) continue;
                if (sb_reserve(sb, r.acc_len[i] + r.seq_len[i] + 64)) { err = ORC_E_OOM; continue; }
                sb->n += (size_t)sprintf(sb->b + sb->n, "%llu\t>%.*s\t%u\t",
                                         (unsigned long long)z.comp_id[rec], (int)r.acc_len[i],
                                         reads + r.acc_off[i], pct);
                for (uint32_t j = 0; j < r.seq_len[i]; j++) {
                    char ch = s[j];
                    sb->b[sb->n++] = (ch >= 'a' && ch <= 'z') ? (char)(ch - 32) : ch;
                }
                sb->b[sb->n++] = '\n';
            }
        }
        free(buf);
    }
    recs_free(&r);
    ctab_free(&z.t);
    free(z.comp_id);
    if (!err) err = concat_chunks(chunks, nchunks, "", out, out_len);
    for (int c = 0; c < nchunks; c++) free(chunks[c].b);
    free(chunks);
    return err;
}

/* ---------------------------------------------------------------- de Bruijn (D8) */

typedef struct { uint64_t *key; uint32_t *node; uint64_t mask; } dmap_t;

static uint32_t dmap_get(dmap_t *m, uint64_t key, uint32_t fresh, int *is_new) {
    uint64_t s = mix64(key) & m->mask;
    for (;;) {
        if (m->key[s] == EMPTY) { m->key[s] = key; m->node[s] = fresh; *is_new = 1; return fresh; }
        if (m->key[s] == key) { *is_new = 0; return m->node[s]; }
        s = (s + 1) & m->mask;
    }
}

/* one record's graph text appended to sb */
static int dbg_record(const char *seq, uint32_t L, int K1, int ss, uint64_t comp, sbuf_t *sb) {
    if (L < (uint32_t)K1) return 0;
    uint64_t nw = L - K1 + 1, cap = 1024;
    while (cap < 2 * nw) cap <<= 1;
    dmap_t m = {malloc(cap * 8), malloc(cap * 4), cap - 1};
    uint32_t *cnt = malloc(nw * 4), *first = malloc(nw * 4);
    int32_t *prev = malloc(nw * 4);
    if (!m.key || !m.node || !cnt || !first || !prev) {
        free(m.key); free(m.node); free(cnt); free(first); free(prev);
        return ORC_E_OOM;
    }
    for (uint64_t i = 0; i < cap; i++) m.key[i] = EMPTY;
    uint32_t n = 0;
    int64_t last_w = -2;
    uint32_t last_node = 0;
    FOR_EACH_KMER(seq, L, K1, !ss, key, w, {
        int is_new;
        uint32_t v = dmap_get(&m, key, n, &is_new);
        if (is_new) {
            cnt[n] = 0;
            first[n] = (uint32_t)w;
            prev[n] = last_w == (int64_t)w - 1 ? (int32_t)last_node : -1;
            n++;
        }
        cnt[v]++;
        last_w = (int64_t)w;
        last_node = v;
    });
    int e = 0;
    if (n) {
        if (sb_reserve(sb, 32 + (size_t)n * (K1 + 40))) e = ORC_E_OOM;
        else {
            sb->n += (size_t)sprintf(sb->b + sb->n, "Component %llu\n", (unsigned long long)comp);
            for (uint32_t i = 0; i < n; i++) {
                sb->n += (size_t)sprintf(sb->b + sb->n, "%u\t%d\t%u\t", i, prev[i], cnt[i]);
                for (int j = 0; j < K1; j++) {
                    char ch = seq[first[i] + j];
                    sb->b[sb->n++] = (ch >= 'a' && ch <= 'z') ? (char)(ch - 32) : ch;
                }
                sb->b[sb->n++] = '\n';
            }
        }
    }
    free(m.key); free(m.node); free(cnt); free(first); free(prev);
    return e;
}

int orc_debruijn(const char *bundle, size_t blen, int K, int ss, int threads, char **out, size_t *out_len) {
    if (K < 1 || K > 30) return ORC_E_INVAL;
    set_threads(threads);
    recs_t b;
    int e = parse_records(bundle, blen, &b);
    if (e) return e;
    sbuf_t *chunks = calloc(b.n ? b.n : 1, sizeof(sbuf_t));
    if (!chunks) { recs_free(&b); return ORC_E_OOM; }
    int err = 0;
#pragma omp parallel for schedule(dynamic, 16)
    for (int64_t i = 0; i < (int64_t)b.n; i++) {
        const char *h = bundle + b.acc_off[i];
        uint32_t hl = b.acc_len[i];
        uint64_t id = (uint64_t)i;
        if (hl > 2 && h[0] == 's' && h[1] == '_' && h[2] >= '0' && h[2] <= '9') {
            id = 0;
            for (uint32_t j = 2; j < hl && h[j] >= '0' && h[j] <= '9'; j++) id = id * 10 + (uint64_t)(h[j] - '0');
        }
        int ee = dbg_record(b.seqbuf + b.seq_off[i], b.seq_len[i], K + 1, ss, id, &chunks[i]);
        if (ee) err = ee;
    }
    if (!err) err = concat_chunks(chunks, (int)b.n, "", out, out_len);
    for (size_t i = 0; i < b.n; i++) free(chunks[i].b);
    free(chunks);
    recs_free(&b);
    return err;
}

int orc_records(const char *text, size_t len, char **out, size_t *out_len) {
    recs_t r;
    int e = parse_records(text, len, &r);
    if (e) return e;
    size_t cap = 16;
    for (size_t i = 0; i < r.n; i++) cap += r.acc_len[i] + r.seq_len[i] + 2;
    char *o = malloc(cap);
    if (!o) { recs_free(&r); return ORC_E_OOM; }
    size_t m = 0;
    for (size_t i = 0; i < r.n; i++) {
        memcpy(o + m, text + r.acc_off[i], r.acc_len[i]); m += r.acc_len[i];
        o[m++] = '\t';
        memcpy(o + m, r.seqbuf + r.seq_off[i], r.seq_len[i]); m += r.seq_len[i];
        o[m++] = '\n';
    }
    recs_free(&r);
    *out = o; *out_len = m;
    return 0;
}

/* ---- FASTQ -> FASTA prep: util/support_scripts/fastQ_to_fastA.pl:60-118,
 * the executable spec of Trinity's `seqtk-trinity seq -A -R N [-r]`
 * (Trinity:2745-2805).  Line by line: a line starting with '@' (after its CRs
 * are removed) opens a record of it and the next three lines; every other
 * line is skipped.  Only the header loses its CRs; the other lines lose just
 * their "\n".  A record is clean when the sequence is non-empty and not "0",
 * the third line starts with '+', the quality line holds a non-space byte and
 * is as long as the sequence (fastQ_to_fastA.pl:86-88).  Name = first
 * whitespace-separated field of the header without '@' (empty if the header
 * starts with whitespace); "/1" or "/2" is added when more fields follow, the
 * name does not already end in /1 or /2, and the next field starts "1:" or
 * "2:" (Casava 1.8, :95-97); then "/append" when append >= 0 (the -a option),
 * or with ORC_FA_IF_MISSING only when the name does not already end in /1 or
 * /2; ORC_FA_REV reverse-complements the sequence with
 * PerlLib/Nuc_translator.pm:286-292's letter map.  A poorly formed record
 * fails the call (ORC_E_PARSE, *bad = 1-based record number) unless
 * ORC_FA_IGNORE_DIRTY skips it. */
static int pl_ws(unsigned char c) { return c == ' ' || c == '\t' || c == '\n' || c == '\r' || c == '\f' || c == '\v'; }

static unsigned char rc_letter(unsigned char c) {
    static const char from[] = "ACGTacgtyrkmYRKMUu", to[] = "TGCAtgcarymkRYMKAa";
    for (int i = 0; from[i]; i++)
        if ((unsigned char)from[i] == c) return (unsigned char)to[i];
    return c;
}

static int fa_ends_12(const char *n, size_t l) { return l >= 2 && n[l - 2] == '/' && (n[l - 1] == '1' || n[l - 1] == '2'); }

int orc_fastq_to_fasta(const char *text, size_t len, int append, int flags, char **out, size_t *out_len, uint64_t *bad) {
    sbuf_t o = {0};
    size_t p = 0;
    uint64_t rec = 0;
    char *hdr = NULL;
    size_t hcap = 0;
    *bad = 0;
    while (p < len) {
        /* one line [p, e) and the next line start q */
        const char *nl = memchr(text + p, '\n', len - p);
        size_t e = nl ? (size_t)(nl - text) : len, q = nl ? e + 1 : len;
        /* the header candidate without CRs */
        size_t hl = 0;
        if (hcap < e - p + 1) { hcap = e - p + 64; free(hdr); hdr = malloc(hcap); if (!hdr) { free(o.b); return ORC_E_OOM; } }
        for (size_t i = p; i < e; i++) if (text[i] != '\r') hdr[hl++] = text[i];
        if (!(hl > 0 && hdr[0] == '@')) { p = q; continue; }
        rec++;
        /* the next three lines (absent at end of input) */
        size_t ls[3], le[3];
        int have[3];
        size_t r = q;
        for (int j = 0; j < 3; j++) {
            have[j] = r < len;
            const char *m = have[j] ? memchr(text + r, '\n', len - r) : NULL;
            ls[j] = r;
            le[j] = have[j] ? (m ? (size_t)(m - text) : len) : r;
            r = have[j] ? (m ? le[j] + 1 : len) : r;
        }
        p = r;
        size_t sl = le[0] - ls[0], ql = le[2] - ls[2];
        int clean = have[0] && have[1] && have[2] && sl > 0 && !(sl == 1 && text[ls[0]] == '0') &&
                    le[1] > ls[1] && text[ls[1]] == '+' && ql == sl;
        if (clean) {
            int ns = 0;
            for (size_t i = ls[2]; i < le[2]; i++) if (!pl_ws((unsigned char)text[i])) { ns = 1; break; }
            clean = ns;
        }
        if (!clean) {
            if (flags & ORC_FA_IGNORE_DIRTY) continue;
            free(hdr); free(o.b);
            *bad = rec;
            return ORC_E_PARSE;
        }
        /* name: first field of the header after '@'; the second decides Casava */
        size_t a = 1, b = 1;
        while (b < hl && !pl_ws((unsigned char)hdr[b])) b++;
        size_t f2 = b;
        while (f2 < hl && pl_ws((unsigned char)hdr[f2])) f2++;
        int more = f2 < hl;
        char suffix[32];
        int sfx = 0;
        if (more && !fa_ends_12(hdr + a, b - a) && f2 + 1 < hl && (hdr[f2] == '1' || hdr[f2] == '2') && hdr[f2 + 1] == ':')
            sfx = snprintf(suffix, sizeof suffix, "/%c", hdr[f2]);
        if (append >= 0) {
            int ends = fa_ends_12(hdr + a, b - a) || sfx;
            if (!(flags & ORC_FA_IF_MISSING) || !ends) sfx += snprintf(suffix + sfx, sizeof suffix - sfx, "/%d", append);
        }
        if (sb_reserve(&o, 4 + (b - a) + sfx + sl)) { free(hdr); free(o.b); return ORC_E_OOM; }
        o.b[o.n++] = '>';
        memcpy(o.b + o.n, hdr + a, b - a); o.n += b - a;
        memcpy(o.b + o.n, suffix, sfx); o.n += sfx;
        o.b[o.n++] = '\n';
        if (flags & ORC_FA_REV)
            for (size_t i = 0; i < sl; i++) o.b[o.n++] = (char)rc_letter((unsigned char)text[le[0] - 1 - i]);
        else {
            memcpy(o.b + o.n, text + ls[0], sl);
            o.n += sl;
        }
        o.b[o.n++] = '\n';
    }
    free(hdr);
    if (!o.b) { o.b = malloc(1); if (!o.b) return ORC_E_OOM; }
    *out = o.b;
    *out_len = o.n;
    return 0;
}

/* ---------------------------------------------------------- normalization tail
 * What util/insilico_read_normalization.pl does with the two coverage-stats
 * tables, restated step by step on their text:
 *   sort    head -n1 S > S.sort && tail -n +2 S | sort -k1,1 >> S.sort
 *           (insilico_read_normalization.pl:865-892, LC_ALL=C from
 *           PerlLib/COMMON.pm:7): rows by their first blank-delimited field,
 *           bytewise, ties by the whole line (sort's last-resort compare);
 *   merge   util/support_scripts/nbkc_merge_left_right_stats.pl --sorted
 *           (insilico:951-965; script lines 89-146): two cursors, a pair when
 *           the accs agree without their "/digit" ending, else the cursor
 *           whose acc is string-less moves; averages printed with "%.1f";
 *   select  util/support_scripts/nbkc_normalize.pl (insilico:972-977; script
 *           lines 68-117): srand(12345); rows below min_cov, with mean <= 0 or
 *           stdev/mean > max_CV are dropped, each other row draws rand(1) and
 *           is kept when the draw is <= max_cov/median; its acc is printed
 *           without a final "/1" or "/2".
 * Single-end (or pairs kept apart, insilico:917-947) selects on one sorted
 * table.  Perl's rand is drand48 (X' = 0x5DEECE66D X + 11 mod 2^48, seed
 * (s << 16) + 0x330E, value X'/2^48); its numeric conversion of these fields
 * is strtod's. */

typedef struct { const char *p; size_t n; } span_t;

static int is_blank_c(unsigned char c) { return c == ' ' || c == '\t'; }
static int is_perl_ws(unsigned char c) { return c == ' ' || (c >= 9 && c <= 13); }

static int span_cmp(span_t a, span_t b) {
    size_t m = a.n < b.n ? a.n : b.n;
    int r = m ? memcmp(a.p, b.p, m) : 0;
    if (r) return r;
    return a.n < b.n ? -1 : a.n > b.n;
}

static span_t first_field(span_t line) {
    size_t i = 0;
    while (i < line.n && !is_blank_c((unsigned char)line.p[i])) i++;
    span_t f = {line.p, i};
    return f;
}

static int cmp_stats_line(const void *x, const void *y) {
    span_t a = *(const span_t *)x, b = *(const span_t *)y;
    int r = span_cmp(first_field(a), first_field(b));
    return r ? r : span_cmp(a, b);
}

/* rows of a table (after its header line), without their "\n" */
static int table_rows(const char *t, size_t len, span_t *head, span_t **rows, size_t *n) {
    size_t cap = 1024, k = 0, i = 0;
    span_t *r = malloc(cap * sizeof *r);
    if (!r) return ORC_E_OOM;
    int have_head = 0;
    while (i < len) {
        size_t j = i;
        while (j < len && t[j] != '\n') j++;
        span_t s = {t + i, j - i};
        if (!have_head) { *head = s; have_head = 1; }
        else {
            if (k == cap) {
                cap *= 2;
                span_t *q = realloc(r, cap * sizeof *r);
                if (!q) { free(r); return ORC_E_OOM; }
                r = q;
            }
            r[k++] = s;
        }
        i = j + 1;
    }
    if (!have_head) { free(r); return ORC_E_PARSE; }
    *rows = r;
    *n = k;
    return 0;
}

/* tab-separated fields of a row; returns their number (at most max) */
static int split_tabs(span_t line, span_t *f, int max) {
    int k = 0;
    size_t i = 0;
    while (k < max) {
        size_t j = i;
        while (j < line.n && line.p[j] != '\t') j++;
        f[k].p = line.p + i; f[k].n = j - i; k++;
        if (j >= line.n) break;
        i = j + 1;
    }
    return k;
}

static double num_of(span_t f) {
    char tmp[64];
    size_t n = f.n < sizeof tmp - 1 ? f.n : sizeof tmp - 1;
    memcpy(tmp, f.p, n);
    tmp[n] = 0;
    return strtod(tmp, NULL);
}

/* acc without a final "/<digit>" when what precedes it is one or more non-space bytes */
static span_t merge_core(span_t a) {
    if (a.n >= 3 && a.p[a.n - 2] == '/' && a.p[a.n - 1] >= '0' && a.p[a.n - 1] <= '9') {
        for (size_t i = 0; i + 2 < a.n; i++)
            if (is_perl_ws((unsigned char)a.p[i])) return a;
        a.n -= 2;
    }
    return a;
}

static span_t strip_12(span_t a) {
    if (a.n >= 2 && a.p[a.n - 2] == '/' && (a.p[a.n - 1] == '1' || a.p[a.n - 1] == '2')) a.n -= 2;
    return a;
}

static int sb_put(sbuf_t *s, const char *p, size_t n) {
    if (sb_reserve(s, n)) return ORC_E_OOM;
    memcpy(s->b + s->n, p, n);
    s->n += n;
    return 0;
}

int orc_norm(const char *left, size_t llen, const char *right, size_t rlen, int max_cov, int min_cov, int max_cv,
             char **table, size_t *table_len, char **accs, size_t *accs_len, uint64_t counts[4]) {
    span_t lh, rh, *lr = NULL, *rr = NULL;
    size_t nl = 0, nr = 0;
    sbuf_t tb = {0}, ab = {0};
    int e = table_rows(left, llen, &lh, &lr, &nl);
    if (!e && right) e = table_rows(right, rlen, &rh, &rr, &nr);
    if (e) { free(lr); return e; }
    qsort(lr, nl, sizeof *lr, cmp_stats_line);
    if (right) qsort(rr, nr, sizeof *rr, cmp_stats_line);
    /* the table nbkc_normalize.pl reads: the merged pairs, or the sorted stats */
    if (right) {
        const char *hdr = "acc\tleft_acc\tleft_median_cov\tleft_mean_cov\tleft_stdev\tright_acc\tright_median_cov\t"
                          "right_mean_cov\tright_stdev\tmedian_cov\tmean_cov\tstdev\n";
        e = sb_put(&tb, hdr, strlen(hdr));
        size_t i = 0, j = 0;
        while (!e && i < nl && j < nr) {
            span_t a[8], b[8];
            if (split_tabs(lr[i], a, 8) != 4 || split_tabs(rr[j], b, 8) != 4) { e = ORC_E_PARSE; break; }
            span_t ca = merge_core(a[0]), cb = merge_core(b[0]);
            if (span_cmp(ca, cb) != 0) {
                if (span_cmp(a[0], b[0]) < 0) i++; else j++;
                continue;
            }
            char avg[3][64];
            for (int q = 0; q < 3; q++) snprintf(avg[q], sizeof avg[q], "%.1f", (num_of(a[q + 1]) + num_of(b[q + 1])) / 2);
            e = sb_put(&tb, ca.p, ca.n);
            for (int q = 0; q < 4 && !e; q++) { e = sb_put(&tb, "\t", 1); if (!e) e = sb_put(&tb, a[q].p, a[q].n); }
            for (int q = 0; q < 4 && !e; q++) { e = sb_put(&tb, "\t", 1); if (!e) e = sb_put(&tb, b[q].p, b[q].n); }
            for (int q = 0; q < 3 && !e; q++) { e = sb_put(&tb, "\t", 1); if (!e) e = sb_put(&tb, avg[q], strlen(avg[q])); }
            if (!e) e = sb_put(&tb, "\n", 1);
            i++; j++;
        }
    } else {
        e = sb_put(&tb, lh.p, lh.n);
        if (!e) e = sb_put(&tb, "\n", 1);
        for (size_t i = 0; i < nl && !e; i++) {
            e = sb_put(&tb, lr[i].p, lr[i].n);
            if (!e) e = sb_put(&tb, "\n", 1);
        }
    }
    free(lr);
    free(rr);
    /* nbkc_normalize.pl over that table, columns looked up by name */
    uint64_t total = 0, selected = 0, aberrant = 0, below = 0;
    if (!e) {
        span_t th, *rows = NULL;
        size_t n = 0;
        e = table_rows(tb.b, tb.n, &th, &rows, &n);
        span_t hf[16];
        int nh = e ? 0 : split_tabs(th, hf, 16);
        int c_acc = -1, c_med = -1, c_mean = -1, c_sd = -1;
        for (int q = 0; q < nh; q++) {
            span_t f = hf[q];
            if (f.n == 3 && !memcmp(f.p, "acc", 3)) c_acc = q;
            else if (f.n == 10 && !memcmp(f.p, "median_cov", 10)) c_med = q;
            else if (f.n == 8 && !memcmp(f.p, "mean_cov", 8)) c_mean = q;
            else if (f.n == 5 && !memcmp(f.p, "stdev", 5)) c_sd = q;
        }
        if (!e && (c_acc < 0 || c_med < 0 || c_mean < 0 || c_sd < 0)) e = ORC_E_PARSE;
        uint64_t x = ((uint64_t)12345 << 16) | 0x330E;
        const uint64_t mask = (1ULL << 48) - 1;
        for (size_t i = 0; i < n && !e; i++) {
            span_t f[16];
            if (split_tabs(rows[i], f, 16) != nh) { e = ORC_E_PARSE; break; }
            total++;
            double med = num_of(f[c_med]);
            if (med < (double)min_cov) { below++; continue; }
            double sd = num_of(f[c_sd]), u = num_of(f[c_mean]);
            if (u <= 0) { aberrant++; continue; }
            double cv = sd / u;
            if (cv > (double)max_cv) { aberrant++; continue; }
            x = (x * 0x5DEECE66DULL + 0xB) & mask;
            double r = ldexp((double)x, -48);
            if (med == 0) { e = ORC_E_INVAL; break; }   /* Perl: Illegal division by zero */
            if (r <= (double)max_cov / med) {
                span_t a = strip_12(f[c_acc]);
                e = sb_put(&ab, a.p, a.n);
                if (!e) e = sb_put(&ab, "\n", 1);
                selected++;
            }
        }
        free(rows);
    }
    if (e) { free(tb.b); free(ab.b); return e; }
    if (!tb.b) tb.b = malloc(1);
    if (!ab.b) ab.b = malloc(1);
    if (!tb.b || !ab.b) { free(tb.b); free(ab.b); return ORC_E_OOM; }
    counts[0] = total; counts[1] = selected; counts[2] = aberrant; counts[3] = below;
    *table = tb.b; *table_len = tb.n;
    *accs = ab.b; *accs_len = ab.n;
    return 0;
}

/* ------------------------------------------------------------ read extraction
 * make_normalized_reads_file of util/insilico_read_normalization.pl:470-584
 * (FASTA input: see fa_chunk below; FASTQ:) the accs file's non-blank lines, each without a final "/" and
 * word character (build_selected_index, :452-466), are the wanted names; every
 * 4-line record of the FASTQ text (PerlLib/Fastq_reader.pm:47-75) whose core
 * name -- the header's first whitespace-delimited field without '@' and
 * without a final "/1" or "/2" (Fastq_reader.pm:106-121), then without its
 * first "_forward" and its first "_reverse" (insilico:529-531) -- is wanted is
 * written out verbatim, in input order.  A malformed record, or a wanted name
 * no record carries (insilico:556-578), is an error: ORC_E_PARSE with
 * *missing = the number of such names. */

static int is_word_c(unsigned char c) {
    return (c >= '0' && c <= '9') || (c >= 'A' && c <= 'Z') || (c >= 'a' && c <= 'z') || c == '_';
}

typedef struct { char *p; size_t n; uint32_t hits; } want_t;

static int cmp_want(const void *x, const void *y) {
    const want_t *a = x, *b = y;
    span_t sa = {a->p, a->n}, sb2 = {b->p, b->n};
    return span_cmp(sa, sb2);
}

static void remove_first(char *s, size_t *n, const char *pat) {
    size_t m = strlen(pat);
    for (size_t i = 0; i + m <= *n; i++)
        if (!memcmp(s + i, pat, m)) {
            memmove(s + i, s + i + m, *n - i - m);
            *n -= m;
            return;
        }
}

/* PerlLib/Fasta_reader.pm:45-70 on one chunk (read up to and including the
 * next "\n>"): the '>' at its start and end dropped, control bytes other than
 * tab and newline and bytes 0x7F-0xFF deleted, header = first line, sequence =
 * the other lines joined with whitespace removed; written ">header\nseq\n"
 * when its accession (first field of the header, without a final "/1" or
 * "/2", insilico:526-527) is wanted. */
static int fa_chunk(const char *c, size_t n, want_t *w, size_t nd, sbuf_t *o) {
    if (n && c[0] == '>') { c++; n--; }
    if (n && c[n - 1] == '>') n--;
    char *hdr = malloc(n + 1), *seq = malloc(n + 1);
    if (!hdr || !seq) { free(hdr); free(seq); return ORC_E_OOM; }
    size_t hl = 0, sl = 0, i = 0;
    for (; i < n && c[i] != '\n'; i++) {
        unsigned char b = (unsigned char)c[i];
        if (b == '\t' || (b >= 32 && b < 127)) hdr[hl++] = (char)b;
    }
    for (; i < n; i++) {
        unsigned char b = (unsigned char)c[i];
        if (b > 32 && b < 127) seq[sl++] = (char)b;
    }
    size_t al = 0;
    if (hl && hdr[0] != ' ' && hdr[0] != '\t')
        while (al < hl && hdr[al] != ' ' && hdr[al] != '\t') al++;
    size_t kl = al;
    if (kl >= 2 && hdr[kl - 2] == '/' && (hdr[kl - 1] == '1' || hdr[kl - 1] == '2')) kl -= 2;
    want_t key = {hdr, kl, 0};
    want_t *hit = nd ? bsearch(&key, w, nd, sizeof *w, cmp_want) : NULL;
    int e = 0;
    if (hit) {
        hit->hits++;
        e = sb_put(o, ">", 1);
        if (!e) e = sb_put(o, hdr, hl);
        if (!e) e = sb_put(o, "\n", 1);
        if (!e) e = sb_put(o, seq, sl);
        if (!e) e = sb_put(o, "\n", 1);
    }
    free(hdr);
    free(seq);
    return e;
}

static int has_word(const char *c, size_t n) {
    for (size_t i = 0; i < n; i++)
        if (is_word_c((unsigned char)c[i])) return 1;
    return 0;
}

/* the next "\n>"-terminated chunk at *pos */
static size_t fa_next(const char *t, size_t len, size_t *pos) {
    size_t a = *pos, q = a;
    while (q + 1 < len && !(t[q] == '\n' && t[q + 1] == '>')) q++;
    size_t end = q + 1 < len ? q + 2 : len;
    *pos = end;
    return end - a;
}

int orc_norm_extract(const char *fq, size_t len, const char *accs, size_t alen, char **out, size_t *out_len,
                     uint64_t *missing) {
    *missing = 0;
    size_t cap = 1024, nw = 0;
    want_t *w = malloc(cap * sizeof *w);
    if (!w) return ORC_E_OOM;
    int e = 0;
    for (size_t i = 0; i < alen && !e;) {
        size_t j = i;
        while (j < alen && accs[j] != '\n') j++;
        size_t n = j - i;
        int blank = 1;
        for (size_t q = 0; q < n; q++) if (!is_perl_ws((unsigned char)accs[i + q])) blank = 0;
        if (!blank) {
            if (n >= 2 && accs[i + n - 2] == '/' && is_word_c((unsigned char)accs[i + n - 1])) n -= 2;
            if (nw == cap) {
                cap *= 2;
                want_t *q = realloc(w, cap * sizeof *w);
                if (!q) { e = ORC_E_OOM; break; }
                w = q;
            }
            w[nw].p = malloc(n ? n : 1);
            if (!w[nw].p) { e = ORC_E_OOM; break; }
            memcpy(w[nw].p, accs + i, n);
            w[nw].n = n;
            w[nw].hits = 0;
            nw++;
        }
        i = j + 1;
    }
    if (!e) qsort(w, nw, sizeof *w, cmp_want);
    /* distinct names only */
    size_t nd = 0;
    for (size_t i = 0; i < nw && !e; i++) {
        if (nd && w[nd - 1].n == w[i].n && !memcmp(w[nd - 1].p, w[i].p, w[i].n)) { free(w[i].p); continue; }
        w[nd++] = w[i];
    }
    sbuf_t o = {0};
    char *name = NULL;
    size_t name_cap = 0;
    size_t first = 0;
    while (first < len && is_perl_ws((unsigned char)fq[first])) first++;
    const int fasta = first < len && fq[first] == '>';
    for (size_t pos = 0; fasta && pos < len && !e;) {
        /* Fasta_reader::next: a chunk without a word character is skipped once */
        size_t a = pos, n = fa_next(fq, len, &pos);
        if (!has_word(fq + a, n)) {
            if (pos >= len) break;   /* the read after it finds nothing: end of input */
            a = pos;
            n = fa_next(fq, len, &pos);
        }
        e = fa_chunk(fq + a, n, w, nd, &o);
    }
    for (size_t pos = 0; !fasta && pos < len && !e;) {
        /* four lines, each with its "\n" when there is one */
        size_t ls[4], le[4], p = pos;
        int nlines = 0;
        while (nlines < 4 && p < len) {
            size_t q = p;
            while (q < len && fq[q] != '\n') q++;
            ls[nlines] = p; le[nlines] = q; nlines++;
            p = q < len ? q + 1 : q;
        }
        /* split(/\n/) drops trailing empty fields: the record needs 4 */
        int fields = nlines;
        while (fields > 0 && le[fields - 1] == ls[fields - 1]) fields--;
        if (fields != 4 || fq[ls[0]] != '@') { e = ORC_E_PARSE; break; }
        size_t a = ls[0] + 1, b = a;
        while (b < le[0] && !is_perl_ws((unsigned char)fq[b])) b++;
        size_t n = b - a;
        if (n + 1 > name_cap) {
            name_cap = 2 * (n + 1);
            char *q = realloc(name, name_cap);
            if (!q) { e = ORC_E_OOM; break; }
            name = q;
        }
        memcpy(name, fq + a, n);
        if (n >= 3 && name[n - 2] == '/' && (name[n - 1] == '1' || name[n - 1] == '2')) n -= 2;
        remove_first(name, &n, "_forward");
        remove_first(name, &n, "_reverse");
        want_t key = {name, n, 0};
        want_t *hit = nd ? bsearch(&key, w, nd, sizeof *w, cmp_want) : NULL;
        if (hit) {
            hit->hits++;
            e = sb_put(&o, fq + pos, p - pos);
        }
        pos = p;
    }
    free(name);
    for (size_t i = 0; i < nd; i++) {
        if (!w[i].hits) (*missing)++;
        free(w[i].p);
    }
    free(w);
    if (!e && *missing) e = ORC_E_PARSE;
    if (e) { free(o.b); return e; }
    if (!o.b) { o.b = malloc(1); if (!o.b) return ORC_E_OOM; }
    *out = o.b;
    *out_len = o.n;
    return 0;
}

void orc_free(void *p) { free(p); }
