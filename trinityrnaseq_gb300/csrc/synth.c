/*
 * synth.c -- seeded synthetic RNA-Seq inputs for the k-mer hot path.
 *
 * The reference ships no benchmark dataset for this path (its only reads are
 * the 30,575-pair smoke fixture under sample_data/test_Trinity_Assembly), so
 * the workloads are generated: random transcriptomes, log-normal expression,
 * reads with substitution errors and N bases, FASTA or constant-quality FASTQ,
 * Inchworm-style bundles of contigs grouped into components ('>s_<id>' records
 * whose contigs are joined by 'X', util/support_scripts/add_LR_reads_to_iworm_bundle.pl:19-47),
 * and power-law read bins.  Every random draw comes from a counter-based
 * stream keyed by (seed, purpose, index), so reads are generated in parallel
 * and the output depends only on the parameters.
 *
 * Read names have a fixed width, so every record of a read set has the same
 * size and its byte offset is known before it is written.
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#include <stdio.h>

#define SYN_E_INVAL (-1)
#define SYN_E_OOM (-3)

/* ------------------------------------------------------------- randomness */

typedef struct { uint64_t s[4]; } rng_t;

static uint64_t splitmix(uint64_t *x) {
    uint64_t z = (*x += 0x9E3779B97F4A7C15ULL);
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ULL;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBULL;
    return z ^ (z >> 31);
}

static void rng_seed(rng_t *r, uint64_t seed, uint64_t purpose, uint64_t index) {
    uint64_t x = seed ^ (purpose * 0xD1B54A32D192ED03ULL) ^ (index * 0x8CB92BA72F3D8DD7ULL);
    for (int i = 0; i < 4; i++) r->s[i] = splitmix(&x);
}

static inline uint64_t rotl(uint64_t x, int k) { return (x << k) | (x >> (64 - k)); }

static uint64_t rng_u64(rng_t *r) {  /* xoshiro256** */
    uint64_t *s = r->s;
    uint64_t res = rotl(s[1] * 5, 7) * 9, t = s[1] << 17;
    s[2] ^= s[0]; s[3] ^= s[1]; s[1] ^= s[2]; s[0] ^= s[3];
    s[2] ^= t; s[3] = rotl(s[3], 45);
    return res;
}

static double rng_unif(rng_t *r) { return (double)(rng_u64(r) >> 11) * (1.0 / 9007199254740992.0); }

static uint64_t rng_below(rng_t *r, uint64_t n) { return n ? rng_u64(r) % n : 0; }

static double rng_normal(rng_t *r) {  /* Box-Muller */
    double u = rng_unif(r), v = rng_unif(r);
    if (u < 1e-300) u = 1e-300;
    return sqrt(-2.0 * log(u)) * cos(6.283185307179586 * v);
}

static const char ACGT[4] = {'A', 'C', 'G', 'T'};

static char comp(char c) {
    switch (c) { case 'A': return 'T'; case 'C': return 'G'; case 'G': return 'C'; case 'T': return 'A'; default: return 'N'; }
}

enum { P_TLEN = 1, P_TSEQ, P_EXPR, P_READ, P_GENE, P_BIN, P_CONTIG, P_COMP };

/* ------------------------------------------------------------ transcripts */

typedef struct {
    uint32_t n;
    uint64_t *off;   /* n+1 offsets into seq */
    char *seq;
    double *cum;     /* cumulative sampling weight (expression x usable length) */
} tx_t;

static void tx_free(tx_t *t) { free(t->off); free(t->seq); free(t->cum); memset(t, 0, sizeof(*t)); }

static int tx_random(tx_t *t, uint64_t seed, uint32_t n, double median, double sigma,
                     uint32_t minlen, uint32_t maxlen) {
    t->n = n;
    t->off = malloc((n + 1) * sizeof(uint64_t));
    if (!t->off) return SYN_E_OOM;
    rng_t r;
    rng_seed(&r, seed, P_TLEN, 0);
    t->off[0] = 0;
    for (uint32_t i = 0; i < n; i++) {
        double L = median * exp(sigma * rng_normal(&r));
        if (L < minlen) L = minlen;
        if (L > maxlen) L = maxlen;
        t->off[i + 1] = t->off[i] + (uint64_t)L;
    }
    t->seq = malloc(t->off[n] + 1);
    if (!t->seq) return SYN_E_OOM;
#pragma omp parallel for schedule(dynamic, 64)
    for (int64_t i = 0; i < (int64_t)n; i++) {
        rng_t q;
        rng_seed(&q, seed, P_TSEQ, (uint64_t)i);
        for (uint64_t j = t->off[i]; j < t->off[i + 1]; j++) t->seq[j] = ACGT[rng_u64(&q) >> 62];
    }
    return 0;
}

/* genes built from shared exons; each isoform keeps a random exon subset */
static int tx_genes(tx_t *t, uint64_t seed, uint32_t n_genes, double exon_median) {
    uint32_t cap = n_genes * 6;
    uint32_t *iso_exons = malloc((size_t)cap * 12 * sizeof(uint32_t));   /* lengths per isoform */
    uint32_t *iso_nex = malloc((size_t)cap * sizeof(uint32_t));
    uint32_t *iso_gene = malloc((size_t)cap * sizeof(uint32_t));
    uint64_t *gene_off = malloc(((size_t)n_genes + 1) * sizeof(uint64_t));
    uint32_t *gene_nex = malloc((size_t)n_genes * sizeof(uint32_t));
    uint32_t *exlen = malloc((size_t)n_genes * 6 * sizeof(uint32_t));
    if (!iso_exons || !iso_nex || !iso_gene || !gene_off || !gene_nex || !exlen) return SYN_E_OOM;
    /* exon structure of every gene */
    gene_off[0] = 0;
    uint32_t niso = 0;
    uint64_t total = 0;
    for (uint32_t g = 0; g < n_genes; g++) {
        rng_t r;
        rng_seed(&r, seed, P_GENE, g);
        uint32_t nex = 2 + (uint32_t)rng_below(&r, 5);
        gene_nex[g] = nex;
        uint64_t glen = 0;
        for (uint32_t e = 0; e < nex; e++) {
            double L = exon_median * exp(0.5 * rng_normal(&r));
            if (L < 30) L = 30;
            if (L > 2000) L = 2000;
            exlen[(size_t)g * 6 + e] = (uint32_t)L;
            glen += (uint32_t)L;
        }
        gene_off[g + 1] = gene_off[g] + glen;
        uint32_t nis = 1 + (uint32_t)rng_below(&r, 6);
        for (uint32_t k = 0; k < nis; k++) {
            uint32_t mask = 0;
            if (k == 0) mask = (1u << nex) - 1;
            else {
                for (uint32_t e = 0; e < nex; e++) if (rng_unif(&r) < 0.75) mask |= 1u << e;
                if (!mask) mask = 1u << rng_below(&r, nex);
            }
            iso_nex[niso] = mask;       /* exon bitmask */
            iso_gene[niso] = g;
            uint64_t L = 0;
            for (uint32_t e = 0; e < nex; e++) if (mask >> e & 1) L += exlen[(size_t)g * 6 + e];
            iso_exons[niso] = (uint32_t)L;
            total += L;
            niso++;
        }
    }
    /* gene sequences */
    char *gseq = malloc(gene_off[n_genes] + 1);
    if (!gseq) return SYN_E_OOM;
#pragma omp parallel for schedule(dynamic, 64)
    for (int64_t g = 0; g < (int64_t)n_genes; g++) {
        rng_t q;
        rng_seed(&q, seed, P_TSEQ, (uint64_t)g);
        for (uint64_t j = gene_off[g]; j < gene_off[g + 1]; j++) gseq[j] = ACGT[rng_u64(&q) >> 62];
    }
    t->n = niso;
    t->off = malloc(((size_t)niso + 1) * sizeof(uint64_t));
    t->seq = malloc(total + 1);
    if (!t->off || !t->seq) return SYN_E_OOM;
    t->off[0] = 0;
    for (uint32_t i = 0; i < niso; i++) {
        uint32_t g = iso_gene[i], mask = iso_nex[i];
        uint64_t w = t->off[i], src = gene_off[g];
        for (uint32_t e = 0; e < gene_nex[g]; e++) {
            uint32_t L = exlen[(size_t)g * 6 + e];
            if (mask >> e & 1) { memcpy(t->seq + w, gseq + src, L); w += L; }
            src += L;
        }
        t->off[i + 1] = w;
    }
    free(gseq); free(iso_exons); free(iso_nex); free(iso_gene); free(gene_off); free(gene_nex); free(exlen);
    return 0;
}

/* sampling weights: log-normal expression x positions a fragment can start at */
static int tx_weights(tx_t *t, uint64_t seed, double sigma, uint32_t min_frag) {
    t->cum = malloc(((size_t)t->n + 1) * sizeof(double));
    if (!t->cum) return SYN_E_OOM;
    rng_t r;
    rng_seed(&r, seed, P_EXPR, 0);
    t->cum[0] = 0;
    for (uint32_t i = 0; i < t->n; i++) {
        uint64_t L = t->off[i + 1] - t->off[i];
        double usable = L >= min_frag ? (double)(L - min_frag + 1) : 0.0;
        t->cum[i + 1] = t->cum[i] + exp(sigma * rng_normal(&r)) * usable;
    }
    return 0;
}

static uint32_t tx_pick(const tx_t *t, rng_t *r) {
    double x = rng_unif(r) * t->cum[t->n];
    uint32_t lo = 0, hi = t->n;
    while (hi - lo > 1) {
        uint32_t mid = (lo + hi) / 2;
        if (t->cum[mid] <= x) lo = mid; else hi = mid;
    }
    return lo;
}

/* copy a read of length L from src (forward or reverse complement), mutate */
static void emit_read(char *dst, const char *src, uint32_t L, int rev, double err, double nrate, rng_t *r) {
    for (uint32_t j = 0; j < L; j++) dst[j] = rev ? comp(src[L - 1 - j]) : src[j];
    for (uint32_t j = 0; j < L; j++) {
        double u = rng_unif(r);
        if (u < err) {
            char c = dst[j];
            int b = c == 'A' ? 0 : c == 'C' ? 1 : c == 'G' ? 2 : 3;
            dst[j] = ACGT[(b + 1 + (int)rng_below(r, 3)) & 3];
        } else if (u < err + nrate) {
            dst[j] = 'N';
        }
    }
}

#define NAME_DIGITS 10

/* Fixed-size record writer.  fastq: "@rNNNNNNNNNN/M\nSEQ\n+\nQUAL\n", else
 * ">rNNNNNNNNNN[/M]\nSEQ\n".  Returns the record size. */
static size_t rec_size(uint32_t L, int fastq, int mate) {
    size_t h = 1 + 1 + NAME_DIGITS + (mate ? 2 : 0) + 1;
    return fastq ? h + L + 1 + 2 + L + 1 : h + L + 1;
}

static char *rec_header(char *p, uint64_t id, int fastq, int mate) {
    char tmp[32];
    *p++ = fastq ? '@' : '>';
    *p++ = 'r';
    snprintf(tmp, sizeof(tmp), "%0*llu", NAME_DIGITS, (unsigned long long)id);
    memcpy(p, tmp, NAME_DIGITS); p += NAME_DIGITS;
    if (mate) { *p++ = '/'; *p++ = (char)('0' + mate); }
    *p++ = '\n';
    return p;
}

static char *rec_tail(char *p, uint32_t L, int fastq) {
    p += L;
    *p++ = '\n';
    if (fastq) {
        *p++ = '+'; *p++ = '\n';
        memset(p, 'I', L); p += L;
        *p++ = '\n';
    }
    return p;
}

/* ------------------------------------------------------------- public API */

void syn_free(void *p) { free(p); }

/* Single-end reads of length read_len from a random transcriptome of
 * n_tx transcripts (log-normal length, median len_median, sigma len_sigma,
 * clipped to [len_min, len_max]); log-normal expression with expr_sigma;
 * uniform starts; 50/50 strand; substitution rate err; N rate nrate. */
int syn_se_reads(uint64_t seed, uint32_t n_tx, double len_median, double len_sigma,
                 uint32_t len_min, uint32_t len_max, double expr_sigma,
                 uint64_t n_reads, uint32_t read_len, double err, double nrate,
                 int fastq, char **out, size_t *out_len, uint64_t *tx_bases) {
    if (!n_tx || !read_len || len_min < read_len) return SYN_E_INVAL;
    tx_t t;
    memset(&t, 0, sizeof(t));
    int e = tx_random(&t, seed, n_tx, len_median, len_sigma, len_min, len_max);
    if (!e) e = tx_weights(&t, seed, expr_sigma, read_len);
    if (e) { tx_free(&t); return e; }
    size_t rs = rec_size(read_len, fastq, 0);
    char *b = malloc(rs * n_reads + 1);
    if (!b) { tx_free(&t); return SYN_E_OOM; }
#pragma omp parallel for schedule(static, 4096)
    for (int64_t i = 0; i < (int64_t)n_reads; i++) {
        rng_t r;
        rng_seed(&r, seed, P_READ, (uint64_t)i);
        uint32_t tx = tx_pick(&t, &r);
        uint64_t L = t.off[tx + 1] - t.off[tx];
        uint64_t start = rng_below(&r, L - read_len + 1);
        int rev = (int)(rng_u64(&r) >> 63);
        char *p = rec_header(b + (size_t)i * rs, (uint64_t)i, fastq, 0);
        emit_read(p, t.seq + t.off[tx] + start, read_len, rev, err, nrate, &r);
        rec_tail(p, read_len, fastq);
    }
    *out = b; *out_len = rs * n_reads;
    if (tx_bases) *tx_bases = t.off[t.n];
    tx_free(&t);
    return 0;
}

/* Paired reads 2 x read_len from n_genes multi-isoform genes (exon length
 * log-normal, median exon_median); fragment ~ normal(frag_mean, frag_sd);
 * left mate forward from the fragment start, right mate reverse complement of
 * its end; pairs flipped 50/50. */
int syn_pe_reads(uint64_t seed, uint32_t n_genes, double exon_median, double expr_sigma,
                 uint64_t n_pairs, uint32_t read_len, double frag_mean, double frag_sd,
                 double err, double nrate, int fastq,
                 char **left, size_t *left_len, char **right, size_t *right_len,
                 uint64_t *tx_bases, uint32_t *n_tx) {
    if (!n_genes || !read_len) return SYN_E_INVAL;
    tx_t t;
    memset(&t, 0, sizeof(t));
    int e = tx_genes(&t, seed, n_genes, exon_median);
    if (!e) e = tx_weights(&t, seed, expr_sigma, read_len);
    if (e) { tx_free(&t); return e; }
    size_t rs = rec_size(read_len, fastq, 1);
    char *lb = malloc(rs * n_pairs + 1), *rb = malloc(rs * n_pairs + 1);
    if (!lb || !rb) { free(lb); free(rb); tx_free(&t); return SYN_E_OOM; }
#pragma omp parallel for schedule(static, 4096)
    for (int64_t i = 0; i < (int64_t)n_pairs; i++) {
        rng_t r;
        rng_seed(&r, seed, P_READ, (uint64_t)i);
        uint32_t tx = tx_pick(&t, &r);
        uint64_t L = t.off[tx + 1] - t.off[tx];
        double f = frag_mean + frag_sd * rng_normal(&r);
        uint64_t F = f < read_len ? read_len : (uint64_t)f;
        if (F > L) F = L;
        uint64_t start = rng_below(&r, L - F + 1);
        const char *frag = t.seq + t.off[tx] + start;
        int flip = (int)(rng_u64(&r) >> 63);
        char *pl = rec_header(lb + (size_t)i * rs, (uint64_t)i, fastq, 1);
        char *pr = rec_header(rb + (size_t)i * rs, (uint64_t)i, fastq, 2);
        emit_read(flip ? pr : pl, frag, read_len, 0, err, nrate, &r);
        emit_read(flip ? pl : pr, frag + F - read_len, read_len, 1, err, nrate, &r);
        rec_tail(pl, read_len, fastq);
        rec_tail(pr, read_len, fastq);
    }
    *left = lb; *right = rb;
    *left_len = rs * n_pairs; *right_len = rs * n_pairs;
    if (tx_bases) *tx_bases = t.off[t.n];
    if (n_tx) *n_tx = t.n;
    tx_free(&t);
    return 0;
}

/* Inchworm-style bundle: n_contigs random contigs (log-normal length, median
 * contig_median, sigma 0.6, clipped to [100, 20000]) grouped into n_comp
 * components of 1..max_per_comp contigs, written as '>s_<id>' records whose
 * contigs are joined by 'X'.  Reads: n_pairs pairs of read_len from the
 * contigs (fragment within one contig) at substitution rate err, written as
 * one FASTA with all left mates, then all right mates (Trinity's both.fa). */
int syn_bundle(uint64_t seed, uint32_t n_contigs, double contig_median,
               uint32_t n_comp, uint32_t max_per_comp, uint64_t n_pairs,
               uint32_t read_len, double err,
               char **bundle, size_t *bundle_len, char **reads, size_t *reads_len,
               uint64_t *contig_bases) {
    if (!n_contigs || !n_comp || n_comp > n_contigs || !read_len) return SYN_E_INVAL;
    tx_t t;
    memset(&t, 0, sizeof(t));
    int e = tx_random(&t, seed, n_contigs, contig_median, 0.6, read_len < 100 ? 100 : read_len, 20000);
    if (!e) e = tx_weights(&t, seed, 1.0, read_len);
    if (e) { tx_free(&t); return e; }
    /* component sizes: each component gets one contig, the rest are spread
     * with sizes capped at max_per_comp */
    uint32_t *csize = calloc(n_comp, sizeof(uint32_t));
    rng_t r;
    rng_seed(&r, seed, P_COMP, 0);
    for (uint32_t c = 0; c < n_comp; c++) csize[c] = 1;
    uint32_t left_over = n_contigs - n_comp;
    while (left_over) {
        uint32_t c = (uint32_t)rng_below(&r, n_comp);
        if (csize[c] < max_per_comp) { csize[c]++; left_over--; }
    }
    /* bundle text: ">s_<c>\n" + contigs joined by X */
    size_t cap = (size_t)t.off[t.n] + (size_t)n_contigs + (size_t)n_comp * 24 + 16;
    char *bb = malloc(cap);
    if (!bb) { free(csize); tx_free(&t); return SYN_E_OOM; }
    size_t m = 0;
    uint32_t ci = 0;
    for (uint32_t c = 0; c < n_comp; c++) {
        m += (size_t)sprintf(bb + m, ">s_%u\n", c);
        for (uint32_t j = 0; j < csize[c]; j++, ci++) {
            if (j) bb[m++] = 'X';
            uint64_t L = t.off[ci + 1] - t.off[ci];
            memcpy(bb + m, t.seq + t.off[ci], L);
            m += L;
        }
        bb[m++] = '\n';
    }
    free(csize);
    size_t rs = rec_size(read_len, 0, 1);
    char *rb = malloc(rs * 2 * n_pairs + 1);
    if (!rb) { free(bb); tx_free(&t); return SYN_E_OOM; }
#pragma omp parallel for schedule(static, 4096)
    for (int64_t i = 0; i < (int64_t)n_pairs; i++) {
        rng_t q;
        rng_seed(&q, seed, P_READ, (uint64_t)i);
        uint32_t tx = tx_pick(&t, &q);
        uint64_t L = t.off[tx + 1] - t.off[tx];
        double f = 300.0 + 50.0 * rng_normal(&q);
        uint64_t F = f < read_len ? read_len : (uint64_t)f;
        if (F > L) F = L;
        uint64_t start = rng_below(&q, L - F + 1);
        const char *frag = t.seq + t.off[tx] + start;
        char *pl = rec_header(rb + (size_t)i * rs, (uint64_t)i, 0, 1);
        char *pr = rec_header(rb + (size_t)(n_pairs + (uint64_t)i) * rs, (uint64_t)i, 0, 2);
        emit_read(pl, frag, read_len, 0, err, 0.0, &q);
        emit_read(pr, frag + F - read_len, read_len, 1, err, 0.0, &q);
        rec_tail(pl, read_len, 0);
        rec_tail(pr, read_len, 0);
    }
    *bundle = bb; *bundle_len = m;
    *reads = rb; *reads_len = rs * 2 * n_pairs;
    if (contig_bases) *contig_bases = t.off[t.n];
    tx_free(&t);
    return 0;
}

/* Power-law read bins: n_bins bins whose read counts follow a power law with
 * exponent alpha on [min_reads, max_reads]; bin b draws read_len reads from
 * its own locus of 1..20 random transcripts (median 1,500 nt) at error err.
 * All bins are written back to back as FASTA; bin_off[b] is the byte offset of
 * bin b (n_bins + 1 entries, caller-allocated). */
int syn_bins(uint64_t seed, uint32_t n_bins, double alpha, uint32_t min_reads,
             uint32_t max_reads, uint32_t read_len, double err,
             char **out, size_t *out_len, uint64_t *bin_off, uint64_t *bin_reads) {
    if (!n_bins || min_reads < 1 || max_reads < min_reads || !read_len) return SYN_E_INVAL;
    rng_t r;
    rng_seed(&r, seed, P_BIN, 0);
    size_t rs = rec_size(read_len, 0, 0);
    uint64_t total = 0;
    double a1 = 1.0 - alpha;
    double lo = pow((double)min_reads, a1), hi = pow((double)max_reads + 1.0, a1);
    for (uint32_t b = 0; b < n_bins; b++) {
        double u = rng_unif(&r);
        double x = pow(lo + u * (hi - lo), 1.0 / a1);   /* inverse CDF of the power law */
        uint64_t n = (uint64_t)x;
        if (n < min_reads) n = min_reads;
        if (n > max_reads) n = max_reads;
        bin_reads[b] = n;
        bin_off[b] = total * rs;
        total += n;
    }
    bin_off[n_bins] = total * rs;
    char *buf = malloc(total * rs + 1);
    if (!buf) return SYN_E_OOM;
    uint64_t first = 0;
    int err_code = 0;
    for (uint32_t b = 0; b < n_bins; b++) {
        rng_t q;
        rng_seed(&q, seed, P_BIN, 1 + (uint64_t)b);
        uint32_t nt = 1 + (uint32_t)rng_below(&q, 20);
        tx_t t;
        memset(&t, 0, sizeof(t));
        int e = tx_random(&t, seed ^ (0x5BD1E995ULL * (b + 1)), nt, 1500.0, 0.5, read_len + 50, 8000);
        if (!e) e = tx_weights(&t, seed ^ (0x5BD1E995ULL * (b + 1)), 1.5, read_len);
        if (e) { tx_free(&t); err_code = e; break; }
#pragma omp parallel for schedule(static, 2048)
        for (int64_t i = 0; i < (int64_t)bin_reads[b]; i++) {
            rng_t z;
            rng_seed(&z, seed, P_READ, first + (uint64_t)i);
            uint32_t tx = tx_pick(&t, &z);
            uint64_t L = t.off[tx + 1] - t.off[tx];
            uint64_t start = rng_below(&z, L - read_len + 1);
            int rev = (int)(rng_u64(&z) >> 63);
            char *p = rec_header(buf + (first + (uint64_t)i) * rs, first + (uint64_t)i, 0, 0);
            emit_read(p, t.seq + t.off[tx] + start, read_len, rev, err, 0.0, &z);
            rec_tail(p, read_len, 0);
        }
        first += bin_reads[b];
        tx_free(&t);
    }
    if (err_code) { free(buf); return err_code; }
    *out = buf; *out_len = total * rs;
    return 0;
}
