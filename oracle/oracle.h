/*
 * oracle.h -- CPU restatement of Trinity's k-mer hot path.
 *
 * TEST INFRASTRUCTURE ONLY.  Nothing in the shipped library, the command-line
 * tools or the serving daemon links, loads or calls this code.  Only the test
 * suite, __graft_entry__.smoke() and bench.py's CPU-baseline leg use it, and
 * there only as the checker / the timed CPU reference.
 *
 * Parity status: the reference's own implementations of these three tools are
 * NOT part of the reference checkout (Inchworm and Chrysalis are empty git
 * submodules, .gitmodules:8-13; jellyfish is an external binary pinned to
 * 2.3.0, Docker/Dockerfile:179-183).  The counting semantics are pinned against
 * the reference's own Perl k-mer counter (util/misc/kmer_counter.pl with
 * PerlLib/Ktree.pm) and window enumerator (util/misc/print_kmers.pl) through
 * committed golden fixtures; the histogram format against
 * util/misc/insilico_norm_kmer_hists/kmer_histo.all.txt; the coverage-stats
 * and readsToComponents column layouts against their live Perl consumers
 * (util/support_scripts/nbkc_merge_left_right_stats.pl, nbkc_normalize.pl,
 * Trinity:2471-2497, partition_chrysalis_graphs_n_reads.pl:98-118).
 * The arithmetic of the statistics (median of an even count, mean/stdev
 * formula and print precision) and the ReadsToTranscripts vote rules are not
 * pinned by anything in the reference tree: "parity unpinned" for those, and
 * the decisions below are documented ones.
 */
#ifndef TRINKMER_ORACLE_H
#define TRINKMER_ORACLE_H
#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Count every k-mer of every record (FASTA or FASTQ).  canonical != 0 merges a
 * k-mer with its reverse complement under the smaller 2-bit code (jellyfish
 * count --canonical, called at Trinity:2612-2619).  Output sorted by key when
 * sorted != 0, else in hash-table order.  Returns 0 or a negative error. */
int orc_count(const char *text, size_t len, int k, int canonical, int threads,
              int sorted, uint64_t **keys, uint32_t **counts, uint64_t *n);
/* orc_count with its table sized for about distinct_hint distinct k-mers
 * (0: for as many as there are windows); -5 when the hint was too small. */
int orc_count_sized(const char *text, size_t len, int k, int canonical, int threads, int sorted,
                    uint64_t distinct_hint, uint64_t **keys, uint32_t **counts, uint64_t *n);

/* jellyfish histo --low low --high high: hist[0] = counts < low,
 * hist[1 + c - low] for low <= c <= high, hist[high - low + 2] = counts > high. */
void orc_histo(const uint32_t *counts, uint64_t n, uint64_t low, uint64_t high,
               uint64_t *hist);

/* jellyfish dump -L min_count: ">COUNT\nKMER\n" records in array order. */
int orc_dump(const uint64_t *keys, const uint32_t *counts, uint64_t n, int k,
             uint32_t min_count, char **out, size_t *out_len);

/* Parse a dump back into (key, count) pairs sorted by key; canonical != 0
 * canonicalises each k-mer (fastaToKmerCoverageStats --DS lookups). */
int orc_load_dump(const char *text, size_t len, int k, int canonical,
                  uint64_t **keys, uint32_t **counts, uint64_t *n);

/* fastaToKmerCoverageStats: one row per read (input order) after a header row.
 * keys/counts: sorted table from orc_count or orc_load_dump. */
int orc_cov_stats(const char *reads, size_t len, const uint64_t *keys,
                  const uint32_t *counts, uint64_t n, int k, int ds,
                  int capture, int threads, char **out, size_t *out_len);

/* Raw per-read statistics (no text), for bit-level comparisons. */
int orc_cov_values(const char *reads, size_t len, const uint64_t *keys,
                   const uint32_t *counts, uint64_t n, int k, int ds,
                   int threads, uint64_t *n_reads, uint32_t **median,
                   float **mean, float **stdev);

/* ReadsToTranscripts: rows "comp\t>acc\tpct\tSEQ\n" in read order. */
int orc_r2t(const char *reads, size_t rlen, const char *bundle, size_t blen,
            int k, int strand, int min_pct, int threads, char **out,
            size_t *out_len);

/* Raw per-read assignment: comp record index (-1 = unassigned), hits, windows. */
int orc_r2t_values(const char *reads, size_t rlen, const char *bundle,
                   size_t blen, int k, int strand, int threads,
                   uint64_t *n_reads, int32_t **rec, uint32_t **hits,
                   uint32_t **nwin);

/* "acc\tsequence\n" per parsed record (the parse the other calls use). */
int orc_records(const char *text, size_t len, char **out, size_t *out_len);

/* FASTQ -> FASTA as util/support_scripts/fastQ_to_fastA.pl prints it (see
 * oracle.c): append >= 0 adds "/append" (-a), flags ORC_FA_*; on a poorly
 * formed record returns ORC_E_PARSE with *bad = its 1-based number unless
 * ORC_FA_IGNORE_DIRTY. */
#define ORC_FA_REV 1
#define ORC_FA_IGNORE_DIRTY 2
#define ORC_FA_IF_MISSING 4
int orc_fastq_to_fasta(const char *text, size_t len, int append, int flags, char **out, size_t *out_len,
                       uint64_t *bad);

/* The normalization tail of util/insilico_read_normalization.pl (see
 * oracle.c): left/right are coverage-stats tables as fastaToKmerCoverageStats
 * prints them (header row first, any row order); right == NULL selects on one
 * side alone.  *table = the table nbkc_normalize.pl reads (the merged pairs
 * from nbkc_merge_left_right_stats.pl --sorted, or the sorted stats); *accs =
 * what nbkc_normalize.pl prints; counts = {rows, selected, aberrant, below
 * min_cov}. */
int orc_norm(const char *left, size_t llen, const char *right, size_t rlen, int max_cov, int min_cov, int max_cv,
             char **table, size_t *table_len, char **accs, size_t *accs_len, uint64_t counts[4]);

/* The FASTQ records whose core names the accs text selects, verbatim and in
 * input order (make_normalized_reads_file); ORC_E_PARSE with *missing > 0
 * when a selected name has no record. */
int orc_norm_extract(const char *fq, size_t len, const char *accs, size_t alen, char **out, size_t *out_len,
                     uint64_t *missing);

void orc_free(void *p);

/* FastaToDeBruijn --graph_per_record -K K [--SS] text (decision D8 in
 * oracle.c): per bundle record "Component <id>" and one line per distinct
 * (K+1)-mer in order of first occurrence. */
int orc_debruijn(const char *bundle, size_t blen, int K, int ss, int threads, char **out, size_t *out_len);

#ifdef __cplusplus
}
#endif
#endif
