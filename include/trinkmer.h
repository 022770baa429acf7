/*
 * trinkmer.h -- C ABI of the GB300 k-mer library (libtrinkmer_cuda.so).
 *
 * The reference reaches this hot path only through three executables that
 * Perl starts with system() (PerlLib/Pipeliner.pm:143-209,
 * util/insilico_read_normalization.pl:797-813, Trinity:2910): jellyfish
 * (Trinity:2612-2638), Inchworm's fastaToKmerCoverageStats
 * (util/insilico_read_normalization.pl:837-846) and Chrysalis'
 * ReadsToTranscripts (Trinity:2237-2251).  There is no library interface in
 * the reference, so this ABI is the one the drop-in executables of this
 * package (tools/) and any foreign-language caller bind; each group below
 * names the command it replaces.
 *
 * Conventions: every function returns TK_OK (0) or a negative TK_E_* status;
 * no C++ exception crosses the ABI; handles are opaque and owned by the
 * library, which also owns all device memory.  Buffers passed in are owned by
 * the caller and described by (pointer, length); `where` says whether a
 * buffer is host memory (TK_HOST) or device memory of the context's GPU
 * (TK_DEVICE).  A handle is used by one thread at a time.  All work of one
 * context is ordered on that context's CUDA stream; functions that return
 * host data synchronise it.
 */
#ifndef TRINKMER_H
#define TRINKMER_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define TK_OK 0
#define TK_E_INVAL (-1)       /* bad argument */
#define TK_E_CUDA (-2)        /* CUDA runtime error */
#define TK_E_OOM (-3)         /* device or host allocation failed */
#define TK_E_PARSE (-4)       /* malformed FASTA/FASTQ/dump input */
#define TK_E_TABLE_FULL (-5)  /* hash table overflow could not be resolved */
#define TK_E_BUDGET (-6)      /* job does not fit the HBM admission budget */
#define TK_E_NODEV (-7)       /* no usable CUDA device */
#define TK_E_RANGE (-8)       /* caller buffer too small */

#define TK_HOST 0
#define TK_DEVICE 1

#define TK_FMT_NONE 0
#define TK_FMT_FASTA 1
#define TK_FMT_FASTQ 2

/* kernel classes for tk_ctx_profile */
#define TK_KID_PARSE 0        /* FASTA/FASTQ split + pack */
#define TK_KID_HLL 1          /* distinct-k-mer estimate (table sizing) */
#define TK_KID_COUNT 2        /* k-mer count insert */
#define TK_KID_COMPACT 3      /* table scan: -L filter + histogram */
#define TK_KID_SORT 4         /* radix sort of keys */
#define TK_KID_DUMP 5         /* dump text formatter */
#define TK_KID_LOAD 6         /* k-mer catalogue load */
#define TK_KID_COVERAGE 7     /* per-read coverage statistics */
#define TK_KID_R2T_BUILD 8    /* bundle k-mer -> record table */
#define TK_KID_R2T_ASSIGN 9   /* read -> component vote */
#define TK_KID_BINS 10        /* batched per-bin counting */
#define TK_KID_SCATTER 11     /* k-mers into hash-partition buckets (count pass 1) */
#define TK_KID_NORM 12        /* normalization: name sort, pair merge, selection */
#define TK_KID_EXTRACT 13     /* normalization: selected FASTQ records */
#define TK_KID_COV_CACHE 14   /* coverage: the L2-resident cache of the most frequent k-mers */
#define TK_KID_DBG 15         /* per-record de Bruijn graphs of a bundle */
#define TK_KID_NUM 16         /* number of kernel classes */

typedef struct tk_ctx tk_ctx;
typedef struct tk_reads tk_reads;
typedef struct tk_table tk_table;
typedef struct tk_r2t tk_r2t;

/* ------------------------------------------------------------- context */

const char *tk_version(void);
const char *tk_status_string(int status);

/* Creates a context on CUDA device `device` with its own stream. */
int tk_ctx_create(int device, tk_ctx **out);
void tk_ctx_destroy(tk_ctx *ctx);
/* Human-readable detail of the context's most recent error. */
const char *tk_ctx_last_error(const tk_ctx *ctx);
/* The context's cudaStream_t, as an opaque pointer. */
void *tk_ctx_stream(tk_ctx *ctx);
int tk_ctx_synchronize(tk_ctx *ctx);
/* CUDA-event timing of the hot kernels on the context's stream: per kernel
 * class, the milliseconds between events recorded around its launches, the
 * number of kernels launched inside those brackets, and its work units. */
int tk_ctx_set_profiling(tk_ctx *ctx, int on);
int tk_ctx_profile(tk_ctx *ctx, int kid, double *ms, uint64_t *launches, uint64_t *units);
int tk_ctx_reset_profile(tk_ctx *ctx);
/* Number of kernels this library has launched on the context. */
uint64_t tk_ctx_kernel_launches(const tk_ctx *ctx);
/* Bytes of device memory currently free / total on the context's GPU. */
int tk_ctx_mem_info(tk_ctx *ctx, uint64_t *free_bytes, uint64_t *total_bytes);
/* Measured random-access ceiling of this GPU: independent random 8-byte
 * accesses per second into a table of about table_bytes (loads, or with
 * atomics != 0 the CAS probe + red.add pair of a count insert).  The
 * roofline denominator for the hash-table kernels. */
int tk_ctx_random_access_rate(tk_ctx *ctx, uint64_t table_bytes, int atomics, double *accesses_per_s);
/* Device blocks of 256 MB and more are kept by the context after they are
 * freed, for the next request of about the same size (up to 128 GB cached per
 * process, or TRINKMER_BLOCK_CACHE_GB); this gives them back to the driver. */
int tk_ctx_trim(tk_ctx *ctx);
/* Probe limit of the hash tables before a key is sent to the overflow list
 * and the table grows (jellyfish count -p/--reprobes; default 4096). */
int tk_ctx_set_reprobes(tk_ctx *ctx, int max_probes);

/* ------------------------------------------------------------- read sets
 * Parse FASTA (PerlLib/Fasta_reader.pm:45-118 semantics: a record starts at a
 * '>' line, its sequence is the following lines with whitespace removed, its
 * accession is the first header token) or 4-line FASTQ
 * (util/support_scripts/fastQ_to_fastA.pl:80-106) into a device-resident read
 * set.  The text is copied to the device when where == TK_HOST; a TK_DEVICE
 * text must stay valid while the read set lives. */
int tk_reads_parse(tk_ctx *ctx, const char *text, uint64_t len, int where, tk_reads **out);
/* Parses n texts into n read sets (out[i] from texts[i]).  With TK_HOST every
 * upload is queued on the context's copy stream first and text i is parsed as
 * soon as its own upload lands, so the uploads of the later texts overlap the
 * parsing of the earlier ones (page-locked host memory lets them run
 * concurrently).  Replaces the one-file-at-a-time read loading of the tools
 * above (no counterpart in the reference's interface: each of its tools reads
 * its FASTA itself).  On error no read set is returned. */
int tk_reads_parse_many(tk_ctx *ctx, const char *const *texts, const uint64_t *lens, uint32_t n, int where,
                        tk_reads **out);
/* Host-only: n_chunks + 1 offsets (cuts[0] = 0, cuts[n_chunks] = len,
 * non-decreasing) that split a FASTA or FASTQ host text into n_chunks pieces
 * of about equal size, each cut at the start of a record ('>' line; for FASTQ
 * an '@' line whose next-but-one line starts with '+').  The pieces parse to
 * the same reads, in order, as the whole text; with tk_reads_parse_many the
 * upload of one piece overlaps the parse of the one before.  Only the bytes
 * around each cut are read.  No counterpart in the reference. */
int tk_split_records(const char *text, uint64_t len, uint32_t n_chunks, uint64_t *cuts);
/* FASTQ -> FASTA read prep (the conversion Trinity runs before counting:
 * `seqtk-trinity seq -A -R {1,2} [-r]`, Trinity:2745-2805; its executable spec
 * is util/support_scripts/fastQ_to_fastA.pl:60-118).  For a read set parsed
 * from FASTQ: ">name[/1|/2][/append]\nSEQUENCE\n" per record, the name the
 * header's first field, "/1" or "/2" from a Casava "1:"/"2:" comment, the
 * sequence line as written (case kept; only the header loses CRs).  append
 * = -1 adds nothing, N >= 0 adds "/N" (the script's -a N), with
 * TK_FA_IF_MISSING only to names not already ending in /1 or /2 (what
 * seqtk-trinity -R N is for).  TK_FA_REVCOMP reverse-complements
 * (PerlLib/Nuc_translator.pm:286-292).  A poorly formed record (sequence
 * empty or "0", quality blank or of another length) fails with TK_E_PARSE
 * unless TK_FA_IGNORE_DIRTY skips it.  out == NULL reports the length only;
 * the text is kept with the read set for the next call with the same
 * options. */
#define TK_FA_REVCOMP 1
#define TK_FA_IGNORE_DIRTY 2
#define TK_FA_IF_MISSING 4
int tk_reads_to_fasta(tk_reads *reads, int append, int flags, int where, char *out, uint64_t cap, uint64_t *len_out);
int tk_reads_info(const tk_reads *reads, uint64_t *n_reads, uint64_t *n_bases,
                  uint32_t *max_len, int *format);
/* Host copies: accession offset/length into the parsed text (n_reads each). */
int tk_reads_names(const tk_reads *reads, uint64_t *name_off, uint32_t *name_len);
/* Host copies of read starts in the packed sequence (n_reads + 1 entries) and
 * of the packed sequence itself (upper-cased bases, '\n' after each read). */
int tk_reads_offsets(const tk_reads *reads, uint64_t *rd_off);
int tk_reads_copy_seq(const tk_reads *reads, char *dst, uint64_t cap);
void tk_reads_free(tk_reads *reads);

/* ------------------------------------------------------------- counting
 * Replaces `jellyfish count -m K [--canonical] -s H -t N -o db reads.fa`
 * (Trinity:2612-2621, util/insilico_read_normalization.pl:617-626),
 * `jellyfish histo` (Trinity:2630, util/insilico_read_normalization.pl:636)
 * and `jellyfish dump -L m` (Trinity:2625, util/insilico_read_normalization.pl:641).
 * A k-mer is k consecutive A/C/G/T (either case); canonical keys are the
 * smaller of a k-mer and its reverse complement in 2-bit A<C<G<T order.
 * capacity_hint = 0 sizes the table from a distinct-k-mer estimate of each
 * batch; the table grows (rehash) whenever it would exceed half load. */
int tk_table_create(tk_ctx *ctx, int k, int canonical, uint64_t capacity_hint, tk_table **out);
int tk_table_add_reads(tk_table *table, const tk_reads *reads);
/* Adds several read sets in one pass over the table (e.g. both mate files:
 * jellyfish counts `cat left.fa right.fa`, Trinity:1641). */
int tk_table_add_reads_multi(tk_table *table, const tk_reads *const *sets, uint32_t n_sets);
/* tk_reads_parse_many followed by tk_table_add_reads_multi, overlapped: with
 * host texts every upload is queued at once, and each text's first counting
 * pass (its windows' bucket histogram, distinct-k-mer sketch and bucketing)
 * runs as soon as the text is parsed, while the later texts still upload;
 * the second pass then counts all of them into the table.  The n read sets
 * are returned in `out` (the caller frees them); on error none is.  The
 * counts equal those of tk_table_add_reads_multi.  No counterpart in the
 * reference (jellyfish reads its files itself). */
int tk_table_count_texts(tk_table *table, const char *const *texts, const uint64_t *lens, uint32_t n, int where,
                         tk_reads **out);
int tk_table_count_text(tk_table *table, const char *text, uint64_t len, int where);
/* distinct k-mers (a scan of the table; pass NULL to skip it), occurrences
 * added, slots. */
int tk_table_info(tk_table *table, uint64_t *distinct, uint64_t *total, uint64_t *capacity);
/* hist[0] = keys with count < low, hist[1 + c - low] for low <= c <= high,
 * hist[high - low + 2] = keys with count > high (high - low + 3 entries). */
int tk_table_histo(tk_table *table, uint64_t low, uint64_t high, uint64_t *hist);
/* (key, count) pairs with count >= min_count sorted by key.  keys == NULL
 * only reports *n_out.  TK_E_RANGE when cap < the number of pairs. */
int tk_table_dump(tk_table *table, uint32_t min_count, int where, uint64_t *keys,
                  uint32_t *counts, uint64_t cap, uint64_t *n_out);
/* The dump as text, ">COUNT\nKMER\n" per pair, sorted by key, into `out`
 * (host or device memory per `where`).  out == NULL formats the dump on the
 * device and only reports *len_out; the formatted text is kept with the
 * table, so the following call with a buffer copies it without recomputing
 * (until the table changes). */
int tk_table_dump_fasta(tk_table *table, uint32_t min_count, int where, char *out, uint64_t cap,
                        uint64_t *len_out);
/* tk_table_dump_fasta into host memory without waiting for the copy: the text
 * is formatted on the GPU, then copied to `out` on the context's copy stream
 * while later work on the context runs.  `out` (page-locked for the copy to
 * overlap) holds the text once tk_ctx_synchronize returns; freeing or changing
 * the table before then is safe.  *len_out is set at once. */
int tk_table_dump_fasta_async(tk_table *table, uint32_t min_count, char *out, uint64_t cap, uint64_t *len_out);
/* Adds (key, count) pairs (a stored database, or another table's dump). */
int tk_table_load_pairs(tk_table *table, const uint64_t *keys, const uint32_t *counts,
                        uint64_t n, int where);
/* Adds the pairs of a ">COUNT\nKMER\n" dump (fastaToKmerCoverageStats --kmers;
 * canonicalised when the table is canonical, i.e. --DS). */
int tk_table_load_dump_fasta(tk_table *table, const char *text, uint64_t len, int where);
void tk_table_free(tk_table *table);

/* ------------------------------------------------------------- coverage
 * Replaces Inchworm's `fastaToKmerCoverageStats --reads R --kmers K
 * --kmer_size 25 [--DS]` (util/insilico_read_normalization.pl:837-846).  Per
 * read, over its windows of k A/C/G/T bases, each k-mer's count in `table`
 * (canonical lookup when the table is canonical; a k-mer absent from the
 * table counts 1, Changelog.txt:536-538): median = element n/2 of the sorted
 * counts, mean = (float)(sum / n), stdev = population standard deviation
 * from exact integer sums; 0, 0, 0 for a read with no window.  Outputs hold
 * n_reads entries each, in read order. */
int tk_coverage_stats(tk_table *table, const tk_reads *reads, int where, uint32_t *median,
                      float *mean, float *stdev);

/* tk_coverage_stats without any device allocation.  No counterpart in the
 * reference: it exists for callers that cannot allocate device memory while
 * they compute -- a resident service whose HBM is already divided into job
 * slots under an admission budget, or a pipeline that must not meet an
 * allocation failure or the implicit synchronisation of cudaMalloc/cudaFree
 * mid-run.  The table and read set are created beforehand (that is where
 * their memory is allocated); median/mean/stdev are DEVICE arrays of n_reads
 * entries owned by the caller.  Reads longer than 256 windows use a fixed
 * 16 MiB slab of static device memory, which limits a read to 131,072
 * windows (TK_E_RANGE beyond that).  The slab is part of the library's
 * device code for the coverage kernels: a GPU commits it when that code is
 * loaded there and holds it until the process exits.  Under CUDA's lazy
 * module loading (the default) that can be the first call of this entry
 * point on the device, which also looks up the slab's address -- so make a
 * first call (an empty read set will do) before dividing the GPU's memory
 * among jobs.  All calls share the slab: calls that overlap on the GPU race.
 * Returns after synchronising the context's stream. */
int tk_coverage_stats_noalloc(tk_table *table, const tk_reads *reads, uint32_t *median,
                              float *mean, float *stdev);

/* ------------------------------------------------------------- read -> component
 * Replaces Chrysalis' `ReadsToTranscripts -i reads.fa -f bundle.fasta -o out
 * -t N -max_mem_reads M [-strand] [-p P]` (Trinity:2237-2251).  The bundle is
 * FASTA with one '>s_<component>' record per component whose contigs are
 * joined by 'X' (util/support_scripts/add_LR_reads_to_iworm_bundle.pl:19-47).
 * Each bundle k-mer belongs to the first record holding it; a read votes once
 * per window for the owner of the window's k-mer; rec = the record with most
 * votes (ties to the earlier record) or -1 without any vote; hits = its votes;
 * nwin = L - k + 1 (0 when L < k). */
int tk_r2t_create(tk_ctx *ctx, const char *bundle, uint64_t len, int where, int k,
                  int strand, tk_r2t **out);
int tk_r2t_info(const tk_r2t *r2t, uint64_t *n_records, uint64_t *n_kmers);
/* Component id (the integer after "s_", else the record ordinal) per record. */
int tk_r2t_component_ids(const tk_r2t *r2t, uint64_t *ids);
int tk_r2t_assign(tk_r2t *r2t, const tk_reads *reads, int where, int32_t *rec,
                  uint32_t *hits, uint32_t *nwin);
void tk_r2t_free(tk_r2t *r2t);

/* ------------------------------------------------------------- de Bruijn graphs
 * Replaces Inchworm's `FastaToDeBruijn --fasta bundled_iworm_contigs.fasta
 * -K (k-1) --graph_per_record [--SS]` (Trinity:2298-2302), whose output
 * util/support_scripts/partition_chrysalis_graphs_n_reads.pl cuts into one
 * graph file per component.  Per bundle record (format as for
 * tk_r2t_create) that has at least one window of K+1 A/C/G/T bases:
 * "Component <id>\n" (id as tk_r2t_component_ids), then one line per
 * distinct (K+1)-mer of the record in order of first occurrence,
 * "<node>\t<prev>\t<count>\t<kmer>\n": node = 0, 1, ... in that order;
 * prev = the node of the window just before the first occurrence, -1 when
 * that is not a window of K+1 A/C/G/T (contig start, 'X' join); count =
 * occurrences in the record, a (K+1)-mer and its reverse complement counted
 * as one node unless `strand`; kmer = the first occurrence, upper case.
 * The header line and one line per k-mer are what the partition script reads
 * (partition_chrysalis_graphs_n_reads.pl:197-223); the node line's columns
 * are this library's (the tool's source is not in the reference).  K is
 * 1..30. */
typedef struct tk_dbg tk_dbg;
int tk_dbg_create(tk_ctx *ctx, const char *bundle, uint64_t len, int where, int K, int strand, tk_dbg **out);
/* components written (records with a window), nodes (= node lines), text bytes */
int tk_dbg_info(const tk_dbg *dbg, uint64_t *n_components, uint64_t *n_nodes, uint64_t *text_len);
int tk_dbg_text(const tk_dbg *dbg, int where, char *out, uint64_t cap);
void tk_dbg_free(tk_dbg *dbg);

/* ------------------------------------------------------------- normalization
 * Replaces what util/insilico_read_normalization.pl does with the coverage
 * statistics of the reads (Trinity:3421-3479 runs it with --pairs_together for
 * paired reads): each side's stats table sorted by read name
 * (`sort -k1,1` under LC_ALL=C, insilico:865-892), the two sorted tables
 * merged by util/support_scripts/nbkc_merge_left_right_stats.pl --sorted
 * (insilico:951-965), the rows selected by nbkc_normalize.pl --max_cov
 * --min_cov --max_CV (insilico:972-977; a side alone, right == NULL, as
 * insilico:917-947 does for single-end reads), and the selected reads
 * extracted from the FASTQ input (make_normalized_reads_file,
 * insilico:470-584).
 *
 * tk_norm_select takes the read sets the statistics belong to (their names;
 * both must stay alive while the tk_norm is used) and their per-read median,
 * mean and stdev as tk_coverage_stats writes them (`where`: TK_HOST or
 * TK_DEVICE arrays of n_reads entries).  The tables it works on are the ones
 * fastaToKmerCoverageStats prints (acc, "%u", "%g", "%g"), so the result is
 * the reference scripts' output on those tables byte for byte: rows in
 * sorted-name order, the merge's two-cursor pairing, averages through
 * "%.1f", nbkc_normalize.pl's srand(12345) draw sequence (Perl's drand48).
 * A mean or stdev outside [1e-17, 1.8e19) (other than 0), or a selected row
 * with median 0 (min_cov <= 0; Perl dies dividing by it), is TK_E_INVAL. */
typedef struct tk_norm tk_norm;
typedef struct tk_norm_counts {
    uint64_t rows;        /* rows nbkc_normalize.pl read (merged pairs, or reads) */
    uint64_t selected;    /* accs printed */
    uint64_t aberrant;    /* mean <= 0 or stdev/mean > max_CV */
    uint64_t below_min;   /* median < min_cov */
} tk_norm_counts;
int tk_norm_select(tk_ctx *ctx, const tk_reads *left, const uint32_t *left_median, const float *left_mean,
                   const float *left_stdev, const tk_reads *right, const uint32_t *right_median,
                   const float *right_mean, const float *right_stdev, int where, int max_cov, int min_cov,
                   int max_cv, tk_norm **out);
/* tk_norm_select over a side whose reads are split across several read sets
 * (e.g. record-aligned pieces of one file, tk_split_records): the side's
 * reads are the sets' reads in order, and its statistics arrays hold them in
 * that order.  No counterpart in the reference (its scripts read whole files). */
int tk_norm_select_multi(tk_ctx *ctx, const tk_reads *const *left, uint32_t n_left, const uint32_t *left_median,
                         const float *left_mean, const float *left_stdev, const tk_reads *const *right,
                         uint32_t n_right, const uint32_t *right_median, const float *right_mean,
                         const float *right_stdev, int where, int max_cov, int min_cov, int max_cv, tk_norm **out);
/* counts and the byte length of the accs text */
int tk_norm_info(const tk_norm *norm, tk_norm_counts *counts, uint64_t *accs_len);
/* nbkc_normalize.pl's output: one selected acc per line (without "/1" or "/2") */
int tk_norm_accs(const tk_norm *norm, int where, char *out, uint64_t cap);
/* The table nbkc_normalize.pl reads: pairs.K25.stats as
 * nbkc_merge_left_right_stats.pl writes it, or a side's sorted stats table
 * (header row first).  out == NULL returns the length only. */
int tk_norm_table(tk_norm *norm, int where, char *out, uint64_t cap, uint64_t *len);
/* The records of `fastq` whose core names the selection holds, in input
 * order: FASTQ records verbatim (the name rules of
 * PerlLib/Fastq_reader.pm:106-121 and insilico:452-466, 529-531), or for a
 * FASTA read set ">header\nsequence\n" as PerlLib/Fasta_reader.pm:45-70 and
 * Sequence::get_FASTA_format print them (insilico:518-527).  The text is kept
 * in the tk_norm until the next call.  A selected name without a record is
 * TK_E_PARSE (the script dies with "not all specified records have been
 * retrieved"); a FASTA accession longer than 256 bytes is TK_E_RANGE. */
int tk_norm_extract(tk_norm *norm, const tk_reads *fastq, uint64_t *len);
/* The same over one side's reads split across several read sets (files or
 * record-aligned pieces, in order): their records back to back, and a
 * selected name counts as found when any of them carries it
 * (make_normalized_reads_file reads all files of a side, insilico:502-545). */
int tk_norm_extract_multi(tk_norm *norm, const tk_reads *const *sets, uint32_t n_sets, uint64_t *len);
int tk_norm_extract_copy(const tk_norm *norm, int where, char *out, uint64_t cap);
/* tk_norm_extract_copy into host memory without waiting: the extracted text
 * is copied to `out` on the context's copy stream while later work on the
 * context runs (e.g. the other side's tk_norm_extract).  `out` (page-locked
 * for the copy to overlap) holds the text once tk_ctx_synchronize returns; a
 * later extraction does not wait for the copy (the earlier device text is
 * kept until its copy has ended), and tk_norm_free orders the context's
 * later work after it.  No counterpart in the reference (make_normalized_reads_file
 * writes each side's file in turn, insilico:470-584). */
int tk_norm_extract_copy_async(tk_norm *norm, char *out, uint64_t cap);
void tk_norm_free(tk_norm *norm);

/* ------------------------------------------------------------- batched bins
 * Replaces the per-bin k-mer counting of Trinity's phase 2 (one
 * `Trinity --single c<comp>.trinity.reads.fa --trinity_complete` per read bin,
 * fanned out by ParaFly, Trinity:3628-3735; each counts its own k-mers,
 * Trinity:2669-2672) with one batched GPU pass.  `text` holds every bin's
 * FASTA back to back; bin b is the records whose header starts in
 * [bin_off[b], bin_off[b+1]) (n_bins + 1 offsets).  Each bin is counted in its
 * own table slice (sized per bin from a sketch, block shape autotuned) by one
 * persistent, CUDA-graph-captured launch, and its ">COUNT\nKMER\n" dump
 * (count >= min_count, sorted by key) is bytes [off[b], off[b+1]) of the
 * result text -- the same bytes as a separate tk_table_dump_fasta of that bin. */
typedef struct tk_bins tk_bins;
int tk_count_bins(tk_ctx *ctx, const char *text, uint64_t len, int where, const uint64_t *bin_off,
                  uint32_t n_bins, int k, int canonical, uint32_t min_count, tk_bins **out);
/* The same with a minimum count per bin (min_counts[n_bins]) and, when
 * `histos` is not NULL, each bin's tk_table_histo(1, 10000) histogram
 * (histos[b * 10002 + i]).  Bins may be FASTQ. */
int tk_count_bins_ex(tk_ctx *ctx, const char *text, uint64_t len, int where, const uint64_t *bin_off,
                     uint32_t n_bins, int k, int canonical, const uint32_t *min_counts, uint64_t *histos,
                     tk_bins **out);
/* total dump bytes and k-mer windows counted */
int tk_bins_info(const tk_bins *bins, uint64_t *text_len, uint64_t *kmers);
/* n_bins + 1 byte offsets of each bin's dump in the text */
int tk_bins_dump_offsets(const tk_bins *bins, uint64_t *offsets);
int tk_bins_dump_text(const tk_bins *bins, char *dst, uint64_t cap);
/* How the batch was counted: the count kernel's block size and the slices'
 * load factor (per mille), both tuned once per device (the load factor on
 * the first batch of at least 50M k-mers, by timing 0.45, 0.6 and 0.75), and
 * how many times overflowing slices were doubled and the count relaunched.
 * The dumps do not depend on any of them. */
int tk_bins_tuning(const tk_bins *bins, int *block, int *load_per_mille, int *relaunches);
void tk_bins_free(tk_bins *bins);

/* ------------------------------------------------------------- serving
 * A resident job server: `slots` worker slots, each with its own context and
 * stream, and an HBM admission budget (0 = 80% of the free memory).  A queued
 * job starts as soon as a slot is free, its memory estimate (an upper bound
 * of what it allocates) fits what the running jobs leave of the budget, and
 * the GPU reports that much memory free (cudaMemGetInfo, plus the blocks the
 * slot keeps cached for reuse, less 1/64 of the GPU as a margin), so jobs
 * arriving while others run are admitted as slots and memory free up and
 * their work overlaps on the GPU.  A job that fits the budget but not the
 * free memory waits until no job runs.  A slot keeps at most budget / slots
 * of freed blocks cached between jobs.
 * Each job computes what the plain calls compute (a result does not depend on
 * the other jobs).  The reference's nearest equivalent is ParaFly's process
 * fan-out (Trinity:3652) and the two concurrent stats processes of
 * util/insilico_read_normalization.pl:853-854.
 *
 * Job kinds and outputs (tk_job_output `which`):
 *   TK_JOB_COUNT      text = reads; 0: dump text (count >= min_count, key order), 1: histo u64[10002]
 *                     (tk_table_histo bins for low 1, high 10000)
 *   TK_JOB_NORMALIZE  text = left mates, text2 = right mates; counted together (canonical when
 *                     `canonical`), then coverage of each: 0..2 left median u32 / mean f32 / stdev f32,
 *                     3..5 the same for the right mates, 6/7 left accession offset u64 / length u32
 *                     into text, 8/9 the same for the right mates into text2.  With max_cov >= 2 the
 *                     pairs are also selected (tk_norm_select with max_cov, min_cov, max_cv) and
 *                     extracted: 10 the accs text, 11 counts u64[4] (tk_norm_counts), 12/13 the
 *                     selected left / right records (tk_norm_extract)
 *   TK_JOB_R2T        text = reads, text2 = bundle; 0: rec i32, 1: hits u32, 2: nwin u32,
 *                     3/4 accession offset u64 / length u32 into text, 5: read starts u64[n+1] in
 *                     6: the packed upper-cased sequences, 7: component id u64 per bundle record
 * Input buffers are host memory owned by the caller and must stay valid until
 * the job has completed (tk_server_wait). */
#define TK_JOB_COUNT 1
#define TK_JOB_NORMALIZE 2
#define TK_JOB_R2T 3

typedef struct tk_job_spec {
    int kind;
    int k;
    int canonical;
    int strand;
    uint32_t min_count;
    const char *text;
    uint64_t len;
    const char *text2;
    uint64_t len2;
    int max_cov;          /* TK_JOB_NORMALIZE: >= 2 selects and extracts (0: statistics only) */
    int min_cov;
    int max_cv;
} tk_job_spec;

typedef struct tk_server tk_server;
int tk_server_create(int device, int slots, uint64_t hbm_budget, tk_server **out);
int tk_server_submit(tk_server *server, const tk_job_spec *spec, uint64_t *job_id);
/* Blocks until the job is done; latency = submit -> done, queued = submit -> start. */
int tk_server_wait(tk_server *server, uint64_t job_id, int *status, uint64_t *latency_ns, uint64_t *queued_ns);
/* Output buffer `which` of a completed job (valid until tk_job_release). */
int tk_job_output(tk_server *server, uint64_t job_id, int which, const void **data, uint64_t *bytes);
const char *tk_job_error(tk_server *server, uint64_t job_id);
int tk_job_release(tk_server *server, uint64_t job_id);
int tk_server_stats(tk_server *server, uint64_t *budget, uint64_t *in_use, int *max_concurrent);
/* Count jobs that ran inside a batched pass: a free slot takes the first
 * queued job that fits and, for a count job, every later queued count job
 * with the same k, strandedness and input format (up to 64 jobs / 256 MB)
 * as the bins of one tk_count_bins_ex pass. */
int tk_server_batched_jobs(tk_server *server, uint64_t *jobs);
/* Admission passes that found a queued job within the budget but above the
 * GPU's free memory (and so left it queued). */
int tk_server_held_by_free_memory(tk_server *server, uint64_t *admissions);
/* Waits for queued and running jobs, then stops the workers. */
void tk_server_destroy(tk_server *server);

#ifdef __cplusplus
}
#endif
#endif
