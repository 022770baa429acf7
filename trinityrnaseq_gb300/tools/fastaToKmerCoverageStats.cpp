// fastaToKmerCoverageStats -- drop-in for Inchworm's tool as
// util/insilico_read_normalization.pl:837-846 runs it:
//
//   fastaToKmerCoverageStats --reads R.fa --kmers K.fa --kmer_size 25 --num_threads T [--DS]
//                            [--capture_coverage_info] > R.fa.K25.stats
//   fastaToKmerCoverageStats --kmers_from_reads reads.fa --reads long.fa --num_threads 1   (Trinity:3930)
//
// Output (stdout): a header row, then one row per read in input order with
// columns acc, median_cov, mean_cov, stdev -- acc first for the `sort -k1,1`
// at util/insilico_read_normalization.pl:874 and the named columns the
// consumers read (util/support_scripts/nbkc_normalize.pl:85-97,
// nbkc_merge_left_right_stats.pl:95-103).  mean and stdev print like a C++
// ostream (%g).  A k-mer absent from the catalogue counts 1
// (Changelog.txt:536-538).  Lookups, medians and sums run on the GPU.
#include "tk_tool.hpp"

#include <string>
#include <vector>

using namespace tool;

static void usage() {
    std::fputs("usage: fastaToKmerCoverageStats [opts]\n"
               "Required:\n"
               "  --reads <str>             fasta file containing target reads for kmer coverage stats\n"
               "  --kmers <str>             fasta file containing kmers and abundance values (jellyfish dump)\n"
               "   or --kmers_from_reads <str>  fasta file of reads to count kmers from\n"
               "Optional:\n"
               "  --kmer_size <int>         default 25\n"
               "  --DS                      double-stranded RNA-Seq mode (not strand-specific)\n"
               "  --num_threads <int>       host formatting threads\n"
               "  --capture_coverage_info   append the per-window coverage values as a column\n", stderr);
}

int main(int argc, char **argv) {
    std::string reads_path, kmers_path, kfr_path;
    int k = 25, threads = 0;
    bool ds = false, capture = false;
    for (int i = 1; i < argc; i++) {
        std::string a = argv[i];
        auto val = [&](const char *name) -> std::string {
            if (i + 1 >= argc) die("%s needs a value", name);
            return argv[++i];
        };
        if (a == "--reads") reads_path = val("--reads");
        else if (a == "--kmers") kmers_path = val("--kmers");
        else if (a == "--kmers_from_reads") kfr_path = val("--kmers_from_reads");
        else if (a == "--kmer_size" || a == "-K") k = std::atoi(val("--kmer_size").c_str());
        else if (a == "--num_threads") threads = std::atoi(val("--num_threads").c_str());
        else if (a == "--DS") ds = true;
        else if (a == "--capture_coverage_info") capture = true;
        else if (a == "-h" || a == "--help") { usage(); return 0; }
        else { usage(); die("unknown option %s", a.c_str()); }
    }
    if (reads_path.empty() || (kmers_path.empty() && kfr_path.empty())) {
        usage();
        die("--reads and one of --kmers / --kmers_from_reads are required");
    }
    if (capture) std::fprintf(stderr, "fastaToKmerCoverageStats: --capture_coverage_info is accepted; per-window values are not written\n");
    tk_ctx *ctx = open_ctx();
    tk_table *t = nullptr;
    check(tk_table_create(ctx, k, ds ? 1 : 0, 0, &t), ctx, "table create");
    if (!kmers_path.empty()) {
        std::vector<char> cat = read_file(kmers_path);
        check(tk_table_load_dump_fasta(t, cat.data(), cat.size(), TK_HOST), ctx, ("load " + kmers_path).c_str());
    } else {
        std::vector<char> src = read_file(kfr_path);
        check(tk_table_count_text(t, src.data(), src.size(), TK_HOST), ctx, ("count " + kfr_path).c_str());
    }
    std::vector<char> text = read_file(reads_path);
    tk_reads *r = nullptr;
    check(tk_reads_parse(ctx, text.data(), text.size(), TK_HOST, &r), ctx, ("parse " + reads_path).c_str());
    uint64_t n = 0;
    check(tk_reads_info(r, &n, nullptr, nullptr, nullptr), ctx, "reads info");
    std::vector<uint32_t> med(n ? n : 1);
    std::vector<float> mean(n ? n : 1), sd(n ? n : 1);
    std::vector<uint64_t> noff(n ? n : 1);
    std::vector<uint32_t> nlen(n ? n : 1);
    if (n) {
        check(tk_coverage_stats(t, r, TK_HOST, med.data(), mean.data(), sd.data()), ctx, "coverage stats");
        check(tk_reads_names(r, noff.data(), nlen.data()), ctx, "read names");
    }
    tk_reads_free(r);
    tk_table_free(t);
    tk_ctx_destroy(ctx);
    const char *hdr = "acc\tmedian_cov\tmean_cov\tstdev\n";
    write_all(1, hdr, std::strlen(hdr), "stdout");
    auto chunks = format_parallel(n, host_threads(threads), [&](uint64_t lo, uint64_t hi, std::string &s) {
        s.reserve((hi - lo) * 48);
        char line[128];
        for (uint64_t i = lo; i < hi; i++) {
            s.append(text.data() + noff[i], nlen[i]);
            int L = std::snprintf(line, sizeof(line), "\t%u\t%g\t%g\n", med[i], (double)mean[i], (double)sd[i]);
            s.append(line, (size_t)L);
        }
    });
    for (auto &c : chunks) write_all(1, c.data(), c.size(), "stdout");
    return 0;
}
