// trinkmer_bins -- the k-mer catalogues of Trinity's phase-2 read bins in one
// batched GPU pass.
//
// Phase 2 runs one `Trinity --single <bin reads.fa> --output <bin reads.fa>.out
// ... --trinity_complete` per bin (util/support_scripts/write_partitioned_trinity_cmds.pl:
// the last field of each line of the reads list file, Trinity:3669-3677), fanned
// out by ParaFly (Trinity:3652); with --trinity_complete each of them counts its
// bin's k-mers with Inchworm's own cataloguer (`inchworm --reads ... -K 25
// [--minKmerCount N] [--DS]`, Trinity:2663-2678).  This tool takes the same
// reads list file and writes, next to every bin, the catalogue that run would
// build -- `<reads.fa>.K<k>.kmers.fa`, ">COUNT\nKMER\n" per k-mer with count
// >= --min_kmer_cov, in key order, the format `inchworm --kmers` reads
// (Trinity:2612-2628) -- from one tk_count_bins_ex call over all bins (a few
// calls when the bins exceed --max_batch_gb).  With --histo it also writes
// `<reads.fa>.K<k>.histo` (jellyfish histo's "count n" lines for the
// non-empty counts 1..10000 and 10001 for the ones above).
//
//   trinkmer_bins --reads_list_file partitioned_reads.files.list [-K 25]
//                 [--min_kmer_cov 1] [--SS] [--histo] [--max_batch_gb 8]
#include "tk_tool.hpp"

#include <string>
#include <vector>

using namespace tool;

static void usage() {
    std::fputs("usage: trinkmer_bins --reads_list_file <list> [-K 25] [--min_kmer_cov N] [--SS] [--histo]\n"
               "                     [--max_batch_gb 8]\n", stderr);
}

static std::vector<std::string> list_files(const std::string &path) {
    std::vector<char> t = read_file(path);
    std::vector<std::string> files;
    size_t i = 0;
    while (i < t.size()) {
        size_t e = i;
        while (e < t.size() && t[e] != '\n') e++;
        // the line's last whitespace-separated field, as write_partitioned_trinity_cmds.pl takes it
        size_t b = e;
        while (b > i && (t[b - 1] == ' ' || t[b - 1] == '\t' || t[b - 1] == '\r')) b--;
        size_t a = b;
        while (a > i && t[a - 1] != ' ' && t[a - 1] != '\t') a--;
        if (b > a) files.emplace_back(t.data() + a, b - a);
        i = e + 1;
    }
    return files;
}

int main(int argc, char **argv) {
    std::string list;
    int k = 25;
    uint32_t min_cov = 1;
    bool ss = false, histo = false;
    double max_gb = 8.0;
    for (int i = 1; i < argc; i++) {
        std::string a = argv[i];
        auto val = [&](const char *name) -> std::string {
            if (i + 1 >= argc) die("%s needs a value", name);
            return argv[++i];
        };
        if (a == "--reads_list_file") list = val("--reads_list_file");
        else if (a == "-K") k = std::atoi(val("-K").c_str());
        else if (a == "--min_kmer_cov" || a == "--minKmerCount") min_cov = (uint32_t)std::atoi(val(a.c_str()).c_str());
        else if (a == "--SS") ss = true;
        else if (a == "--histo") histo = true;
        else if (a == "--max_batch_gb") max_gb = std::atof(val("--max_batch_gb").c_str());
        else if (a == "-h" || a == "--help") { usage(); return 0; }
        else { usage(); die("unknown option %s", a.c_str()); }
    }
    if (list.empty()) {
        usage();
        die("--reads_list_file is required");
    }
    if (k < 1 || k > 31) die("-K must be in 1..31");
    if (min_cov < 1) min_cov = 1;
    const std::vector<std::string> files = list_files(list);
    tk_ctx *ctx = open_ctx();
    const uint64_t max_bytes = (uint64_t)(max_gb * 1e9);
    const std::string sfx = ".K" + std::to_string(k);
    size_t f0 = 0;
    while (f0 < files.size()) {
        // the next batch: bins back to back, each ending with a newline
        std::vector<char> text;
        std::vector<uint64_t> off{0};
        size_t f1 = f0;
        while (f1 < files.size() && (f1 == f0 || text.size() < max_bytes)) {
            std::vector<char> t = read_file(files[f1]);
            text.insert(text.end(), t.begin(), t.end());
            if (!t.empty() && t.back() != '\n') text.push_back('\n');
            off.push_back(text.size());
            f1++;
        }
        const uint32_t n = (uint32_t)(f1 - f0);
        std::vector<uint32_t> minc(n, min_cov);
        std::vector<uint64_t> hist(histo ? (size_t)n * 10002 : 0);
        tk_bins *b = nullptr;
        check(tk_count_bins_ex(ctx, text.data(), text.size(), TK_HOST, off.data(), n, k, ss ? 0 : 1, minc.data(),
                               histo ? hist.data() : nullptr, &b),
              ctx, "batched bin count");
        uint64_t len = 0;
        check(tk_bins_info(b, &len, nullptr), ctx, "bins info");
        std::vector<uint64_t> doff(n + 1);
        check(tk_bins_dump_offsets(b, doff.data()), ctx, "bin offsets");
        std::vector<char> dump(len ? len : 1);
        if (len) check(tk_bins_dump_text(b, dump.data(), len), ctx, "bin dumps");
        tk_bins_free(b);
        for (uint32_t i = 0; i < n; i++) {
            const std::string &f = files[f0 + i];
            AtomicFile out(f + sfx + ".kmers.fa");
            out.write(dump.data() + doff[i], doff[i + 1] - doff[i]);
            out.commit();
            if (histo) {
                AtomicFile h(f + sfx + ".histo");
                std::string s;
                const uint64_t *hb = hist.data() + (size_t)i * 10002;
                for (int c = 1; c <= 10001; c++)   // jellyfish histo's lines: non-empty bins, 10001 = above 10000
                    if (hb[c]) s += std::to_string(c) + " " + std::to_string(hb[c]) + "\n";
                h.write(s);
                h.commit();
            }
        }
        f0 = f1;
    }
    tk_ctx_destroy(ctx);
    return 0;
}
