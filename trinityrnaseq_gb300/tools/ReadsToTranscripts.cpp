// ReadsToTranscripts -- drop-in for Chrysalis' tool as Trinity:2237-2251 runs it:
//
//   ReadsToTranscripts -i both.fa -f bundled_iworm_contigs.fasta -o readsToComponents.out
//                      -t CPU -max_mem_reads 50000000 [-strand] [-p 10]
//
// Output rows "component_id \t >read_acc \t pct \t READSEQ" (columns read at
// Trinity:2474, util/support_scripts/partition_chrysalis_graphs_n_reads.pl:103,
// add_LR_reads_to_iworm_bundle.pl:19-25); the driver sorts them with
// `sort -k1,1n -k3,3nr -k2,2` (Trinity:2258).  Reads are upper-cased
// (Changelog.txt:467); a read with fewer than -p percent of its k-mers on the
// winning component is not written (Changelog.txt:870-873).  Bundle table,
// lookups and the vote run on the GPU; reads are processed -max_mem_reads at a
// time.
#include "tk_tool.hpp"

#include <string>
#include <vector>

using namespace tool;

static void usage() {
    std::fputs("usage: ReadsToTranscripts -i <reads.fa> -f <bundle.fasta> -o <out> [-t threads] [-max_mem_reads N]\n"
               "                          [-strand] [-p min_pct] [-k kmer_size]\n", stderr);
}

// end offset of the record block holding at most `max_reads` records from `pos`
static size_t next_chunk(const std::vector<char> &t, size_t pos, uint64_t max_reads) {
    uint64_t seen = 0;
    size_t i = pos;
    const size_t n = t.size();
    while (i < n) {
        bool line_start = i == 0 || t[i - 1] == '\n';
        if (line_start && t[i] == '>') {
            if (seen == max_reads) return i;
            seen++;
        }
        const void *nl = std::memchr(t.data() + i, '\n', n - i);
        i = nl ? (size_t)((const char *)nl - t.data()) + 1 : n;
    }
    return n;
}

int main(int argc, char **argv) {
    std::string reads_path, bundle_path, out_path;
    int k = 25, threads = 0, min_pct = 0;
    bool strand = false;
    uint64_t max_mem_reads = 50000000;
    for (int i = 1; i < argc; i++) {
        std::string a = argv[i];
        auto val = [&](const char *name) -> std::string {
            if (i + 1 >= argc) die("%s needs a value", name);
            return argv[++i];
        };
        if (a == "-i") reads_path = val("-i");
        else if (a == "-f") bundle_path = val("-f");
        else if (a == "-o") out_path = val("-o");
        else if (a == "-t") threads = std::atoi(val("-t").c_str());
        else if (a == "-k") k = std::atoi(val("-k").c_str());
        else if (a == "-p") min_pct = std::atoi(val("-p").c_str());
        else if (a == "-max_mem_reads") {
            std::string v = val("-max_mem_reads");
            if (!parse_u64(v.c_str(), &max_mem_reads) || !max_mem_reads) die("bad -max_mem_reads %s", v.c_str());
        } else if (a == "-strand") strand = true;
        else if (a == "-h" || a == "--help") { usage(); return 0; }
        else { usage(); die("unknown option %s", a.c_str()); }
    }
    if (reads_path.empty() || bundle_path.empty() || out_path.empty()) {
        usage();
        die("-i, -f and -o are required");
    }
    tk_ctx *ctx = open_ctx();
    std::vector<char> bundle = read_file(bundle_path);
    tk_r2t *z = nullptr;
    check(tk_r2t_create(ctx, bundle.data(), bundle.size(), TK_HOST, k, strand ? 1 : 0, &z), ctx, "bundle table");
    uint64_t nrec = 0;
    check(tk_r2t_info(z, &nrec, nullptr), ctx, "bundle info");
    std::vector<uint64_t> comp(nrec ? nrec : 1);
    if (nrec) check(tk_r2t_component_ids(z, comp.data()), ctx, "component ids");
    bundle.clear();
    bundle.shrink_to_fit();

    std::vector<char> text = read_file(reads_path);
    AtomicFile out(out_path);
    const int T = host_threads(threads);
    size_t pos = 0;
    while (pos < text.size()) {
        size_t end = next_chunk(text, pos, max_mem_reads);
        tk_reads *r = nullptr;
        check(tk_reads_parse(ctx, text.data() + pos, end - pos, TK_HOST, &r), ctx, ("parse " + reads_path).c_str());
        uint64_t n = 0;
        check(tk_reads_info(r, &n, nullptr, nullptr, nullptr), ctx, "reads info");
        if (n) {
            std::vector<int32_t> rec(n);
            std::vector<uint32_t> hits(n), nwin(n), nlen(n);
            std::vector<uint64_t> noff(n), roff(n + 1);
            check(tk_r2t_assign(z, r, TK_HOST, rec.data(), hits.data(), nwin.data()), ctx, "assign");
            check(tk_reads_names(r, noff.data(), nlen.data()), ctx, "read names");
            check(tk_reads_offsets(r, roff.data()), ctx, "read offsets");
            std::vector<char> seq(roff[n] ? roff[n] : 1);
            check(tk_reads_copy_seq(r, seq.data(), roff[n]), ctx, "read sequences");
            const char *base = text.data() + pos;
            auto chunks = format_parallel(n, T, [&](uint64_t lo, uint64_t hi, std::string &s) {
                char head[64];
                for (uint64_t i = lo; i < hi; i++) {
                    if (rec[i] < 0 || nwin[i] == 0) continue;
                    uint32_t pct = (uint32_t)((100ull * hits[i]) / nwin[i]);
                    if (min_pct > 0 && pct < (uint32_t)min_pct) continue;
                    int L = std::snprintf(head, sizeof(head), "%llu\t>", (unsigned long long)comp[(size_t)rec[i]]);
                    s.append(head, (size_t)L);
                    s.append(base + noff[i], nlen[i]);
                    L = std::snprintf(head, sizeof(head), "\t%u\t", pct);
                    s.append(head, (size_t)L);
                    s.append(seq.data() + roff[i], roff[i + 1] - roff[i] - 1);
                    s.push_back('\n');
                }
            });
            for (auto &c : chunks) out.write(c);
        }
        tk_reads_free(r);
        pos = end;
    }
    out.commit();
    tk_r2t_free(z);
    tk_ctx_destroy(ctx);
    return 0;
}
