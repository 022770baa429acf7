// FastaToDeBruijn -- drop-in for Inchworm's tool as Trinity:2298-2302 runs it:
//
//   FastaToDeBruijn --fasta bundled_iworm_contigs.fasta -K 24 --graph_per_record [--SS] --threads CPU
//       > bundled_iworm_contigs.fasta.deBruijn
//
// Writes, per bundle record with at least one window of K+1 A/C/G/T bases,
// "Component <id>" and one line per distinct (K+1)-mer of the record in order
// of first occurrence: "<node>\t<prev>\t<count>\t<kmer>" (include/trinkmer.h,
// tk_dbg_create).  util/support_scripts/partition_chrysalis_graphs_n_reads.pl
// reads the "Component" lines and counts the lines after each as the
// component's k-mers.  The graphs are built on the GPU; --threads is accepted
// for the command line's sake.  Only --graph_per_record is supported (the
// mode Trinity uses).
#include "tk_tool.hpp"

#include <string>
#include <vector>

using namespace tool;

static void usage() {
    std::fputs("usage: FastaToDeBruijn --fasta <bundle.fasta> -K <kmer_length> --graph_per_record [--SS]\n"
               "                       [--threads N]  (graph text on stdout)\n", stderr);
}

int main(int argc, char **argv) {
    std::string fasta;
    int K = -1;
    bool per_record = false, ss = false;
    for (int i = 1; i < argc; i++) {
        std::string a = argv[i];
        auto val = [&](const char *name) -> std::string {
            if (i + 1 >= argc) die("%s needs a value", name);
            return argv[++i];
        };
        if (a == "--fasta") fasta = val("--fasta");
        else if (a == "-K") K = std::atoi(val("-K").c_str());
        else if (a == "--graph_per_record") per_record = true;
        else if (a == "--SS") ss = true;
        else if (a == "--threads") (void)val("--threads");
        else if (a == "-h" || a == "--help") { usage(); return 0; }
        else { usage(); die("unknown option %s", a.c_str()); }
    }
    if (fasta.empty() || K < 1) {
        usage();
        die("--fasta and -K are required");
    }
    if (!per_record) die("only --graph_per_record is supported (one graph per bundle record)");
    tk_ctx *ctx = open_ctx();
    std::vector<char> bundle = read_file(fasta);
    tk_dbg *g = nullptr;
    check(tk_dbg_create(ctx, bundle.data(), bundle.size(), TK_HOST, K, ss ? 1 : 0, &g), ctx, "de Bruijn graphs");
    uint64_t len = 0;
    check(tk_dbg_info(g, nullptr, nullptr, &len), ctx, "graph info");
    std::vector<char> text(len ? len : 1);
    if (len) check(tk_dbg_text(g, TK_HOST, text.data(), len), ctx, "graph text");
    write_all(1, text.data(), len, "stdout");
    tk_dbg_free(g);
    tk_ctx_destroy(ctx);
    return 0;
}
