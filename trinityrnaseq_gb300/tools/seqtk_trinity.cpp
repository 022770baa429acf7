// seqtk-trinity -- drop-in for the `seq` conversion Trinity runs on FASTQ input
// before counting (Trinity:2782-2805):
//
//   cat reads.fq | seqtk-trinity seq -A -R {1|2} [-r] -  >> left.fa / right.fa
//
// FASTQ in, FASTA out (stdout): ">name/1\nSEQUENCE\n" per record.  The
// conversion follows util/support_scripts/fastQ_to_fastA.pl (the script
// Trinity runs instead with --NO_SEQTK, Trinity:2770-2779): name = the
// header's first field, "/1" or "/2" from a Casava "1:"/"2:" comment, the
// sequence line as written; -R N adds "/N" to names that do not already end in
// /1 or /2; -r reverse-complements (strand-specific RF libraries).  A poorly
// formed record stops the run with a non-zero exit, as the script does.  The
// parse and the conversion run on the GPU.
#include "tk_tool.hpp"

#include <string>
#include <vector>

using namespace tool;

static void usage() {
    std::fputs("usage: seqtk-trinity seq -A [-R 1|2] [-r] [in.fq|-]\n"
               "  -A       FASTA output (required)\n"
               "  -R INT   append /INT to read names that do not end in /1 or /2\n"
               "  -r       reverse complement the sequences\n", stderr);
}

int main(int argc, char **argv) {
    if (argc < 2 || std::string(argv[1]) != "seq") {
        usage();
        die("only the 'seq' command is provided");
    }
    bool fasta = false, rev = false;
    int append = -1;
    std::string path = "-";
    for (int i = 2; i < argc; i++) {
        std::string a = argv[i];
        if (a == "-A") fasta = true;
        else if (a == "-r") rev = true;
        else if (a == "-R") {
            if (i + 1 >= argc) die("-R needs a value");
            uint64_t v = 0;
            if (!parse_u64(argv[++i], &v) || v > 0x7FFFFFFF) die("-R needs a non-negative integer");
            append = (int)v;
        } else if (a == "-h" || a == "--help") {
            usage();
            return 0;
        } else if (a.size() > 1 && a[0] == '-') {
            usage();
            die("unsupported option %s", a.c_str());
        } else {
            path = a;
        }
    }
    if (!fasta) {
        usage();
        die("-A (FASTA output) is required");
    }
    std::vector<char> text = read_file(path == "-" ? std::string("/dev/stdin") : path);
    tk_ctx *ctx = open_ctx();
    tk_reads *reads = nullptr;
    check(tk_reads_parse(ctx, text.data(), text.size(), TK_HOST, &reads), ctx, "parse");
    uint64_t n_reads = 0;
    int format = 0;
    check(tk_reads_info(reads, &n_reads, nullptr, nullptr, &format), ctx, "reads info");
    if (n_reads && format != TK_FMT_FASTQ) die("%s: input is not FASTQ", path.c_str());
    const int flags = (rev ? TK_FA_REVCOMP : 0) | TK_FA_IF_MISSING;
    uint64_t len = 0;
    check(tk_reads_to_fasta(reads, append, flags, TK_HOST, nullptr, 0, &len), ctx, "fastq to fasta");
    std::vector<char> out(len ? len : 1);
    check(tk_reads_to_fasta(reads, append, flags, TK_HOST, out.data(), out.size(), &len), ctx, "fastq to fasta");
    write_all(1, out.data(), len, "stdout");
    tk_reads_free(reads);
    tk_ctx_destroy(ctx);
    return 0;
}
