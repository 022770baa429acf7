// insilico_read_normalization -- drop-in for util/insilico_read_normalization.pl,
// the command Trinity runs before assembly (Trinity:3421-3479):
//
//   insilico_read_normalization --seqType fq|fa --JM 10G --max_cov 200 --min_cov 1
//       --CPU N --output DIR --max_CV 10000 [--SS_lib_type RF]
//       (--left a.fq[,b.fq] --right a.fq[,b.fq] [--pairs_together] [--PARALLEL_STATS]
//        | --single s.fq[,t.fq])
//
// The script's steps run as one GPU pass over device-resident data: the
// FASTQ -> FASTA prep (seqtk-trinity seq -A -R 1|2 [-r], insilico:656-688),
// canonical 25-mer counting of both sides (jellyfish count --canonical,
// insilico:604-643; its -L 2 dump only drops k-mers the statistics count as 1
// anyway), the per-read coverage statistics (fastaToKmerCoverageStats --DS,
// insilico:816-850), the sort / pair merge / selection (sort -k1,1,
// nbkc_merge_left_right_stats.pl --sorted, nbkc_normalize.pl; insilico:865-985)
// and the extraction of the selected records (insilico:470-584).  The outputs
// are the script's: DIR/<base>.normalized_K25_maxC<M>_minC<m>_maxCV<V>.fq per
// side, with DIR/left.norm.fq and DIR/right.norm.fq (or single.norm.fq)
// symlinked to them (insilico:393-456), and the selection summary on stderr.
// FASTA input (--seqType fa) is counted as it is and extracted with
// PerlLib/Fasta_reader.pm's rules (the .fa outputs); reverse-complemented
// FASTA (an R in --SS_lib_type with fa, insilico:692-697) is not provided.
// No intermediate file is written.
#include "tk_tool.hpp"

#include <sys/stat.h>
#include <unistd.h>

#include <string>
#include <vector>

using namespace tool;

static void usage() {
    std::fputs("usage: insilico_read_normalization --seqType fq|fa --JM <n>G --max_cov <int> [--min_cov <int>]\n"
               "         [--max_CV <int>] [--CPU <int>] [--output <dir>] [--SS_lib_type F|R|FR|RF]\n"
               "         (--left <fq>[,<fq>...] --right <fq>[,<fq>...] [--pairs_together] | --single <fq>[,...])\n"
               "         [--left_list <file>] [--right_list <file>] [--KMER_SIZE 25] [--PARALLEL_STATS]\n"
               "         [--no_cleanup] [--NO_SEQTK] [--tmp_dir_name <name>]\n", stderr);
}

static std::vector<std::string> split_commas(const std::vector<std::string> &in) {
    std::vector<std::string> out;
    for (const std::string &s : in) {
        size_t a = 0;
        while (a <= s.size()) {
            size_t b = s.find(',', a);
            if (b == std::string::npos) b = s.size();
            if (b > a) out.push_back(s.substr(a, b - a));
            a = b + 1;
        }
    }
    return out;
}

static std::vector<std::string> read_list(const std::string &path) {
    std::vector<char> t = read_file(path);
    std::vector<std::string> out;
    std::string cur;
    for (char ch : t) {
        if (ch == '\n') {
            size_t a = cur.find_first_not_of(" \t\r"), b = cur.find_last_not_of(" \t\r");
            if (a != std::string::npos) out.push_back(cur.substr(a, b - a + 1));
            cur.clear();
        } else cur.push_back(ch);
    }
    size_t a = cur.find_first_not_of(" \t\r"), b = cur.find_last_not_of(" \t\r");
    if (a != std::string::npos) out.push_back(cur.substr(a, b - a + 1));
    return out;
}

static std::string base_name(const std::string &p) {
    size_t s = p.find_last_of('/');
    return s == std::string::npos ? p : p.substr(s + 1);
}

static std::string full_path(const std::string &p) {
    if (!p.empty() && p[0] == '/') return p;
    char buf[4096];
    if (!getcwd(buf, sizeof buf)) die("cannot read the working directory");
    return std::string(buf) + "/" + p;
}

// the files of one side back to back, each ending in a newline
static std::vector<char> read_side(const std::vector<std::string> &files) {
    std::vector<char> all;
    for (const std::string &f : files) {
        std::vector<char> t = read_file(f);
        all.insert(all.end(), t.begin(), t.end());
        if (!all.empty() && all.back() != '\n') all.push_back('\n');
    }
    return all;
}

struct Side {
    std::string tag;                    // left / right / single
    std::vector<std::string> files;
    std::vector<char> fastq;
    std::vector<char> fasta;            // the side's reads as FASTA (seqtk-trinity's output), until counted
    tk_reads *fq = nullptr, *fa = nullptr;
    std::vector<uint32_t> med;
    std::vector<float> mean, sd;
    uint64_t n = 0;
};

static void print_summary(const tk_norm_counts &c, int min_cov) {
    if (!c.rows) die("no reads made it to the normalization process");
    const double t = (double)c.rows;
    std::fprintf(stderr, "%llu / %llu = %.2f%% reads selected during normalization.\n", (unsigned long long)c.selected,
                 (unsigned long long)c.rows, c.selected / t * 100);
    std::fprintf(stderr, "%llu / %llu = %.2f%% reads discarded as likely aberrant based on coverage profiles.\n",
                 (unsigned long long)c.aberrant, (unsigned long long)c.rows, c.aberrant / t * 100);
    std::fprintf(stderr, "%llu / %llu = %.2f%% reads discarded as below minimum coverage threshold=%d\n",
                 (unsigned long long)c.below_min, (unsigned long long)c.rows, c.below_min / t * 100, min_cov);
}

int main(int argc, char **argv) {
    std::string seq_type, jm, ss, out_dir, left_list, right_list;
    std::vector<std::string> left, right, single;
    int max_cov = 0, min_cov = 0, max_cv = 10000, kmer = 25;
    bool pairs_together = false;
    std::vector<std::string> *multi = nullptr;   // a list option takes every value up to the next option
    for (int i = 1; i < argc; i++) {
        std::string a = argv[i];
        auto val = [&]() -> std::string {
            if (i + 1 >= argc) die("%s needs a value", a.c_str());
            multi = nullptr;
            return argv[++i];
        };
        auto ival = [&]() -> int {
            std::string v = val();
            uint64_t x = 0;
            if (!parse_u64(v.c_str(), &x) || x > 0x7FFFFFFF) die("%s needs a non-negative integer", a.c_str());
            return (int)x;
        };
        if (a.size() > 1 && a[0] == '-') multi = nullptr;
        if (a == "--seqType") seq_type = val();
        else if (a == "--JM") jm = val();
        else if (a == "--max_cov") max_cov = ival();
        else if (a == "--min_cov") min_cov = ival();
        else if (a == "--max_CV") max_cv = ival();
        else if (a == "--KMER_SIZE" || a == "--kmer_size") kmer = ival();
        else if (a == "--CPU" || a == "--jelly_s") (void)ival();
        else if (a == "--output") out_dir = val();
        else if (a == "--SS_lib_type") ss = val();
        else if (a == "--left_list") left_list = val();
        else if (a == "--right_list") right_list = val();
        else if (a == "--tmp_dir_name") (void)val();
        else if (a == "--left") { left.push_back(val()); multi = &left; }
        else if (a == "--right") { right.push_back(val()); multi = &right; }
        else if (a == "--single") { single.push_back(val()); multi = &single; }
        else if (a == "--pairs_together") pairs_together = true;
        else if (a == "--PARALLEL_STATS" || a == "--no_cleanup" || a == "--NO_SEQTK" ||
                 a == "--__devel_report_kmer_cov_stats") {
        } else if (a == "-h" || a == "--help") {
            usage();
            return 0;
        } else if (multi && !(a.size() > 1 && a[0] == '-')) multi->push_back(a);
        else {
            usage();
            die("do not understand option: %s", a.c_str());
        }
    }
    if (seq_type != "fq" && seq_type != "fa") {
        usage();
        die("set --seqType to 'fq' or 'fa'");
    }
    const bool fa_in = seq_type == "fa";
    if (jm.size() < 2 || jm[0] < '0' || jm[0] > '9' || jm.find_first_not_of("0123456789.") != jm.size() - 1 ||
        jm.back() != 'G')
        die("must set --JM to number of G of RAM (ie. 10G)");
    if (!ss.empty() && ss != "R" && ss != "F" && ss != "RF" && ss != "FR")
        die("unrecognized SS_lib_type value of %s. Should be: F, R, RF, or FR", ss.c_str());
    if (ss == "R") ss = "F";   // one strand-specific end needs no reverse complement (insilico:198-203)
    if (fa_in && ss.find('R') != std::string::npos)
        die("reverse-complemented FASTA input (--seqType fa with an R in --SS_lib_type) is not provided by this tool");
    if (!left_list.empty()) left = read_list(left_list);
    if (!right_list.empty()) right = read_list(right_list);
    left = split_commas(left);
    right = split_commas(right);
    single = split_commas(single);
    if (single.empty() && (left.empty() || right.empty())) die("need either options 'left' and 'right' or option 'single'");
    if (max_cov < 2) die("need to set --max_cov at least 2");
    if (kmer < 1 || kmer > 31) die("--KMER_SIZE must be 1..31");
    if (pairs_together && (left.empty() || right.empty()))
        die("if setting --pairs_together, must use the --left and --right parameters.");
    out_dir = full_path(out_dir.empty() ? "." : out_dir);
    mkdir(out_dir.c_str(), 0777);
    struct stat st;
    if (stat(out_dir.c_str(), &st) != 0 || !S_ISDIR(st.st_mode)) die("cannot mkdir %s", out_dir.c_str());

    std::vector<Side> sides;
    if (!left.empty() && !right.empty()) {
        sides.resize(2);
        sides[0].tag = "left";
        sides[0].files = left;
        sides[1].tag = "right";
        sides[1].files = right;
    } else {
        sides.resize(1);
        sides[0].tag = "single";
        sides[0].files = single;
    }
    tk_ctx *ctx = open_ctx();
    const bool strand = !ss.empty();
    tk_table *t = nullptr;
    check(tk_table_create(ctx, kmer, strand ? 0 : 1, 0, &t), ctx, "table create");
    for (size_t s = 0; s < sides.size(); s++) {
        Side &d = sides[s];
        d.fastq = read_side(d.files);
        check(tk_reads_parse(ctx, d.fastq.data(), d.fastq.size(), TK_HOST, &d.fq), ctx, ("parse " + d.tag).c_str());
        int fmt = 0;
        uint64_t n = 0;
        check(tk_reads_info(d.fq, &n, nullptr, nullptr, &fmt), ctx, "reads info");
        if (n && fmt != (fa_in ? TK_FMT_FASTA : TK_FMT_FASTQ))
            die("%s input is not %s", d.tag.c_str(), fa_in ? "FASTA" : "FASTQ");
        d.n = n;
        if (fa_in) continue;   // FASTA is counted as it is (insilico:692-705 concatenates it)
        // seqtk-trinity seq -A -R {1|2} [-r]: "-r" for the side whose library letter is R
        const char letter = s < ss.size() ? ss[s] : 0;
        const int flags = TK_FA_IF_MISSING | (letter == 'R' ? TK_FA_REVCOMP : 0);
        const int append = d.tag == "right" ? 2 : 1;
        uint64_t flen = 0;
        check(tk_reads_to_fasta(d.fq, append, flags, TK_HOST, nullptr, 0, &flen), ctx, "fastq to fasta");
        d.fasta.resize(flen ? flen : 1);
        check(tk_reads_to_fasta(d.fq, append, flags, TK_HOST, d.fasta.data(), d.fasta.size(), &flen), ctx,
              "fastq to fasta");
        d.fasta.resize(flen);
    }
    // both sides counted in one pass over the table (jellyfish counts
    // `cat left.fa right.fa`, insilico:617-626)
    if (fa_in) {
        std::vector<const tk_reads *> sets;
        for (Side &d : sides) sets.push_back(d.fq);
        check(tk_table_add_reads_multi(t, sets.data(), (uint32_t)sets.size()), ctx, "k-mer count");
        for (Side &d : sides) d.fa = d.fq;
    } else {
        std::vector<const char *> texts;
        std::vector<uint64_t> lens;
        for (Side &d : sides) {
            texts.push_back(d.fasta.data());
            lens.push_back(d.fasta.size());
        }
        std::vector<tk_reads *> fa(sides.size(), nullptr);
        check(tk_table_count_texts(t, texts.data(), lens.data(), (uint32_t)texts.size(), TK_HOST, fa.data()), ctx,
              "k-mer count");
        for (size_t s = 0; s < sides.size(); s++) {
            sides[s].fa = fa[s];
            std::vector<char>().swap(sides[s].fasta);
        }
    }
    for (Side &d : sides) {
        d.med.resize(d.n ? d.n : 1);
        d.mean.resize(d.n ? d.n : 1);
        d.sd.resize(d.n ? d.n : 1);
        if (d.n) check(tk_coverage_stats(t, d.fa, TK_HOST, d.med.data(), d.mean.data(), d.sd.data()), ctx, "coverage stats");
    }
    tk_table_free(t);
    // selection: the pairs together, or each side on its own
    std::vector<tk_norm *> sel(sides.size(), nullptr);
    if (sides.size() == 2 && pairs_together) {
        check(tk_norm_select(ctx, sides[0].fa, sides[0].med.data(), sides[0].mean.data(), sides[0].sd.data(), sides[1].fa,
                             sides[1].med.data(), sides[1].mean.data(), sides[1].sd.data(), TK_HOST, max_cov, min_cov,
                             max_cv, &sel[0]),
              ctx, "normalization");
        sel[1] = sel[0];
        tk_norm_counts c;
        check(tk_norm_info(sel[0], &c, nullptr), ctx, "normalization");
        if (!c.rows)
            die("pairs.K%d.stats is empty.  Be sure to check your fastq reads and ensure that the read names are "
                "identical except for the /1 or /2 designation.", kmer);
        print_summary(c, min_cov);
    } else {
        for (size_t s = 0; s < sides.size(); s++) {
            Side &d = sides[s];
            check(tk_norm_select(ctx, d.fa, d.med.data(), d.mean.data(), d.sd.data(), nullptr, nullptr, nullptr, nullptr,
                                 TK_HOST, max_cov, min_cov, max_cv, &sel[s]),
                  ctx, "normalization");
            tk_norm_counts c;
            check(tk_norm_info(sel[s], &c, nullptr), ctx, "normalization");
            print_summary(c, min_cov);
        }
    }
    std::vector<std::string> outputs;
    for (size_t s = 0; s < sides.size(); s++) {
        Side &d = sides[s];
        uint64_t len = 0;
        check(tk_norm_extract(sel[s], d.fq, &len), ctx, ("capture normalized reads from " + d.tag).c_str());
        std::vector<char> text(len ? len : 1);
        check(tk_norm_extract_copy(sel[s], TK_HOST, text.data(), text.size()), ctx, "capture normalized reads");
        const std::string base = d.files.size() == 1 ? base_name(d.files[0]) : base_name(d.files[0]) + "_ext_all_reads";
        const std::string name = base + ".normalized_K" + std::to_string(kmer) + "_maxC" + std::to_string(max_cov) +
                                 "_minC" + std::to_string(min_cov) + "_maxCV" + std::to_string(max_cv) + "." +
                                 seq_type;
        const std::string path = out_dir + "/" + name;
        FILE *f = std::fopen(path.c_str(), "wb");
        if (!f) die("cannot write to %s", path.c_str());
        if (len && std::fwrite(text.data(), 1, len, f) != len) die("cannot write to %s", path.c_str());
        std::fclose(f);
        const std::string link = out_dir + "/" + d.tag + ".norm." + seq_type;
        unlink(link.c_str());
        if (symlink(name.c_str(), link.c_str()) != 0) die("cannot link %s", link.c_str());
        outputs.push_back(path);
    }
    if (sel.size() == 2 && sel[1] == sel[0]) sel[1] = nullptr;
    for (tk_norm *n : sel) tk_norm_free(n);
    for (Side &d : sides) {
        if (d.fa != d.fq) tk_reads_free(d.fa);
        tk_reads_free(d.fq);
    }
    tk_ctx_destroy(ctx);
    std::fprintf(stderr, "\n\nNormalization complete. See outputs: \n");
    for (const std::string &o : outputs) std::fprintf(stderr, "\t%s\n", o.c_str());
    return 0;
}
