// jellyfish -- drop-in for the jellyfish 2.x subcommands Trinity runs:
//
//   jellyfish count -t N -m 25 -s H [-o mer_counts.jf] [--canonical] reads.fa ...   (Trinity:2612-2621,
//                                                 util/insilico_read_normalization.pl:617-626)
//   jellyfish histo -t N -o out.histo db            (Trinity:2630, util/insilico_read_normalization.pl:636)
//   jellyfish dump -L m db > kmers.fa               (Trinity:2625, util/insilico_read_normalization.pl:641)
//   jellyfish --version                             (Trinity:4066-4073 wants a 2.x version)
//
// Counting, the histogram and the dump text run on the GPU through the C ABI
// (include/trinkmer.h).  The database file is this tool's own format (the
// reference unlinks it right after dump and histo, Trinity:2636-2638): a
// 32-byte header "TKJFDB01", k, canonical flag, pair count, then the sorted
// u64 keys and the u32 counts.  -s (hash size) and -t are accepted; the table
// is sized from a distinct-k-mer estimate and the GPU does the work.
#include "tk_tool.hpp"

#include <algorithm>
#include <string>
#include <vector>

using namespace tool;

static const char kMagic[8] = {'T', 'K', 'J', 'F', 'D', 'B', '0', '1'};

struct Db {
    uint32_t k = 0, canonical = 0;
    std::vector<uint64_t> keys;
    std::vector<uint32_t> counts;
};

static void write_db(const std::string &path, const Db &db) {
    AtomicFile f(path);
    char hdr[32] = {0};
    std::memcpy(hdr, kMagic, 8);
    uint64_t n = db.keys.size();
    std::memcpy(hdr + 8, &db.k, 4);
    std::memcpy(hdr + 12, &db.canonical, 4);
    std::memcpy(hdr + 16, &n, 8);
    f.write(hdr, 32);
    if (n) {
        f.write(reinterpret_cast<const char *>(db.keys.data()), n * 8);
        f.write(reinterpret_cast<const char *>(db.counts.data()), n * 4);
    }
    f.commit();
}

static Db read_db(const std::string &path) {
    std::vector<char> b = read_file(path);
    if (b.size() < 32 || std::memcmp(b.data(), kMagic, 8) != 0)
        die("%s is not a database written by this jellyfish count", path.c_str());
    Db db;
    uint64_t n = 0;
    std::memcpy(&db.k, b.data() + 8, 4);
    std::memcpy(&db.canonical, b.data() + 12, 4);
    std::memcpy(&n, b.data() + 16, 8);
    if (b.size() != 32 + n * 12) die("%s is truncated", path.c_str());
    db.keys.resize(n);
    db.counts.resize(n);
    if (n) {
        std::memcpy(db.keys.data(), b.data() + 32, n * 8);
        std::memcpy(db.counts.data(), b.data() + 32 + n * 8, n * 4);
    }
    return db;
}

static void usage() {
    std::fputs("Usage: jellyfish <cmd> [options] arg...\n"
               "Where <cmd> is one of: count, histo, dump\n"
               "Options:\n  --version  Display version\n  --help     This message\n", stderr);
}

static bool opt_val(int argc, char **argv, int &i, const char *shortf, const char *longf, std::string *out) {
    std::string a = argv[i];
    if (a == shortf || a == longf) {
        if (i + 1 >= argc) die("option %s needs a value", a.c_str());
        *out = argv[++i];
        return true;
    }
    std::string lp = std::string(longf) + "=";
    if (a.compare(0, lp.size(), lp) == 0) {
        *out = a.substr(lp.size());
        return true;
    }
    if (std::strlen(shortf) == 2 && a.size() > 2 && a.compare(0, 2, shortf) == 0 && a[1] != '-') {
        *out = a.substr(2);   // -m25 style
        return true;
    }
    return false;
}

static int cmd_count(int argc, char **argv) {
    int k = 0;
    bool canonical = false;
    std::string out = "mer_counts.jf", v;
    int reprobes = 0;
    std::vector<std::string> files;
    for (int i = 2; i < argc; i++) {
        std::string a = argv[i];
        if (opt_val(argc, argv, i, "-m", "--mer-len", &v)) k = std::atoi(v.c_str());
        else if (opt_val(argc, argv, i, "-o", "--output", &v)) out = v;
        else if (opt_val(argc, argv, i, "-s", "--size", &v)) {
            uint64_t s;
            if (!parse_u64(v.c_str(), &s)) die("bad --size %s", v.c_str());
        } else if (opt_val(argc, argv, i, "-t", "--threads", &v)) {
        } else if (opt_val(argc, argv, i, "-p", "--reprobes", &v)) reprobes = std::atoi(v.c_str());
        else if (opt_val(argc, argv, i, "-c", "--counter-len", &v) || opt_val(argc, argv, i, "-L", "--lower-count", &v) ||
                 opt_val(argc, argv, i, "-U", "--upper-count", &v) || opt_val(argc, argv, i, "-g", "--generator", &v) ||
                 opt_val(argc, argv, i, "-G", "--Generators", &v) || opt_val(argc, argv, i, "-S", "--shell", &v) ||
                 opt_val(argc, argv, i, "-Q", "--min-qual-char", &v) || opt_val(argc, argv, i, "-F", "--Files", &v) ||
                 opt_val(argc, argv, i, "-x", "--out-counter-len", &v)) {
            std::fprintf(stderr, "jellyfish count: option %s ignored\n", a.c_str());
        } else if (a == "-C" || a == "--canonical" || a == "--both-strands") canonical = true;
        else if (a == "--disk" || a == "--no-merge" || a == "--no-unlink" || a == "--text") {
            std::fprintf(stderr, "jellyfish count: option %s ignored\n", a.c_str());
        } else if (!a.empty() && a[0] == '-') die("jellyfish count: unknown option %s", a.c_str());
        else files.push_back(a);
    }
    if (k < 1 || k > 31) die("jellyfish count: -m must be in 1..31 (got %d)", k);
    if (files.empty()) die("jellyfish count: no input file");
    tk_ctx *ctx = open_ctx();
    if (reprobes > 0) check(tk_ctx_set_reprobes(ctx, reprobes), ctx, "set reprobes");
    tk_table *t = nullptr;
    check(tk_table_create(ctx, k, canonical ? 1 : 0, 0, &t), ctx, "table create");
    // every file, cut into record-aligned pieces of about 1 GB, counted in one
    // pass over the table: each piece is parsed and bucketed while the later
    // ones upload (tk_table_count_texts)
    std::vector<std::vector<char>> texts;
    for (const std::string &f : files) texts.push_back(read_file(f));
    std::vector<const char *> ptrs;
    std::vector<uint64_t> lens;
    for (const std::vector<char> &x : texts) {
        const uint32_t n = (uint32_t)std::min<uint64_t>(16, std::max<uint64_t>(1, x.size() >> 30));
        std::vector<uint64_t> cuts(n + 1);
        check(tk_split_records(x.data(), x.size(), n, cuts.data()), ctx, "split records");
        for (uint32_t i = 0; i < n; i++) {
            ptrs.push_back(x.data() + cuts[i]);
            lens.push_back(cuts[i + 1] - cuts[i]);
        }
    }
    std::vector<tk_reads *> sets(ptrs.size(), nullptr);
    std::string what = "count";
    for (const std::string &f : files) what += " " + f;
    check(tk_table_count_texts(t, ptrs.data(), lens.data(), (uint32_t)ptrs.size(), TK_HOST, sets.data()), ctx,
          what.c_str());
    for (tk_reads *r : sets) tk_reads_free(r);
    texts.clear();
    Db db;
    db.k = (uint32_t)k;
    db.canonical = canonical ? 1 : 0;
    uint64_t n = 0;
    check(tk_table_dump(t, 1, TK_HOST, nullptr, nullptr, 0, &n), ctx, "dump size");
    db.keys.resize(n);
    db.counts.resize(n);
    uint64_t m = 0;
    if (n) check(tk_table_dump(t, 1, TK_HOST, db.keys.data(), db.counts.data(), n, &m), ctx, "dump");
    tk_table_free(t);
    tk_ctx_destroy(ctx);
    write_db(out, db);
    return 0;
}

static tk_table *table_from_db(tk_ctx *ctx, const Db &db) {
    tk_table *t = nullptr;
    check(tk_table_create(ctx, (int)db.k, (int)db.canonical, 0, &t), ctx, "table create");
    if (!db.keys.empty())
        check(tk_table_load_pairs(t, db.keys.data(), db.counts.data(), db.keys.size(), TK_HOST), ctx, "load db");
    return t;
}

static int cmd_histo(int argc, char **argv) {
    std::string out, v, dbpath;
    uint64_t low = 1, high = 10000, inc = 1;
    bool full = false;
    for (int i = 2; i < argc; i++) {
        std::string a = argv[i];
        if (opt_val(argc, argv, i, "-o", "--output", &v)) out = v;
        else if (opt_val(argc, argv, i, "-l", "--low", &v)) { if (!parse_u64(v.c_str(), &low)) die("bad --low"); }
        else if (opt_val(argc, argv, i, "-h", "--high", &v)) { if (!parse_u64(v.c_str(), &high)) die("bad --high"); }
        else if (opt_val(argc, argv, i, "-i", "--increment", &v)) { if (!parse_u64(v.c_str(), &inc)) die("bad --increment"); }
        else if (opt_val(argc, argv, i, "-t", "--threads", &v)) {}
        else if (a == "-f" || a == "--full") full = true;
        else if (!a.empty() && a[0] == '-') die("jellyfish histo: unknown option %s", a.c_str());
        else dbpath = a;
    }
    if (dbpath.empty()) die("jellyfish histo: no database");
    if (inc != 1) die("jellyfish histo: only --increment 1 is supported");
    if (low < 1 || high < low) die("jellyfish histo: need 1 <= low <= high");
    Db db = read_db(dbpath);
    tk_ctx *ctx = open_ctx();
    tk_table *t = table_from_db(ctx, db);
    std::vector<uint64_t> h(high - low + 3);
    check(tk_table_histo(t, low, high, h.data()), ctx, "histo");
    tk_table_free(t);
    tk_ctx_destroy(ctx);
    // bin 0 collects counts below low (labelled low-1), the last counts above high (high+1)
    std::string s;
    char line[64];
    for (size_t b = 0; b < h.size(); b++) {
        uint64_t label = b == 0 ? low - 1 : (b == h.size() - 1 ? high + 1 : low + b - 1);
        if (!h[b] && (!full || b == 0)) continue;
        int L = std::snprintf(line, sizeof(line), "%llu %llu\n", (unsigned long long)label, (unsigned long long)h[b]);
        s.append(line, (size_t)L);
    }
    if (out.empty()) write_all(1, s.data(), s.size(), "stdout");
    else {
        AtomicFile f(out);
        f.write(s);
        f.commit();
    }
    return 0;
}

static int cmd_dump(int argc, char **argv) {
    std::string out, v, dbpath;
    uint64_t lower = 1, upper = UINT64_MAX;
    bool column = false, tab = false;
    for (int i = 2; i < argc; i++) {
        std::string a = argv[i];
        if (opt_val(argc, argv, i, "-L", "--lower-count", &v)) { if (!parse_u64(v.c_str(), &lower)) die("bad -L"); }
        else if (opt_val(argc, argv, i, "-U", "--upper-count", &v)) { if (!parse_u64(v.c_str(), &upper)) die("bad -U"); }
        else if (opt_val(argc, argv, i, "-o", "--output", &v)) out = v;
        else if (a == "-c" || a == "--column") column = true;
        else if (a == "-t" || a == "--tab") tab = true;
        else if (!a.empty() && a[0] == '-') die("jellyfish dump: unknown option %s", a.c_str());
        else dbpath = a;
    }
    if (dbpath.empty()) die("jellyfish dump: no database");
    Db db = read_db(dbpath);
    std::string text;
    if (!column && upper == UINT64_MAX) {
        // the default FASTA-like dump is formatted on the GPU (K4)
        tk_ctx *ctx = open_ctx();
        tk_table *t = table_from_db(ctx, db);
        uint64_t len = 0;
        uint32_t lo = (uint32_t)std::min<uint64_t>(lower, 0xFFFFFFFFull);
        check(tk_table_dump_fasta(t, lo, TK_HOST, nullptr, 0, &len), ctx, "dump");
        text.resize(len);
        if (len) check(tk_table_dump_fasta(t, lo, TK_HOST, &text[0], len, &len), ctx, "dump copy");
        tk_table_free(t);
        tk_ctx_destroy(ctx);
    } else {
        const char sep = tab ? '\t' : ' ';
        char kmer[40];
        for (size_t i = 0; i < db.keys.size(); i++) {
            if (db.counts[i] < lower || db.counts[i] > upper) continue;
            for (uint32_t j = 0; j < db.k; j++) kmer[j] = "ACGT"[(db.keys[i] >> (2 * (db.k - 1 - j))) & 3];
            kmer[db.k] = 0;
            char line[96];
            int L = column ? std::snprintf(line, sizeof(line), "%s%c%u\n", kmer, sep, db.counts[i])
                           : std::snprintf(line, sizeof(line), ">%u\n%s\n", db.counts[i], kmer);
            text.append(line, (size_t)L);
        }
    }
    if (out.empty()) write_all(1, text.data(), text.size(), "stdout");
    else {
        AtomicFile f(out);
        f.write(text);
        f.commit();
    }
    return 0;
}

int main(int argc, char **argv) {
    if (argc < 2) {
        usage();
        return 1;
    }
    std::string cmd = argv[1];
    if (cmd == "--version" || cmd == "-V" || cmd == "version") {
        std::printf("jellyfish 2.3.0\n");
        return 0;
    }
    if (cmd == "--help" || cmd == "-h") {
        usage();
        return 0;
    }
    if (cmd == "count") return cmd_count(argc, argv);
    if (cmd == "histo") return cmd_histo(argc, argv);
    if (cmd == "dump") return cmd_dump(argc, argv);
    usage();
    die("unknown command %s", cmd.c_str());
}
