// trinkmerd -- resident k-mer job daemon on one GPU.
//
//   trinkmerd --socket /path/sock [--slots 4] [--budget-gb 150] [--device 0]
//
// Clients connect to the Unix socket and send one request line; the daemon
// reads the input files, runs the job on the job server (tk_server_*: worker
// slots with their own streams, admission by an HBM budget, jobs overlapping
// on the GPU), writes the outputs atomically in the formats of the reference
// tools, and answers one line:
//
//   COUNT <k> <canonical 0|1> <min_count> <reads> <dump_out> [<histo_out>]
//         -> the `jellyfish dump -L min_count` text and the `jellyfish histo` file
//   NORMALIZE <k> <ds 0|1> <left.fa> <right.fa> <left_stats_out> <right_stats_out>
//         -> the two `fastaToKmerCoverageStats` tables (k-mers counted over both files)
//   SELECT <k> <ds 0|1> <max_cov> <min_cov> <max_CV> <left> <right> <left_out> <right_out> <accs_out>
//         -> the whole in-silico normalization of the pairs (util/insilico_read_normalization.pl
//            --pairs_together): the selected records of each side and nbkc_normalize.pl's accs
//   R2T <k> <strand 0|1> <min_pct> <reads.fa> <bundle.fasta> <out>
//         -> the `ReadsToTranscripts` rows
//   STATS -> OK <jobs> <p50_ms> <p99_ms> <max_concurrent>
//   QUIT  -> stops accepting, finishes running jobs, exits
//
// Answers: "OK <job_id> <latency_ms> <queued_ms>" or "ERR <message>".
#include "tk_tool.hpp"

#include <algorithm>
#include <atomic>
#include <mutex>
#include <sstream>
#include <string>
#include <vector>

#include <poll.h>
#include <sys/socket.h>
#include <sys/un.h>

using namespace tool;

static tk_server *g_srv = nullptr;
static std::atomic<bool> g_quit{false};
static std::mutex g_lat_mu;
static std::vector<double> g_lat;

template <typename T>
static const T *out_as(uint64_t id, int which, uint64_t *count) {
    const void *p = nullptr;
    uint64_t b = 0;
    if (tk_job_output(g_srv, id, which, &p, &b) != TK_OK) return nullptr;
    *count = b / sizeof(T);
    return static_cast<const T *>(p);
}

static void write_chunks(const std::string &path, const std::string &head, const std::vector<std::string> &chunks) {
    AtomicFile f(path);
    f.write(head);
    for (auto &c : chunks) f.write(c);
    f.commit();
}

static std::string histo_text(const uint64_t *h, uint64_t nb) {
    std::string s;
    char line[64];
    for (uint64_t b = 1; b < nb; b++) {
        if (!h[b]) continue;
        int L = std::snprintf(line, sizeof(line), "%llu %llu\n", (unsigned long long)b, (unsigned long long)h[b]);
        s.append(line, (size_t)L);
    }
    return s;
}

static bool readable(const std::string &p) { return ::access(p.c_str(), R_OK) == 0; }

static std::string handle(const std::string &req) {
    std::istringstream in(req);
    std::string cmd;
    in >> cmd;
    if (cmd == "STATS") {
        std::lock_guard<std::mutex> g(g_lat_mu);
        std::vector<double> v = g_lat;
        std::sort(v.begin(), v.end());
        auto pct = [&](double q) { return v.empty() ? 0.0 : v[std::min(v.size() - 1, (size_t)(q * (double)v.size()))]; };
        int maxc = 0;
        tk_server_stats(g_srv, nullptr, nullptr, &maxc);
        char b[160];
        std::snprintf(b, sizeof(b), "OK %zu %.3f %.3f %d", v.size(), pct(0.5), pct(0.99), maxc);
        return b;
    }
    if (cmd == "QUIT") {
        g_quit = true;
        return "OK";
    }
    tk_job_spec s{};
    std::vector<char> t1, t2;
    std::string o1, o2, o3;
    int min_pct = 0;
    if (cmd == "COUNT") {
        std::string reads;
        in >> s.k >> s.canonical >> s.min_count >> reads >> o1;
        in >> o2;
        if (!in && o1.empty()) return "ERR usage: COUNT k canonical min_count reads dump_out [histo_out]";
        s.kind = TK_JOB_COUNT;
        if (!readable(reads)) return "ERR cannot read " + reads;
        t1 = read_file(reads);
    } else if (cmd == "NORMALIZE") {
        std::string l, r;
        in >> s.k >> s.canonical >> l >> r >> o1 >> o2;
        if (!in) return "ERR usage: NORMALIZE k ds left right left_out right_out";
        s.kind = TK_JOB_NORMALIZE;
        if (!readable(l) || !readable(r)) return "ERR cannot read " + l + " or " + r;
        t1 = read_file(l);
        t2 = read_file(r);
    } else if (cmd == "SELECT") {
        std::string l, r;
        in >> s.k >> s.canonical >> s.max_cov >> s.min_cov >> s.max_cv >> l >> r >> o1 >> o2 >> o3;
        if (!in) return "ERR usage: SELECT k ds max_cov min_cov max_CV left right left_out right_out accs_out";
        if (s.max_cov < 2) return "ERR max_cov must be at least 2";
        s.kind = TK_JOB_NORMALIZE;
        if (!readable(l) || !readable(r)) return "ERR cannot read " + l + " or " + r;
        t1 = read_file(l);
        t2 = read_file(r);
    } else if (cmd == "R2T") {
        std::string reads, bundle;
        in >> s.k >> s.strand >> min_pct >> reads >> bundle >> o1;
        if (!in) return "ERR usage: R2T k strand min_pct reads bundle out";
        s.kind = TK_JOB_R2T;
        s.canonical = !s.strand;
        if (!readable(reads) || !readable(bundle)) return "ERR cannot read " + reads + " or " + bundle;
        t1 = read_file(reads);
        t2 = read_file(bundle);
    } else {
        return "ERR unknown command";
    }
    s.text = t1.data();
    s.len = t1.size();
    s.text2 = t2.data();
    s.len2 = t2.size();
    uint64_t id = 0;
    if (tk_server_submit(g_srv, &s, &id) != TK_OK) return "ERR bad job";
    int st = 0;
    uint64_t lat = 0, q = 0;
    tk_server_wait(g_srv, id, &st, &lat, &q);
    if (st != TK_OK) {
        std::string m = std::string("ERR ") + tk_status_string(st) + ": " + tk_job_error(g_srv, id);
        tk_job_release(g_srv, id);
        return m;
    }
    const int T = host_threads(0);
    uint64_t n = 0, n2 = 0;
    if (s.kind == TK_JOB_COUNT) {
        const char *dump = out_as<char>(id, 0, &n);
        write_chunks(o1, std::string(dump, n), {});
        if (!o2.empty()) {
            const uint64_t *h = out_as<uint64_t>(id, 1, &n2);
            write_chunks(o2, histo_text(h, n2), {});
        }
    } else if (s.kind == TK_JOB_NORMALIZE && s.max_cov >= 2) {
        const char *accs = out_as<char>(id, 10, &n);
        write_chunks(o3, std::string(accs, n), {});
        for (int side = 0; side < 2; side++) {
            const char *recs = out_as<char>(id, 12 + side, &n2);
            write_chunks(side ? o2 : o1, std::string(recs, n2), {});
        }
    } else if (s.kind == TK_JOB_NORMALIZE) {
        const char *hdr = "acc\tmedian_cov\tmean_cov\tstdev\n";
        for (int side = 0; side < 2; side++) {
            const uint32_t *med = out_as<uint32_t>(id, 3 * side, &n);
            const float *mean = out_as<float>(id, 3 * side + 1, &n2);
            const float *sd = out_as<float>(id, 3 * side + 2, &n2);
            const uint64_t *noff = out_as<uint64_t>(id, 6 + 2 * side, &n2);
            const uint32_t *nlen = out_as<uint32_t>(id, 7 + 2 * side, &n2);
            const char *text = side ? t2.data() : t1.data();
            write_chunks(side ? o2 : o1, hdr, format_stats_rows(text, noff, nlen, med, mean, sd, n, T));
        }
    } else {
        const int32_t *rec = out_as<int32_t>(id, 0, &n);
        const uint32_t *hits = out_as<uint32_t>(id, 1, &n2);
        const uint32_t *nwin = out_as<uint32_t>(id, 2, &n2);
        const uint64_t *noff = out_as<uint64_t>(id, 3, &n2);
        const uint32_t *nlen = out_as<uint32_t>(id, 4, &n2);
        const uint64_t *roff = out_as<uint64_t>(id, 5, &n2);
        const char *seq = out_as<char>(id, 6, &n2);
        const uint64_t *comp = out_as<uint64_t>(id, 7, &n2);
        write_chunks(o1, "", format_r2t_rows(t1.data(), noff, nlen, roff, seq, rec, hits, nwin, comp, min_pct, n, T));
    }
    tk_job_release(g_srv, id);
    {
        std::lock_guard<std::mutex> g(g_lat_mu);
        g_lat.push_back((double)lat / 1e6);
    }
    char b[128];
    std::snprintf(b, sizeof(b), "OK %llu %.3f %.3f", (unsigned long long)id, (double)lat / 1e6, (double)q / 1e6);
    return b;
}

static void serve_client(int fd) {
    std::string req;
    char buf[4096];
    ssize_t r;
    while ((r = ::read(fd, buf, sizeof(buf))) > 0) {
        req.append(buf, (size_t)r);
        if (req.find('\n') != std::string::npos) break;
    }
    req = req.substr(0, req.find('\n'));
    std::string ans = handle(req) + "\n";
    write_all(fd, ans.data(), ans.size(), "client");
    ::close(fd);
}

int main(int argc, char **argv) {
    std::string sock;
    int slots = 4, device = 0;
    double budget_gb = 150;
    for (int i = 1; i < argc; i++) {
        std::string a = argv[i];
        auto val = [&]() -> std::string {
            if (i + 1 >= argc) die("%s needs a value", a.c_str());
            return argv[++i];
        };
        if (a == "--socket") sock = val();
        else if (a == "--slots") slots = std::atoi(val().c_str());
        else if (a == "--budget-gb") budget_gb = std::atof(val().c_str());
        else if (a == "--device") device = std::atoi(val().c_str());
        else die("unknown option %s", a.c_str());
    }
    if (sock.empty()) die("--socket is required");
    check(tk_server_create(device, slots, (uint64_t)(budget_gb * 1e9), &g_srv), nullptr, "server create");
    int lfd = ::socket(AF_UNIX, SOCK_STREAM, 0);
    if (lfd < 0) die("socket: %s", std::strerror(errno));
    sockaddr_un addr{};
    addr.sun_family = AF_UNIX;
    if (sock.size() >= sizeof(addr.sun_path)) die("socket path too long");
    std::strcpy(addr.sun_path, sock.c_str());
    ::unlink(sock.c_str());
    if (::bind(lfd, (sockaddr *)&addr, sizeof(addr)) != 0) die("bind %s: %s", sock.c_str(), std::strerror(errno));
    if (::listen(lfd, 64) != 0) die("listen: %s", std::strerror(errno));
    std::fprintf(stderr, "trinkmerd: listening on %s (%d slots, %.1f GB budget)\n", sock.c_str(), slots, budget_gb);
    std::vector<std::thread> clients;
    while (!g_quit) {
        pollfd p{lfd, POLLIN, 0};
        int pr = ::poll(&p, 1, 200);   // wake up regularly to see a QUIT
        if (pr < 0 && errno != EINTR) break;
        if (pr <= 0) continue;
        int fd = ::accept(lfd, nullptr, nullptr);
        if (fd < 0) {
            if (errno == EINTR) continue;
            break;
        }
        clients.emplace_back(serve_client, fd);
    }
    for (auto &t : clients) t.join();
    ::close(lfd);
    ::unlink(sock.c_str());
    tk_server_destroy(g_srv);
    return 0;
}
