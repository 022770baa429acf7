// tk_tool.hpp -- host helpers shared by the drop-in executables.
//
// The reference's tools are separate processes that Perl starts with
// system(); success is exit code 0 and any failure is a non-zero code with a
// message on stderr (PerlLib/Pipeliner.pm:176-188).  Outputs named on the
// command line are written to a temporary file and renamed into place, so a
// crash never leaves a file that passes the driver's `-s file` checks
// (util/insilico_read_normalization.pl:907, Trinity:1841).
#pragma once

#include <cerrno>
#include <cstdarg>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <thread>
#include <vector>

#include <fcntl.h>
#include <sys/stat.h>
#include <unistd.h>

#include "trinkmer.h"

namespace tool {

[[noreturn]] inline void die(const char *fmt, ...) {
    va_list ap;
    va_start(ap, fmt);
    std::fputs("Error: ", stderr);
    std::vfprintf(stderr, fmt, ap);
    std::fputc('\n', stderr);
    va_end(ap);
    std::exit(1);
}

// aborts with the context's error text on a non-zero status
inline void check(int st, tk_ctx *ctx, const char *what) {
    if (st != TK_OK)
        die("%s failed: %s%s%s", what, tk_status_string(st), ctx ? ": " : "", ctx ? tk_ctx_last_error(ctx) : "");
}

inline std::vector<char> read_file(const std::string &path) {
    std::vector<char> buf;
    FILE *f = std::fopen(path.c_str(), "rb");
    if (!f) die("cannot open %s: %s", path.c_str(), std::strerror(errno));
    struct stat st;
    if (fstat(fileno(f), &st) == 0 && st.st_size > 0) buf.reserve((size_t)st.st_size);
    char tmp[1 << 16];
    size_t n;
    // read in large blocks; works for pipes and /dev/stdin too
    std::vector<char> big(1 << 24);
    while ((n = std::fread(big.data(), 1, big.size(), f)) > 0) buf.insert(buf.end(), big.data(), big.data() + n);
    (void)tmp;
    if (std::ferror(f)) die("cannot read %s: %s", path.c_str(), std::strerror(errno));
    std::fclose(f);
    return buf;
}

inline void write_all(int fd, const char *p, size_t n, const std::string &what) {
    while (n) {
        ssize_t w = ::write(fd, p, n);
        if (w < 0) {
            if (errno == EINTR) continue;
            die("cannot write %s: %s", what.c_str(), std::strerror(errno));
        }
        p += w;
        n -= (size_t)w;
    }
}

// Writes to path.tmp.<pid> and renames it to path on commit().
class AtomicFile {
  public:
    explicit AtomicFile(const std::string &path) : path_(path), tmp_(path + ".tmp." + std::to_string(getpid())) {
        fd_ = ::open(tmp_.c_str(), O_WRONLY | O_CREAT | O_TRUNC, 0644);
        if (fd_ < 0) die("cannot create %s: %s", tmp_.c_str(), std::strerror(errno));
    }
    ~AtomicFile() {
        if (fd_ >= 0) {
            ::close(fd_);
            ::unlink(tmp_.c_str());
        }
    }
    void write(const char *p, size_t n) { write_all(fd_, p, n, tmp_); }
    void write(const std::string &s) { write(s.data(), s.size()); }
    void commit() {
        if (::close(fd_) != 0) die("cannot close %s: %s", tmp_.c_str(), std::strerror(errno));
        fd_ = -1;
        if (std::rename(tmp_.c_str(), path_.c_str()) != 0)
            die("cannot rename %s to %s: %s", tmp_.c_str(), path_.c_str(), std::strerror(errno));
    }

  private:
    std::string path_, tmp_;
    int fd_ = -1;
};

inline int host_threads(int requested) {
    int hw = (int)std::thread::hardware_concurrency();
    if (hw <= 0) hw = 1;
    return requested > 0 ? std::min(requested, hw) : hw;
}

// Formats items [0, n) in `threads` contiguous chunks, each into its own
// string, and returns the chunks in order.
template <typename F>
std::vector<std::string> format_parallel(uint64_t n, int threads, F &&fmt_range) {
    int T = (int)std::max<uint64_t>(1, std::min<uint64_t>((uint64_t)threads, (n + 4095) / 4096));
    std::vector<std::string> out((size_t)T);
    std::vector<std::thread> pool;
    for (int t = 0; t < T; t++) {
        uint64_t lo = n * t / T, hi = n * (t + 1) / T;
        pool.emplace_back([&, t, lo, hi] { fmt_range(lo, hi, out[(size_t)t]); });
    }
    for (auto &th : pool) th.join();
    return out;
}

inline bool parse_u64(const char *s, uint64_t *v) {
    if (!s || !*s) return false;
    char *end = nullptr;
    errno = 0;
    double d = std::strtod(s, &end);   // jellyfish accepts sizes like 1e9 or 100M
    if (end && (*end == 'k' || *end == 'K')) { d *= 1e3; end++; }
    else if (end && (*end == 'M' || *end == 'm')) { d *= 1e6; end++; }
    else if (end && (*end == 'G' || *end == 'g')) { d *= 1e9; end++; }
    if (errno || !end || *end || d < 0) return false;
    *v = (uint64_t)d;
    return true;
}

// fastaToKmerCoverageStats rows "acc\tmedian\tmean\tstdev\n" (%g, a C++ ostream's default)
inline std::vector<std::string> format_stats_rows(const char *text, const uint64_t *noff, const uint32_t *nlen,
                                                  const uint32_t *med, const float *mean, const float *sd,
                                                  uint64_t n, int threads) {
    return format_parallel(n, threads, [&](uint64_t lo, uint64_t hi, std::string &s) {
        s.reserve((hi - lo) * 48);
        char line[128];
        for (uint64_t i = lo; i < hi; i++) {
            s.append(text + noff[i], nlen[i]);
            int L = std::snprintf(line, sizeof(line), "\t%u\t%g\t%g\n", med[i], (double)mean[i], (double)sd[i]);
            s.append(line, (size_t)L);
        }
    });
}

// readsToComponents rows "comp\t>acc\tpct\tSEQ\n"; reads without a component
// or below min_pct percent are left out
inline std::vector<std::string> format_r2t_rows(const char *text, const uint64_t *noff, const uint32_t *nlen,
                                                const uint64_t *roff, const char *seq, const int32_t *rec,
                                                const uint32_t *hits, const uint32_t *nwin, const uint64_t *comp,
                                                int min_pct, uint64_t n, int threads) {
    return format_parallel(n, threads, [&](uint64_t lo, uint64_t hi, std::string &s) {
        char head[64];
        for (uint64_t i = lo; i < hi; i++) {
            if (rec[i] < 0 || nwin[i] == 0) continue;
            uint32_t pct = (uint32_t)((100ull * hits[i]) / nwin[i]);
            if (min_pct > 0 && pct < (uint32_t)min_pct) continue;
            int L = std::snprintf(head, sizeof(head), "%llu\t>", (unsigned long long)comp[(size_t)rec[i]]);
            s.append(head, (size_t)L);
            s.append(text + noff[i], nlen[i]);
            L = std::snprintf(head, sizeof(head), "\t%u\t", pct);
            s.append(head, (size_t)L);
            s.append(seq + roff[i], roff[i + 1] - roff[i] - 1);
            s.push_back('\n');
        }
    });
}

inline tk_ctx *open_ctx() {
    tk_ctx *ctx = nullptr;
    int dev = 0;
    if (const char *e = std::getenv("TK_DEVICE")) dev = std::atoi(e);
    int st = tk_ctx_create(dev, &ctx);
    if (st != TK_OK) die("cannot open CUDA device %d: %s", dev, tk_status_string(st));
    return ctx;
}

}  // namespace tool
