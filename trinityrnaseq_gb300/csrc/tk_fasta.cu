// tk_fasta.cu -- FASTQ -> FASTA read prep on the GPU: the conversion Trinity
// runs before counting (`seqtk-trinity seq -A -R {1,2} [-r]`, Trinity:2745-2805),
// whose executable spec is util/support_scripts/fastQ_to_fastA.pl:60-118.
//
// Input is a parsed FASTQ read set (tk_reads_parse has checked the 4-line
// structure: '@' header, '+' third line).  One thread per record re-reads the
// record's four lines from the device copy of the text and applies the
// script's rules:
//   * only the header loses its CRs; sequence and quality lines lose just
//     their "\n" (a CRLF sequence keeps its CR, as the script prints it);
//   * a record is clean when its sequence is non-empty and not "0", and its
//     quality line holds a non-space byte and is as long as the sequence;
//   * name = first whitespace-separated field after '@' (empty if the header
//     starts with whitespace); "/1" or "/2" is added when another field
//     follows, the name does not end in /1 or /2 and that field starts "1:"
//     or "2:" (Casava 1.8); then "/append" (every name, the script's -a, or
//     with TK_FA_IF_MISSING only names not ending in /1 or /2);
//   * TK_FA_REVCOMP maps each byte through ACGTacgtyrkmYRKMUu ->
//     TGCAtgcarymkRYMKAa in reverse order (PerlLib/Nuc_translator.pm:286-292).
// Pass 1 sizes every record's output (0 for a skipped record), a scan places
// them, pass 2 writes ">" name suffix "\n" sequence "\n".
#include "tk_internal.cuh"

#include <string>

namespace tk {

constexpr int FA_THREADS = 256;

__device__ __forceinline__ bool pl_ws(uint32_t c) { return c == ' ' || c - 9u < 5u; }

__device__ __forceinline__ uint8_t rc_letter(uint8_t c) {
    switch (c) {
        case 'A': return 'T'; case 'C': return 'G'; case 'G': return 'C'; case 'T': return 'A';
        case 'a': return 't'; case 'c': return 'g'; case 'g': return 'c'; case 't': return 'a';
        case 'y': return 'r'; case 'r': return 'y'; case 'k': return 'm'; case 'm': return 'k';
        case 'Y': return 'R'; case 'R': return 'Y'; case 'K': return 'M'; case 'M': return 'K';
        case 'U': return 'A'; case 'u': return 'a';
        default: return c;
    }
}

__device__ __forceinline__ uint64_t line_end(const char *__restrict__ t, uint64_t len, uint64_t p) {
    while (p < len && t[p] != '\n') p++;
    return p;
}

// decimal digits of v (v >= 0)
__device__ __forceinline__ uint32_t n_digits(uint32_t v) {
    uint32_t d = 1;
    while (v >= 10) { v /= 10; d++; }
    return d;
}

struct FaRec {
    uint64_t name0, name1;   // header bytes [name0, name1) hold the first field (CRs skipped when copied)
    uint32_t name_len;       // the field's length without CRs
    uint64_t seq0;           // sequence line
    uint32_t seq_len;        // bytes before its "\n", CRs included
    uint32_t suffix;         // 0 none, else the Casava mate digit ('1' or '2')
    bool ends12;             // the name ends in /1 or /2
    bool clean;
};

__device__ FaRec fa_record(const char *__restrict__ t, uint64_t len, uint64_t at) {
    FaRec f;
    const uint64_t he = line_end(t, len, at);
    const uint64_t s0 = he + 1, se = line_end(t, len, s0);
    const uint64_t p0 = se + 1, pe = line_end(t, len, p0);
    const uint64_t q0 = pe + 1, qe = line_end(t, len, q0);
    // first field of the header (after '@'), CRs removed before splitting
    uint64_t p = at + 1;
    uint32_t nl = 0;
    uint8_t last = 0, prev = 0;
    while (p < he) {
        const uint8_t c = (uint8_t)t[p];
        if (c != '\r') {
            if (pl_ws(c)) break;
            prev = last;
            last = c;
            nl++;
        }
        p++;
    }
    f.name0 = at + 1;
    f.name1 = p;
    f.name_len = nl;
    f.ends12 = nl >= 2 && prev == '/' && (last == '1' || last == '2');
    // the next field: "1:" or "2:" adds the mate suffix
    while (p < he && (pl_ws((uint8_t)t[p]) || t[p] == '\r')) p++;
    f.suffix = 0;
    if (p < he && !f.ends12) {
        uint8_t a = 0, b = 0;
        uint64_t q = p;
        while (q < he && t[q] == '\r') q++;
        if (q < he) a = (uint8_t)t[q++];
        while (q < he && t[q] == '\r') q++;
        if (q < he) b = (uint8_t)t[q];
        if ((a == '1' || a == '2') && b == ':') f.suffix = a;
    }
    f.seq0 = s0;
    const uint64_t sl = se > s0 ? se - s0 : 0, ql = qe > q0 ? qe - q0 : 0;
    f.seq_len = (uint32_t)sl;
    bool ok = s0 < len && q0 <= len && sl > 0 && !(sl == 1 && t[s0] == '0') && ql == sl;
    if (ok) {
        bool ns = false;
        for (uint64_t i = q0; i < qe && !ns; i++) ns = !pl_ws((uint8_t)t[i]);
        ok = ns;
    }
    f.clean = ok;
    return f;
}

__device__ __forceinline__ uint32_t fa_suffix_len(const FaRec &f, int append, int flags) {
    uint32_t n = f.suffix ? 2u : 0u;
    if (append >= 0 && !((flags & TK_FA_IF_MISSING) && (f.ends12 || f.suffix))) n += 1u + n_digits((uint32_t)append);
    return n;
}

__global__ void k_fa_len(const char *__restrict__ text, uint64_t len, const uint64_t *__restrict__ name_off,
                         uint64_t n, int append, int flags, uint32_t *__restrict__ out_len,
                         unsigned long long *__restrict__ first_bad) {
    const uint64_t r = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (r >= n) return;
    const FaRec f = fa_record(text, len, name_off[r] - 1);
    if (!f.clean) {
        out_len[r] = 0;
        if (!(flags & TK_FA_IGNORE_DIRTY)) atomicMin(first_bad, (unsigned long long)r);
        return;
    }
    out_len[r] = 1u + f.name_len + fa_suffix_len(f, append, flags) + 1u + f.seq_len + 1u;
}

__global__ void k_fa_write(const char *__restrict__ text, uint64_t len, const uint64_t *__restrict__ name_off,
                           uint64_t n, int append, int flags, const uint64_t *__restrict__ out_off,
                           char *__restrict__ out) {
    const uint64_t r = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (r >= n) return;
    if (out_off[r + 1] == out_off[r]) return;   // skipped record
    const FaRec f = fa_record(text, len, name_off[r] - 1);
    char *o = out + out_off[r];
    *o++ = '>';
    for (uint64_t p = f.name0; p < f.name1; p++)
        if (text[p] != '\r') *o++ = text[p];
    if (f.suffix) {
        *o++ = '/';
        *o++ = (char)f.suffix;
    }
    if (append >= 0 && !((flags & TK_FA_IF_MISSING) && (f.ends12 || f.suffix))) {
        *o++ = '/';
        const uint32_t d = n_digits((uint32_t)append);
        uint32_t v = (uint32_t)append;
        for (uint32_t i = 0; i < d; i++) {
            o[d - 1 - i] = (char)('0' + v % 10);
            v /= 10;
        }
        o += d;
    }
    *o++ = '\n';
    if (flags & TK_FA_REVCOMP)
        for (uint32_t i = 0; i < f.seq_len; i++) *o++ = (char)rc_letter((uint8_t)text[f.seq0 + f.seq_len - 1 - i]);
    else
        for (uint32_t i = 0; i < f.seq_len; i++) *o++ = text[f.seq0 + i];
    *o = '\n';
}

// FASTA text of a FASTQ read set into *d_text (device, caller frees with dfree).
int reads_fasta(tk_reads *r, int append, int flags, char **d_text, uint64_t *text_len) {
    tk_ctx *c = r->ctx;
    *d_text = nullptr;
    *text_len = 0;
    const uint64_t n = r->n_reads;
    uint32_t *lens = nullptr;
    uint64_t *offs = nullptr;
    unsigned long long *bad = nullptr;
    TK_TRY(dmalloc(c, (void **)&lens, (n ? n : 1) * 4, "fasta record lengths"));
    int e = dmalloc(c, (void **)&offs, (n + 1) * 8, "fasta record offsets");
    if (!e) e = dmalloc(c, (void **)&bad, 8, "fasta first bad record");
    if (!e) e = cuda_check(c, cudaMemsetAsync(bad, 0xFF, 8, c->stream), "bad reset");
    const unsigned grid = (unsigned)((n + FA_THREADS - 1) / FA_THREADS);
    if (!e && n) {
        k_fa_len<<<grid, FA_THREADS, 0, c->stream>>>(r->d_text, r->text_len, r->d_name_off, n, append, flags, lens, bad);
        c->launches++;
        e = check_launch(c, "fasta lengths");
    }
    unsigned long long hbad = ~0ULL;
    uint64_t total = 0;
    if (!e && n) e = scan_excl_u32_to_u64(c, lens, offs, n, &total);   // synchronises
    if (!e) e = cuda_check(c, cudaMemcpyAsync(&hbad, bad, 8, cudaMemcpyDeviceToHost, c->stream), "bad d2h");
    if (!e) e = cuda_check(c, cudaStreamSynchronize(c->stream), "fasta sync");
    if (!e && hbad != ~0ULL)
        e = set_err(c, TK_E_PARSE, "FASTQ input: improperly formatted entry (record " + std::to_string(hbad + 1) + ")");
    if (!e && n) {
        cudaMemcpyAsync(offs + n, &total, 8, cudaMemcpyHostToDevice, c->stream);
        e = dmalloc(c, (void **)d_text, total ? total : 1, "fasta text");
        if (!e && total) {
            k_fa_write<<<grid, FA_THREADS, 0, c->stream>>>(r->d_text, r->text_len, r->d_name_off, n, append, flags, offs,
                                                           *d_text);
            c->launches++;
            e = check_launch(c, "fasta write");
        }
    }
    if (!e) *text_len = total;
    dfree(c, lens);
    dfree(c, offs);
    if (bad) dfree(c, bad);
    if (e && *d_text) {
        dfree(c, *d_text);
        *d_text = nullptr;
    }
    return e;
}

}  // namespace tk
