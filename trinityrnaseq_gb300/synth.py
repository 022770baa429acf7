"""Seeded synthetic workloads for the k-mer hot path (wrapper of csrc/synth.c).

The reference ships no benchmark data for this path, so inputs with the
shapes of the workloads below are generated; every byte depends only on the
seed and the parameters.

* ``transcriptome_reads``  2,000 transcripts (log-normal length, median 1,500,
  sigma 0.5, clipped to 300-8,000), log-normal expression (sigma 1.5),
  single-end 76-nt reads, 50/50 strand, 0.5% substitutions, FASTA.
* ``gene_pairs``           20,000 genes of 1-6 isoforms from shared exons
  (exon length log-normal, median 150), 2x100-nt pairs, fragment
  normal(300, 50), 1% substitutions, 0.01% N, constant-quality FASTQ.
* ``bundle_reads``         contigs (log-normal, median 400) grouped into
  components, written as '>s_<id>' records with contigs joined by 'X', plus
  2x100-nt reads from them at 1% error, one FASTA (all left then all right).
* ``power_law_bins``       bins with power-law (alpha 1.8) read counts, each
  from its own 1-20-transcript locus, 100-nt reads at 1% error.
"""
from __future__ import annotations

import ctypes as C
from pathlib import Path

import numpy as np

LIB = Path(__file__).resolve().parent / "lib" / "libtrinkmer_synth.so"
_lib = None


def _load() -> C.CDLL:
    global _lib
    if _lib is None:
        if not LIB.exists():
            from .build import build
            build()
        lib = C.CDLL(str(LIB))
        vp, u64, u32, d, P = C.c_void_p, C.c_uint64, C.c_uint32, C.c_double, C.POINTER
        lib.syn_se_reads.argtypes = [u64, u32, d, d, u32, u32, d, u64, u32, d, d, C.c_int, P(vp), P(C.c_size_t),
                                     P(u64)]
        lib.syn_pe_reads.argtypes = [u64, u32, d, d, u64, u32, d, d, d, d, C.c_int, P(vp), P(C.c_size_t), P(vp),
                                     P(C.c_size_t), P(u64), P(u32)]
        lib.syn_bundle.argtypes = [u64, u32, d, u32, u32, u64, u32, d, P(vp), P(C.c_size_t), P(vp), P(C.c_size_t),
                                   P(u64)]
        lib.syn_bins.argtypes = [u64, u32, d, u32, u32, u32, d, P(vp), P(C.c_size_t), vp, vp]
        lib.syn_free.argtypes = [vp]
        lib.syn_free.restype = None
        _lib = lib
    return _lib


def _take(p: C.c_void_p, n: int) -> np.ndarray:
    """Copies a generator buffer into a numpy uint8 array and frees it."""
    lib = _load()
    out = np.empty(n, dtype=np.uint8)
    if n:
        C.memmove(out.ctypes.data, p, n)
    lib.syn_free(p)
    return out


def _chk(st: int, what: str) -> None:
    if st != 0:
        raise RuntimeError(f"synthetic generator {what} failed with status {st}")


def transcriptome_reads(seed: int = 1, n_transcripts: int = 2000, n_reads: int = 1_000_000, read_len: int = 76,
                        err: float = 0.005, n_rate: float = 0.0, fastq: bool = False, len_median: float = 1500.0,
                        len_sigma: float = 0.5, len_min: int = 300, len_max: int = 8000,
                        expr_sigma: float = 1.5) -> np.ndarray:
    lib = _load()
    p, n, tb = C.c_void_p(), C.c_size_t(), C.c_uint64()
    _chk(lib.syn_se_reads(seed, n_transcripts, len_median, len_sigma, len_min, len_max, expr_sigma, n_reads,
                          read_len, err, n_rate, int(fastq), C.byref(p), C.byref(n), C.byref(tb)), "se_reads")
    return _take(p, n.value)


def gene_pairs(seed: int = 2, n_genes: int = 20000, n_pairs: int = 20_000_000, read_len: int = 100,
               frag_mean: float = 300.0, frag_sd: float = 50.0, err: float = 0.01, n_rate: float = 0.0001,
               fastq: bool = True, exon_median: float = 150.0, expr_sigma: float = 1.5):
    """(left, right) mates as uint8 arrays."""
    lib = _load()
    lp, ln, rp, rn, tb, nt = C.c_void_p(), C.c_size_t(), C.c_void_p(), C.c_size_t(), C.c_uint64(), C.c_uint32()
    _chk(lib.syn_pe_reads(seed, n_genes, exon_median, expr_sigma, n_pairs, read_len, frag_mean, frag_sd, err, n_rate,
                          int(fastq), C.byref(lp), C.byref(ln), C.byref(rp), C.byref(rn), C.byref(tb), C.byref(nt)),
         "pe_reads")
    return _take(lp, ln.value), _take(rp, rn.value)


def bundle_reads(seed: int = 4, n_contigs: int = 100_000, contig_median: float = 400.0, n_components: int = 30_000,
                 max_per_component: int = 40, n_pairs: int = 50_000_000, read_len: int = 100, err: float = 0.01):
    """(bundle FASTA, reads FASTA) as uint8 arrays."""
    lib = _load()
    bp, bn, rp, rn, cb = C.c_void_p(), C.c_size_t(), C.c_void_p(), C.c_size_t(), C.c_uint64()
    _chk(lib.syn_bundle(seed, n_contigs, contig_median, n_components, max_per_component, n_pairs, read_len, err,
                        C.byref(bp), C.byref(bn), C.byref(rp), C.byref(rn), C.byref(cb)), "bundle")
    return _take(bp, bn.value), _take(rp, rn.value)


def power_law_bins(seed: int = 3, n_bins: int = 5000, alpha: float = 1.8, min_reads: int = 50,
                   max_reads: int = 200_000, read_len: int = 100, err: float = 0.01):
    """(FASTA of all bins back to back, byte offsets [n_bins+1], reads per bin)."""
    lib = _load()
    p, n = C.c_void_p(), C.c_size_t()
    off = np.zeros(n_bins + 1, dtype=np.uint64)
    cnt = np.zeros(n_bins, dtype=np.uint64)
    _chk(lib.syn_bins(seed, n_bins, alpha, min_reads, max_reads, read_len, err, C.byref(p), C.byref(n),
                      off.ctypes.data, cnt.ctypes.data), "bins")
    return _take(p, n.value), off, cnt
