"""Shared test helpers: k-mer encoding and the orderings the reference uses."""
from __future__ import annotations

import gzip
from collections import Counter
from pathlib import Path

import numpy as np

CODE = {c: i for i, c in enumerate("ACGT")}
COMP = str.maketrans("ACGT", "TGCA")


def encode(kmer: str) -> int:
    v = 0
    for ch in kmer:
        v = (v << 2) | CODE[ch]
    return v


def revcomp(s: str) -> str:
    return s.translate(COMP)[::-1]


def is_acgt(s: str) -> bool:
    return all(c in "ACGT" for c in s.upper())


def canonical_counts_from_windows(windows, canonical=True) -> dict:
    """jellyfish count semantics over a list of window strings."""
    cnt = Counter()
    for w in windows:
        if not is_acgt(w):
            continue
        w = w.upper()
        if canonical:
            r = revcomp(w)
            w = min(w, r)
        cnt[w] += 1
    return dict(cnt)


def kmer_counter_to_canonical(text: bytes) -> dict:
    """Turns util/misc/kmer_counter.pl DS-mode output (each window and its
    reverse complement counted as strings) into canonical counts: windows with
    a non-ACGT character are dropped, case is folded, and the count of a
    canonical key is the DS count of that key (odd k has no palindromes)."""
    folded = Counter()
    for line in text.decode().splitlines():
        kmer, c = line.split("\t")
        if not is_acgt(kmer):
            continue
        folded[kmer.upper()] += int(c)
    return {k: v for k, v in folded.items() if k <= revcomp(k)}


def dict_to_arrays(d: dict):
    items = sorted((encode(k), v) for k, v in d.items())
    return (np.array([a for a, _ in items], dtype=np.uint64), np.array([b for _, b in items], dtype=np.uint32))


def read_gz(p: Path) -> bytes:
    return gzip.decompress(p.read_bytes())


def trinity_r2t_sort(rows: bytes) -> bytes:
    """`sort -k1,1n -k3,3nr -k2,2` under LC_ALL=C (Trinity:2258), with sort's
    last-resort whole-line byte comparison."""
    lines = [l for l in rows.split(b"\n") if l]

    def key(l):
        f = l.split(b"\t")
        return (int(f[0]), -int(f[2]), f[1], l)

    return b"".join(l + b"\n" for l in sorted(lines, key=key))


def sort_stats(text: bytes) -> bytes:
    """head -n1 + `sort -k1,1` of the rest (util/insilico_read_normalization.pl:874)."""
    lines = text.split(b"\n")
    head, body = lines[0], [l for l in lines[1:] if l]
    body.sort(key=lambda l: (l.split(b"\t", 1)[0], l))
    return head + b"\n" + b"".join(l + b"\n" for l in body)
