"""GB300-native Trinity k-mer hot path.

Drop-in replacements for the three native tools Trinity drives on this path
-- ``jellyfish count/histo/dump`` (canonical k=25 counting), Inchworm's
``fastaToKmerCoverageStats`` and Chrysalis' ``ReadsToTranscripts`` -- and for
Inchworm's ``FastaToDeBruijn`` per-component graphs and
the steps around them (``seqtk-trinity`` read prep, the in-silico
normalization's sort / pair merge / selection / extraction), built on
hand-written sm_103a CUDA kernels behind the C ABI in ``include/trinkmer.h``.
"""
from .kmer import (Context, DeBruijnGraphs, KmerTable, Normalization, ReadSet, ReadsToTranscripts, coverage_stats,
                   format_histo, format_r2t, format_stats)

__all__ = ["Context", "DeBruijnGraphs", "KmerTable", "Normalization", "ReadSet", "ReadsToTranscripts",
           "coverage_stats", "format_histo", "format_stats", "format_r2t"]
