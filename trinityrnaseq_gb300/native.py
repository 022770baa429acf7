"""ctypes binding of ``lib/libtrinkmer_cuda.so`` (declared in ``include/trinkmer.h``).

The shared library is the only compute path: if it is missing or no GPU is
present, the calls raise; there is no CPU fallback in this package.
"""
from __future__ import annotations

import ctypes as C
import os
from pathlib import Path

PKG = Path(__file__).resolve().parent
LIB_PATH = PKG / "lib" / "libtrinkmer_cuda.so"

TK_OK = 0
TK_E_INVAL = -1
TK_E_CUDA = -2
TK_E_OOM = -3
TK_E_PARSE = -4
TK_E_TABLE_FULL = -5
TK_E_BUDGET = -6
TK_E_NODEV = -7
TK_E_RANGE = -8

TK_HOST = 0
TK_DEVICE = 1

TK_FMT_NONE, TK_FMT_FASTA, TK_FMT_FASTQ = 0, 1, 2

TK_FA_REVCOMP, TK_FA_IGNORE_DIRTY, TK_FA_IF_MISSING = 1, 2, 4

KID = {
    "parse": 0, "hll": 1, "count": 2, "compact": 3, "sort": 4, "dump": 5, "load": 6,
    "coverage": 7, "r2t_build": 8, "r2t_assign": 9, "bins": 10, "scatter": 11, "norm": 12, "extract": 13,
    "cov_cache": 14, "dbg": 15,
}

u64, u32, i32, vp = C.c_uint64, C.c_uint32, C.c_int32, C.c_void_p
P = C.POINTER

# name -> (restype, argtypes); every symbol include/trinkmer.h declares
SIGNATURES = {
    "tk_version": (C.c_char_p, []),
    "tk_status_string": (C.c_char_p, [C.c_int]),
    "tk_ctx_create": (C.c_int, [C.c_int, P(vp)]),
    "tk_ctx_destroy": (None, [vp]),
    "tk_ctx_last_error": (C.c_char_p, [vp]),
    "tk_ctx_stream": (vp, [vp]),
    "tk_ctx_synchronize": (C.c_int, [vp]),
    "tk_ctx_set_profiling": (C.c_int, [vp, C.c_int]),
    "tk_ctx_profile": (C.c_int, [vp, C.c_int, P(C.c_double), P(u64), P(u64)]),
    "tk_ctx_reset_profile": (C.c_int, [vp]),
    "tk_ctx_kernel_launches": (u64, [vp]),
    "tk_ctx_mem_info": (C.c_int, [vp, P(u64), P(u64)]),
    "tk_ctx_set_reprobes": (C.c_int, [vp, C.c_int]),
    "tk_ctx_random_access_rate": (C.c_int, [vp, u64, C.c_int, P(C.c_double)]),
    "tk_ctx_trim": (C.c_int, [vp]),
    "tk_reads_parse": (C.c_int, [vp, vp, u64, C.c_int, P(vp)]),
    "tk_reads_parse_many": (C.c_int, [vp, P(vp), P(u64), u32, C.c_int, P(vp)]),
    "tk_split_records": (C.c_int, [vp, u64, u32, P(u64)]),
    "tk_reads_to_fasta": (C.c_int, [vp, C.c_int, C.c_int, C.c_int, vp, u64, P(u64)]),
    "tk_reads_info": (C.c_int, [vp, P(u64), P(u64), P(u32), P(C.c_int)]),
    "tk_reads_names": (C.c_int, [vp, vp, vp]),
    "tk_reads_offsets": (C.c_int, [vp, vp]),
    "tk_reads_copy_seq": (C.c_int, [vp, vp, u64]),
    "tk_reads_free": (None, [vp]),
    "tk_table_create": (C.c_int, [vp, C.c_int, C.c_int, u64, P(vp)]),
    "tk_table_add_reads": (C.c_int, [vp, vp]),
    "tk_table_add_reads_multi": (C.c_int, [vp, P(vp), u32]),
    "tk_table_count_texts": (C.c_int, [vp, P(vp), P(u64), u32, C.c_int, P(vp)]),
    "tk_table_count_text": (C.c_int, [vp, vp, u64, C.c_int]),
    "tk_table_info": (C.c_int, [vp, P(u64), P(u64), P(u64)]),
    "tk_table_histo": (C.c_int, [vp, u64, u64, vp]),
    "tk_table_dump": (C.c_int, [vp, u32, C.c_int, vp, vp, u64, P(u64)]),
    "tk_table_dump_fasta": (C.c_int, [vp, u32, C.c_int, vp, u64, P(u64)]),
    "tk_table_dump_fasta_async": (C.c_int, [vp, u32, vp, u64, P(u64)]),
    "tk_table_load_pairs": (C.c_int, [vp, vp, vp, u64, C.c_int]),
    "tk_table_load_dump_fasta": (C.c_int, [vp, vp, u64, C.c_int]),
    "tk_table_free": (None, [vp]),
    "tk_coverage_stats": (C.c_int, [vp, vp, C.c_int, vp, vp, vp]),
    "tk_coverage_stats_noalloc": (C.c_int, [vp, vp, vp, vp, vp]),
    "tk_r2t_create": (C.c_int, [vp, vp, u64, C.c_int, C.c_int, C.c_int, P(vp)]),
    "tk_r2t_info": (C.c_int, [vp, P(u64), P(u64)]),
    "tk_r2t_component_ids": (C.c_int, [vp, vp]),
    "tk_r2t_assign": (C.c_int, [vp, vp, C.c_int, vp, vp, vp]),
    "tk_r2t_free": (None, [vp]),
    "tk_norm_select": (C.c_int, [vp, vp, vp, vp, vp, vp, vp, vp, vp, C.c_int, C.c_int, C.c_int, C.c_int, P(vp)]),
    "tk_norm_select_multi": (C.c_int, [vp, vp, u32, vp, vp, vp, vp, u32, vp, vp, vp, C.c_int, C.c_int, C.c_int,
                                       C.c_int, P(vp)]),
    "tk_norm_info": (C.c_int, [vp, vp, P(u64)]),
    "tk_norm_accs": (C.c_int, [vp, C.c_int, vp, u64]),
    "tk_norm_table": (C.c_int, [vp, C.c_int, vp, u64, P(u64)]),
    "tk_norm_extract": (C.c_int, [vp, vp, P(u64)]),
    "tk_norm_extract_multi": (C.c_int, [vp, vp, u32, P(u64)]),
    "tk_norm_extract_copy": (C.c_int, [vp, C.c_int, vp, u64]),
    "tk_norm_extract_copy_async": (C.c_int, [vp, vp, u64]),
    "tk_dbg_create": (C.c_int, [vp, vp, u64, C.c_int, C.c_int, C.c_int, P(vp)]),
    "tk_dbg_info": (C.c_int, [vp, P(u64), P(u64), P(u64)]),
    "tk_dbg_text": (C.c_int, [vp, C.c_int, vp, u64]),
    "tk_dbg_free": (None, [vp]),
    "tk_norm_free": (None, [vp]),
    "tk_count_bins": (C.c_int, [vp, vp, u64, C.c_int, vp, u32, C.c_int, C.c_int, u32, P(vp)]),
    "tk_count_bins_ex": (C.c_int, [vp, vp, u64, C.c_int, vp, u32, C.c_int, C.c_int, vp, vp, P(vp)]),
    "tk_bins_info": (C.c_int, [vp, P(u64), P(u64)]),
    "tk_bins_dump_offsets": (C.c_int, [vp, vp]),
    "tk_bins_dump_text": (C.c_int, [vp, vp, u64]),
    "tk_bins_tuning": (C.c_int, [vp, P(C.c_int), P(C.c_int), P(C.c_int)]),
    "tk_bins_free": (None, [vp]),
}


TK_JOB_COUNT, TK_JOB_NORMALIZE, TK_JOB_R2T = 1, 2, 3


class JobSpec(C.Structure):
    _fields_ = [("kind", C.c_int), ("k", C.c_int), ("canonical", C.c_int), ("strand", C.c_int),
                ("min_count", C.c_uint32), ("text", C.c_void_p), ("len", C.c_uint64), ("text2", C.c_void_p),
                ("len2", C.c_uint64), ("max_cov", C.c_int), ("min_cov", C.c_int), ("max_cv", C.c_int)]


SIGNATURES.update({
    "tk_server_create": (C.c_int, [C.c_int, C.c_int, u64, P(vp)]),
    "tk_server_submit": (C.c_int, [vp, P(JobSpec), P(u64)]),
    "tk_server_wait": (C.c_int, [vp, u64, P(C.c_int), P(u64), P(u64)]),
    "tk_job_output": (C.c_int, [vp, u64, C.c_int, P(vp), P(u64)]),
    "tk_job_error": (C.c_char_p, [vp, u64]),
    "tk_job_release": (C.c_int, [vp, u64]),
    "tk_server_stats": (C.c_int, [vp, P(u64), P(u64), P(C.c_int)]),
    "tk_server_destroy": (None, [vp]),
    "tk_server_batched_jobs": (C.c_int, [vp, P(u64)]),
    "tk_server_held_by_free_memory": (C.c_int, [vp, P(u64)]),
})


class TrinkmerError(RuntimeError):
    def __init__(self, status: int, where: str, detail: str = ""):
        self.status = status
        msg = f"{where}: status {status}"
        if _lib is not None:
            msg += f" ({_lib.tk_status_string(status).decode()})"
        if detail:
            msg += f": {detail}"
        super().__init__(msg)


_lib = None


def load() -> C.CDLL:
    """Loads the CUDA library once; raises if it was not built."""
    global _lib
    if _lib is not None:
        return _lib
    path = Path(os.environ.get("TRINKMER_LIB", LIB_PATH))
    if not path.exists():
        raise RuntimeError(f"{path} is missing: build it first (python -c 'import __graft_entry__ as g; g.build()')")
    lib = C.CDLL(str(path))
    for name, (res, args) in SIGNATURES.items():
        fn = getattr(lib, name, None)
        if fn is None:
            continue
        fn.restype = res
        fn.argtypes = args
    _lib = lib
    return lib


def check(status: int, where: str, ctx=None) -> None:
    if status != TK_OK:
        detail = ""
        if ctx is not None and _lib is not None:
            detail = (_lib.tk_ctx_last_error(ctx) or b"").decode(errors="replace")
        raise TrinkmerError(status, where, detail)
