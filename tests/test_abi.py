"""The C-ABI library loads and exports every function include/trinkmer.h
declares; without a GPU it refuses to run (no CPU fallback).  CPU only."""
import ctypes as C
import re
import shutil
import subprocess

import pytest

from tests.conftest import ROOT


def declared_symbols():
    out = set()
    for h in (ROOT / "include").glob("*.h"):
        text = re.sub(r"/\*.*?\*/", "", h.read_text(), flags=re.S)
        out |= set(re.findall(r"\b(tk_\w+)\s*\(", text))
    return out


def test_header_declares_the_entry_points():
    syms = declared_symbols()
    for s in ("tk_ctx_create", "tk_reads_parse", "tk_table_add_reads", "tk_table_dump_fasta", "tk_table_histo",
              "tk_table_load_dump_fasta", "tk_coverage_stats", "tk_r2t_create", "tk_r2t_assign"):
        assert s in syms


def test_library_exports_every_declared_symbol(native_built):
    lib = C.CDLL(str(native_built["cuda"]))
    missing = [s for s in sorted(declared_symbols()) if not hasattr(lib, s)]
    assert not missing, missing


def test_binding_covers_the_header(native_built):
    from trinityrnaseq_gb300 import native
    missing = [s for s in declared_symbols() if s not in native.SIGNATURES]
    assert not missing, missing


def _has_gpu() -> bool:
    if shutil.which("nvidia-smi") is None:
        return False
    return subprocess.run(["nvidia-smi", "-L"], stdout=subprocess.DEVNULL, stderr=subprocess.DEVNULL).returncode == 0


@pytest.mark.skipif(_has_gpu(), reason="a GPU is present")
def test_no_gpu_means_no_context(native_built):
    from trinityrnaseq_gb300 import Context, native
    with pytest.raises(native.TrinkmerError) as ei:
        Context(0)
    assert ei.value.status in (native.TK_E_NODEV, native.TK_E_CUDA)


def test_status_strings(native_built):
    from trinityrnaseq_gb300 import native
    lib = native.load()
    assert lib.tk_status_string(native.TK_E_TABLE_FULL) == b"hash table full"
    assert b"sm_103a" in lib.tk_version()
