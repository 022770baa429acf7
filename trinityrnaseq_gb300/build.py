"""In-tree build of the native parts of the package.

* ``lib/libtrinkmer_cuda.so`` -- the CUDA kernels and the C ABI
  (``include/trinkmer.h``), compiled for sm_103a only.
* ``lib/libtrinkmer_synth.so`` -- the seeded synthetic-input generator (C).
* ``bin/jellyfish``, ``bin/fastaToKmerCoverageStats``, ``bin/ReadsToTranscripts``
  -- the drop-in executables (C++ host code over the C ABI).

Translation units are compiled in parallel; nothing is installed outside the
package directory.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys
from pathlib import Path

PKG = Path(__file__).resolve().parent
ROOT = PKG.parent
CSRC = PKG / "csrc"
TOOLS = PKG / "tools"
OBJ = PKG / "_obj"
LIB = PKG / "lib"
BIN = PKG / "bin"
INCLUDE = ROOT / "include"

CUDA_SOURCES = ["tk_api.cu", "tk_scan.cu", "tk_parse.cu", "tk_table.cu", "tk_cov.cu", "tk_r2t.cu", "tk_bins.cu", "tk_server.cu",
                "tk_fasta.cu", "tk_norm.cu", "tk_dbg.cu"]
TOOL_SOURCES = {
    "jellyfish": ["jellyfish.cpp"],
    "fastaToKmerCoverageStats": ["fastaToKmerCoverageStats.cpp"],
    "ReadsToTranscripts": ["ReadsToTranscripts.cpp"],
    "trinkmerd": ["trinkmerd.cpp"],
    "seqtk-trinity": ["seqtk_trinity.cpp"],
    "insilico_read_normalization": ["insilico_read_normalization.cpp"],
    "FastaToDeBruijn": ["FastaToDeBruijn.cpp"],
    "trinkmer_bins": ["trinkmer_bins.cpp"],
}

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "-Xcompiler", "-Wall",
              "--ptxas-options=-v"] if os.environ.get("TK_PTXAS_VERBOSE") else [
              "-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC"]


def _nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and Path(cand).exists():
            return cand
    raise RuntimeError("nvcc not found: the CUDA toolkit is required to build libtrinkmer_cuda.so")


def _run(cmd: list[str]) -> None:
    r = subprocess.run(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
    if r.returncode != 0:
        raise RuntimeError("build step failed:\n" + " ".join(cmd) + "\n" + r.stdout)
    if os.environ.get("TK_BUILD_VERBOSE") and r.stdout.strip():
        sys.stderr.write(r.stdout)


def _stale(out: Path, deps: list[Path]) -> bool:
    if not out.exists():
        return True
    t = out.stat().st_mtime
    return any(d.stat().st_mtime > t for d in deps if d.exists())


def build(force: bool = False, jobs: int | None = None) -> dict:
    """Compiles everything; returns the paths of the built artefacts."""
    nvcc = _nvcc()
    OBJ.mkdir(exist_ok=True)
    LIB.mkdir(exist_ok=True)
    BIN.mkdir(exist_ok=True)
    headers = list(CSRC.glob("*.cuh")) + [INCLUDE / "trinkmer.h"]
    jobs = jobs or max(2, min(len(CUDA_SOURCES) + 4, os.cpu_count() or 4))

    def cu_obj(src: str) -> Path:
        s = CSRC / src
        o = OBJ / (s.stem + ".o")
        if force or _stale(o, [s] + headers):
            _run([nvcc, *ARCH, *NVCC_FLAGS, "-I", str(INCLUDE), "-c", str(s), "-o", str(o)])
        return o

    synth_so = LIB / "libtrinkmer_synth.so"
    cuda_so = LIB / "libtrinkmer_cuda.so"

    def synth() -> Path:
        s = CSRC / "synth.c"
        if force or _stale(synth_so, [s]):
            _run(["gcc", "-O2", "-std=gnu11", "-fPIC", "-fopenmp", "-shared", "-o", str(synth_so), str(s), "-lm"])
        return synth_so

    with cf.ThreadPoolExecutor(jobs) as ex:
        fut_objs = [ex.submit(cu_obj, s) for s in CUDA_SOURCES]
        fut_synth = ex.submit(synth)
        objs = [f.result() for f in fut_objs]
        fut_synth.result()
        if force or _stale(cuda_so, objs):
            _run([nvcc, *ARCH, "-shared", "-o", str(cuda_so), *map(str, objs), "-lcudart"])

        def tool(name: str, srcs: list[str]) -> Path:
            out = BIN / name
            deps = [TOOLS / s for s in srcs] + list(TOOLS.glob("*.hpp")) + [INCLUDE / "trinkmer.h", cuda_so]
            if force or _stale(out, deps):
                _run(["g++", "-O2", "-std=c++17", "-pthread", "-I", str(INCLUDE), "-I", str(TOOLS),
                      *[str(TOOLS / s) for s in srcs], "-o", str(out),
                      "-L", str(LIB), "-ltrinkmer_cuda", "-Wl,-rpath,$ORIGIN/../lib"])
            return out

        tools = {n: ex.submit(tool, n, s) for n, s in TOOL_SOURCES.items() if all((TOOLS / x).exists() for x in s)}
        built_tools = {n: f.result() for n, f in tools.items()}
    return {"cuda": cuda_so, "synth": synth_so, "tools": built_tools}


if __name__ == "__main__":
    print(build(force="--force" in sys.argv))
