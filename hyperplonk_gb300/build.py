"""Builds libhp_cuda.so (all CUDA sources under csrc/) for sm_103a, in tree.

Each translation unit is compiled in parallel with nvcc into
hyperplonk_gb300/_build/, then linked into one shared library that exports the
C ABI declared in include/hp_cuda.h.  No CMake, no torch extension machinery:
the library is plain C ABI so any host language can bind it.
"""
from __future__ import annotations

import concurrent.futures
import os
import pathlib
import shutil
import subprocess

PKG = pathlib.Path(__file__).resolve().parent
ROOT = PKG.parent
CSRC = PKG / "csrc"
BUILD = PKG / "_build"
LIB = BUILD / "libhp_cuda.so"
PROBE_DIR = ROOT / "bench_probe"  # integer-pipe ceilings, read by bench.py (not part of the library)
PROBE_LIB = PROBE_DIR / "_build" / "libhp_probe.so"
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC", "-Xcompiler", "-O2",
              "--expt-relaxed-constexpr", f"-I{ROOT / 'include'}"]


# CUDA runtime entry points the library's own calls go through
# csrc/runtime_audit.cpp for (counting and host-side failure injection)
AUDITED = ["cudaMalloc", "cudaHostAlloc", "cudaMallocHost", "cudaMallocAsync", "cudaMallocFromPoolAsync",
           "cudaFree", "cudaFreeHost", "cudaFreeAsync", "cudaMemcpy", "cudaMemcpyAsync", "cudaMemset",
           "cudaMemsetAsync", "cudaStreamSynchronize", "cudaEventSynchronize", "cudaDeviceSynchronize"]
WRAP_FLAGS = [f"-Xlinker=--wrap={name}" for name in AUDITED]


def _nvcc() -> str:
    cand = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(cand):
        raise RuntimeError("nvcc not found: the CUDA toolkit is required to build libhp_cuda.so")
    return cand


def sources() -> list[pathlib.Path]:
    """CUDA translation units plus host-only C++ (the transcript)."""
    return sorted(CSRC.glob("*.cu")) + sorted(CSRC.glob("*.cpp"))


def _headers() -> list[pathlib.Path]:
    return (sorted(CSRC.glob("*.cuh")) + sorted(CSRC.glob("*.h")) + sorted(CSRC.glob("*.inc"))
            + sorted((ROOT / "include").glob("*.h")))


def _stale(obj: pathlib.Path, src: pathlib.Path, headers: list[pathlib.Path]) -> bool:
    if not obj.exists():
        return True
    t = obj.stat().st_mtime
    return src.stat().st_mtime > t or any(h.stat().st_mtime > t for h in headers)


def build(verbose: bool = False, extra_flags: list[str] | None = None) -> pathlib.Path:
    """Compile every csrc/*.cu and link libhp_cuda.so; returns the library path."""
    BUILD.mkdir(exist_ok=True)
    nvcc = _nvcc()
    headers = _headers()
    if extra_flags is None and os.environ.get("HP_EXTRA_NVCC_FLAGS"):
        # tuning hook: e.g. HP_EXTRA_NVCC_FLAGS="-DHP_FQ_INLINE" (a changed flag set rebuilds everything)
        extra_flags = os.environ["HP_EXTRA_NVCC_FLAGS"].split()
    flags = NVCC_FLAGS + (extra_flags or [])
    # objects built with other flags (a tuning build) are rebuilt: the flag
    # set of the last build is kept beside the objects
    stamp = BUILD / "flags.txt"
    flag_text = " ".join(ARCH + flags)
    flags_changed = not stamp.exists() or stamp.read_text() != flag_text
    jobs = []
    for src in sources():
        obj = BUILD / (src.stem + ".o")
        if _stale(obj, src, headers) or flags_changed:
            jobs.append([nvcc, *ARCH, *flags, "-c", str(src), "-o", str(obj)])

    def run(cmd):
        if verbose:
            print(" ".join(cmd), flush=True)
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"nvcc failed for {cmd[-3]}:\n{r.stdout}\n{r.stderr}")
        return r

    with concurrent.futures.ThreadPoolExecutor(max_workers=max(1, min(len(jobs), os.cpu_count() or 4))) as ex:
        list(ex.map(run, jobs))
    objs = [str(BUILD / (s.stem + ".o")) for s in sources()]
    if jobs or not LIB.exists():
        tmp = BUILD / "libhp_cuda.so.tmp"
        run([nvcc, *ARCH, "-shared", "-cudart", "static", "-o", str(tmp), *objs, *WRAP_FLAGS])
        os.replace(tmp, LIB)
    stamp.write_text(flag_text)
    probe_src = PROBE_DIR / "int_probe.cu"
    if probe_src.exists() and (not PROBE_LIB.exists() or _stale(PROBE_LIB, probe_src, headers)):
        PROBE_LIB.parent.mkdir(exist_ok=True)
        tmp = PROBE_LIB.parent / "libhp_probe.so.tmp"
        run([nvcc, *ARCH, *flags, f"-I{CSRC}", "-shared", "-cudart", "static", str(probe_src), "-o", str(tmp)])
        os.replace(tmp, PROBE_LIB)
    return LIB


if __name__ == "__main__":
    print(build(verbose=True))
