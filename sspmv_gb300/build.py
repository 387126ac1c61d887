"""In-tree build of libsspmv.so (sm_103a) and of the CPU oracle.

`build_library()` compiles every source under sspmv_gb300/csrc with nvcc for
sm_103a only (one -gencode), in parallel, into sspmv_gb300/_build/, and links
sspmv_gb300/lib/libsspmv.so.  Objects are rebuilt when a source or header is
newer than the object.
"""
from __future__ import annotations

import os
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor
from pathlib import Path

PKG = Path(__file__).resolve().parent
ROOT = PKG.parent
CSRC = PKG / "csrc"
BUILD = PKG / "_build"
LIBDIR = PKG / "lib"
LIB = LIBDIR / "libsspmv.so"
NVCC = os.environ.get("NVCC", "/usr/local/cuda/bin/nvcc")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
COMMON = ["-O3", "-std=c++17", "-lineinfo", f"-I{ROOT / 'include'}", f"-I{CSRC}",
          "-Xcompiler", "-fPIC,-fopenmp,-Wall,-Wno-unused-function"]


def _sources():
    return sorted([p for p in CSRC.iterdir() if p.suffix in (".cu", ".cpp")])


def _headers():
    hs = [p for p in CSRC.iterdir() if p.suffix in (".cuh", ".h", ".inc")]
    hs += list((ROOT / "include").glob("*.h"))
    return hs


def _stale(obj: Path, src: Path, newest_header: float) -> bool:
    if not obj.exists():
        return True
    t = obj.stat().st_mtime
    return src.stat().st_mtime > t or newest_header > t


def _compile(src: Path, extra: list[str]) -> tuple[Path, str]:
    obj = BUILD / (src.name + ".o")
    cmd = [NVCC, *ARCH, *COMMON, *extra, "-c", str(src), "-o", str(obj)]
    if src.suffix == ".cpp":
        cmd = [NVCC, *COMMON, *extra, "-x", "c++", "-c", str(src), "-o", str(obj)]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"compile failed: {' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
    return obj, r.stderr


def build_library(verbose: bool = False, extra: list[str] | None = None, jobs: int | None = None) -> Path:
    extra = list(extra or [])
    BUILD.mkdir(exist_ok=True)
    LIBDIR.mkdir(exist_ok=True)
    srcs = _sources()
    newest = max((h.stat().st_mtime for h in _headers()), default=0.0)
    todo = [s for s in srcs if _stale(BUILD / (s.name + ".o"), s, newest)]
    jobs = jobs or min(len(todo) or 1, os.cpu_count() or 4)
    with ThreadPoolExecutor(max_workers=jobs) as ex:
        for obj, err in ex.map(lambda s: _compile(s, extra), todo):
            if verbose:
                print(f"[sspmv] built {obj.name}", file=sys.stderr)
                if err.strip():
                    print(err, file=sys.stderr)
    objs = [BUILD / (s.name + ".o") for s in srcs]
    if todo or not LIB.exists() or any(o.stat().st_mtime > LIB.stat().st_mtime for o in objs):
        cmd = [NVCC, *ARCH, "-shared", "-o", str(LIB), *map(str, objs), "-Xcompiler", "-fopenmp", "-lgomp"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"link failed: {' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
    return LIB


SYNTH_LIB = LIBDIR / "libsspmv_synth.so"
PROBE_SRC = CSRC / "probe" / "calibrate.cu"
PROBE_LIB = LIBDIR / "libsspmv_probe.so"


def build_probe() -> Path:
    """lib/libsspmv_probe.so: the benchmark's measurement probes (random
    gather rate, FP64 FMA rate), linked against libsspmv.so; not part of the
    library's C ABI."""
    obj = BUILD / "calibrate.cu.o"
    newest = max([PROBE_SRC.stat().st_mtime] + [h.stat().st_mtime for h in _headers()])
    if not PROBE_LIB.exists() or PROBE_LIB.stat().st_mtime < max(newest, LIB.stat().st_mtime):
        BUILD.mkdir(exist_ok=True)
        _compile(PROBE_SRC, [])
        cmd = [NVCC, *ARCH, "-shared", "-o", str(PROBE_LIB), str(obj), f"-L{LIBDIR}", "-lsspmv",
               "-Xlinker", "-rpath=$ORIGIN"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"probe link failed: {' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
    return PROBE_LIB


def build_synth() -> Path:
    """lib/libsspmv_synth.so: the seeded matrix generator (csrc/synth.cpp)
    alone, host code only, so CPU-only callers need not load libsspmv.so."""
    LIBDIR.mkdir(exist_ok=True)
    src = CSRC / "synth.cpp"
    hdr = ROOT / "include" / "sspmv.h"
    if SYNTH_LIB.exists() and SYNTH_LIB.stat().st_mtime >= max(src.stat().st_mtime, hdr.stat().st_mtime):
        return SYNTH_LIB
    cxx = os.environ.get("CXX", "g++")
    cmd = [cxx, "-O3", "-std=c++17", "-fPIC", "-fopenmp", "-shared", f"-I{ROOT / 'include'}", str(src),
           "-o", str(SYNTH_LIB)]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"synth build failed: {' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
    return SYNTH_LIB


CLI_SRC = PKG / "cli" / "benchmark_spmv.cpp"
BINDIR = PKG / "bin"
CLI_FORMATS = ("csr", "coo", "ell", "sell", "sell_c_sigma", "sell_c_R", "dia", "bsr", "csr5")


def build_cli() -> Path:
    """sspmv_gb300/bin/benchmark_spmv (links libsspmv.so by rpath) and the
    benchmark_spmv_<fmt> names the reference's programs have."""
    BINDIR.mkdir(exist_ok=True)
    exe = BINDIR / "benchmark_spmv"
    if not exe.exists() or exe.stat().st_mtime < max(CLI_SRC.stat().st_mtime, LIB.stat().st_mtime):
        cmd = [NVCC, "-O2", "-std=c++17", f"-I{ROOT / 'include'}", "-x", "c++", str(CLI_SRC), "-o", str(exe),
               f"-L{LIBDIR}", "-lsspmv", "-lcudart", "-Xlinker", "-rpath=$ORIGIN/../lib"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"cli build failed: {' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
    for f in CLI_FORMATS:
        link = BINDIR / f"benchmark_spmv_{f}"
        if not link.is_symlink():
            if link.exists():
                link.unlink()
            link.symlink_to("benchmark_spmv")
    return exe


def build_oracle(ref_root: str | None = None) -> None:
    """CPU oracle (test infrastructure): oracle/liboracle.so, plus the
    reference harness oracle/_ref/libref.so when ref_root (default: the
    SSPMV_REF_ROOT environment variable) names a checkout of the reference
    sources."""
    od = ROOT / "oracle"
    subprocess.run(["make", "-s", "-C", str(od)], check=True)
    ref_root = ref_root or os.environ.get("SSPMV_REF_ROOT")
    if ref_root and Path(ref_root, "LeSpMV", "include").is_dir():
        subprocess.run(["make", "-s", "-C", str(od), "ref", f"REF_ROOT={ref_root}"], check=True)


if __name__ == "__main__":
    print(build_library(verbose=True))
    print(build_synth())
    print(build_probe())
    print(build_cli())
    build_oracle()
