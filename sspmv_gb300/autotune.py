"""Measured kernel selection (the library's autotuner).

The reference fixes its tuning parameters at compile time (SELL C and sigma,
BSR block size: include/general_config.h:17-26).  Here each candidate is run
on the GPU, timed with CUDA events with L2 flushed before every run, and the
fastest is kept.  Results are plain dicts, so a caller can store them as an
append-only JSONL log keyed by matrix and re-apply them without re-measuring.

CSR candidates: merge-path kernel, vector kernel with 2..32 lanes per row.
SELL-c-sigma candidates (re-conversion per point): C in {8,16,32} x sigma in
{256, 4096, N}.  BSR candidates: r x c in {2,4,8,16}^2 (feasible ones).
"""
from __future__ import annotations

import json
from pathlib import Path

from . import lespmv as L

L2_FLUSH = 256 << 20


def time_spmv(M, x, y, reps: int = 10, warmup: int = 2, flush=None, stream=None) -> float:
    """Median milliseconds of one SpMV (alpha=1, beta=0) with L2 flushed."""
    import torch
    stream = stream or torch.cuda.current_stream()
    if flush is None:
        flush = torch.empty(L2_FLUSH // 4, dtype=torch.float32, device=x.device)
    ts = []
    for i in range(warmup + reps):
        flush.zero_()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        L.LeSpMV(1.0, M, x, 0.0, y, stream)
        e1.record(stream)
        e1.synchronize()
        if i >= warmup:
            ts.append(e0.elapsed_time(e1))
    ts.sort()
    return ts[len(ts) // 2]


CSR_CANDIDATES = [(0, 0)] + [(1, vs) for vs in (2, 4, 8, 16, 32)]


def tune_kernel(M, x, y, candidates, reps: int = 10) -> dict:
    """Times each (kernel_flag, param) on matrix M, applies the fastest."""
    import torch
    flush = torch.empty(L2_FLUSH // 4, dtype=torch.float32, device=x.device)
    table = []
    for flag, param in candidates:
        M.set_kernel(flag, param)
        table.append({"kernel_flag": flag, "param": param, "ms": time_spmv(M, x, y, reps, flush=flush)})
    best = min(table, key=lambda r: r["ms"])
    M.set_kernel(best["kernel_flag"], best["param"])
    return {"format": M.fmt, "best": best, "table": table, "bytes": M.algorithmic_bytes()}


def tune_csr(M, x, y, reps: int = 10) -> dict:
    return tune_kernel(M, x, y, CSR_CANDIDATES, reps)


# Kernel candidates per format (formats with one kernel are not listed).
KERNEL_CANDIDATES = {"csr": CSR_CANDIDATES}


def tune_format(M, x, y, reps: int = 10) -> dict | None:
    cands = KERNEL_CANDIDATES.get(M.fmt)
    if not cands:
        return None
    return tune_kernel(M, x, y, cands, reps)


def append_log(path: str | Path, key: str, result: dict) -> None:
    """Append-only JSONL record (restart skips keys already present)."""
    with open(path, "a") as f:
        f.write(json.dumps({"key": key, **result}) + "\n")


def load_log(path: str | Path) -> dict:
    out = {}
    p = Path(path)
    if p.exists():
        for line in p.read_text().splitlines():
            if line.strip():
                rec = json.loads(line)
                out[rec["key"]] = rec
    return out
