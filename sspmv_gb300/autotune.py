"""Measured kernel selection (the library's autotuner).

The reference fixes its tuning parameters at compile time (SELL C and sigma,
BSR block size: include/general_config.h:17-26).  Here each candidate is run
on the GPU, timed with CUDA events with L2 flushed before every run, and the
fastest is kept.  Results are plain dicts, so a caller can store them as an
append-only JSONL log keyed by matrix and re-apply them without re-measuring.

CSR candidates: stream kernel (default), merge-path kernel, vector kernel with
1..32 lanes per row, row-block kernel (short rows) with windows of 512..4096
nonzeros, pipelined row kernel (short rows) with 1..8 lanes per row, either
value-load point and CTAs of 256 or 1024 threads.
S-ELL / SELL-c-sigma / SELL-c-R: after the layout, the thread-pass cap (the
cost model's choice against caps of 16..128 slots).
SELL-c-sigma candidates (re-conversion per point): C in {8,16,32} x sigma in
{256, 4096, N}.  BSR candidates: r x c in {2,4,8,16}^2 (feasible ones).
"""
from __future__ import annotations

import json
from pathlib import Path

from . import lespmv as L

L2_FLUSH = 256 << 20


class L2Flush:
    """Evicts the 129 MB L2 between timed SpMVs: a 256 MiB write, then a
    256 MiB read.  The read pass leaves only clean lines, so the timed kernel
    does not pay for writing the flush's dirty lines back to HBM (about 5 us
    on an 84 MB matrix, a quarter of its SpMV).  Call it on the stream the
    timed kernel runs on (the current stream)."""

    def __init__(self, device):
        import torch
        self.w = torch.empty(L2_FLUSH // 4, dtype=torch.float32, device=device)
        self.r = torch.zeros(L2_FLUSH // 4, dtype=torch.float32, device=device)
        self.acc = torch.zeros((), dtype=torch.float32, device=device)

    def __call__(self):
        import torch
        self.w.zero_()
        torch.sum(self.r, dim=0, out=self.acc)


# Longest dithering delay before a timed launch, in GPU clock cycles: a
# little more than one 2.048 us step of the event timer at 2.07 GHz.
DITHER_CYCLES = 4608


def time_spmv(M, x, y, reps: int = 10, warmup: int = 2, flush=None, stream=None) -> float:
    """Milliseconds of one SpMV (alpha=1, beta=0) with L2 flushed: the mean
    of the middle half of the sorted samples.  CUDA event times come in
    steps of 2.048 us on this GPU, and a launch that always follows the same
    flush starts at the same phase of a step, so every sample can land on the
    same step, up to one step off the true time.  A spin of a random length
    (0 to one step) between the flush and the start event spreads the phase:
    the samples then fall on the two steps around the true time in
    proportion, and their mean converges to it."""
    import random
    import torch
    stream = stream or torch.cuda.current_stream()
    if flush is None:
        flush = L2Flush(x.device)
    sleep = getattr(torch.cuda, "_sleep", None)
    rng = random.Random(7)
    ts = []
    for i in range(warmup + reps):
        flush()
        if sleep is not None:
            with torch.cuda.stream(stream):
                sleep(rng.randrange(DITHER_CYCLES))
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        L.LeSpMV(1.0, M, x, 0.0, y, stream)
        e1.record(stream)
        e1.synchronize()
        if i >= warmup:
            ts.append(e0.elapsed_time(e1))
    ts.sort()
    q = len(ts) // 4
    mid = ts[q:len(ts) - q] or ts
    return sum(mid) / len(mid)


CSR_CANDIDATES = ([(0, 0), (2, 0)] + [(1, vs) for vs in (1, 2, 4, 8, 16, 32)] +
                  [(3, w) for w in (512, 1024, 2048, 4096)] + [(4, p) for p in range(16)])


def tune_kernel(M, x, y, candidates, reps: int = 10) -> dict:
    """Times each (kernel_flag, param) on matrix M, applies the fastest."""
    flush = L2Flush(x.device)
    table = []
    for flag, param in candidates:
        M.set_kernel(flag, param)
        table.append({"kernel_flag": flag, "param": param, "ms": time_spmv(M, x, y, reps, flush=flush)})
    best = min(table, key=lambda r: r["ms"])
    M.set_kernel(best["kernel_flag"], best["param"])
    return {"format": M.fmt, "best": best, "table": table, "bytes": M.algorithmic_bytes()}


def tune_csr(M, x, y, reps: int = 10) -> dict:
    return tune_kernel(M, x, y, CSR_CANDIDATES, reps)


# Sliced formats: the thread-pass cap (param; 0 = the library's cost model).
SLICED_CAPS = [(0, 0), (0, 16), (0, 32), (0, 64), (0, 128)]

# Kernel candidates per format (formats with one kernel are not listed).
KERNEL_CANDIDATES = {"csr": CSR_CANDIDATES, "coo": [(0, 0), (1, 0)], "sell": SLICED_CAPS,
                     "sell_c_sigma": SLICED_CAPS, "sell_c_R": SLICED_CAPS,
                     "bsr": [(0, 0), (1, 0), (2, 0)],  # BSR: default choice, thread-per-row, block-stream
                     "dia": [(0, 0), (1, 0)]}  # DIA: thread per row, x windows staged by bulk copies


def conversion_candidates(fmt: str, num_rows: int) -> list[dict]:
    """Converter parameters tried per format (the reference's defaults first)."""
    if fmt == "sell":
        return [dict(chunkwidth=c, alignment=a) for c in (4, 8, 16, 32) for a in (0, 1)]
    if fmt == "sell_c_sigma":
        sig_n = max(32, -(-num_rows // 32) * 32)  # sigma = N, a multiple of every C tried
        out = [dict(slicewidth=0, chunkwidth=0, alignment=0)]
        out += [dict(slicewidth=s, chunkwidth=c, alignment=a) for c in (8, 16, 32) for s in (256, 4096, sig_n)
                for a in (0, 1)]
        return out
    if fmt == "sell_c_R":
        return [dict(chunkwidth=c, alignment=a) for c in (4, 8, 16, 32) for a in (0, 1)]
    if fmt == "csr5":
        return [dict(sigma=0, omega=0), dict(sigma=16, omega=32), dict(sigma=32, omega=32), dict(sigma=8, omega=32),
                dict(sigma=16, omega=16)]
    if fmt == "bsr":
        return [dict(blockDimRow=r, blockDimCol=c) for r, c in ((2, 2), (4, 4), (8, 8), (2, 4), (4, 2), (4, 8),
                                                                (8, 4), (1, 4), (4, 1))]
    return []


def tune_conversion(csr, fmt: str, x, y, reps: int = 8, max_fill: float = 4.0):
    """Converts `csr` with each candidate parameter set of `fmt`, times one
    SpMV of each and keeps the fastest.  Returns (matrix, record) or
    (None, None) when no candidate converts."""
    flush = L2Flush(x.device)
    best, table = None, []
    for kw in conversion_candidates(fmt, csr.num_rows):
        if fmt == "bsr":
            nnzb = L.count_blocks(csr, kw["blockDimRow"], kw["blockDimCol"])
            if nnzb * kw["blockDimRow"] * kw["blockDimCol"] > max_fill * max(csr.num_nnzs, 1):
                continue
        try:
            M = getattr(L, f"csr_to_{fmt}")(csr, **kw)
        except L.SSPMVError:
            continue
        ms = time_spmv(M, x, y, reps, flush=flush)
        table.append({"params": kw, "ms": ms})
        if best is None or ms < best[1]:
            if best is not None:
                best[0].delete()
            best = (M, ms, kw)
        else:
            M.delete()
    if best is None:
        return None, None
    M, ms, kw = best
    rec = {"format": fmt, "params": kw, "ms": ms, "table": table}
    if fmt in KERNEL_CANDIDATES:  # then the kernel for the chosen layout
        k = tune_kernel(M, x, y, KERNEL_CANDIDATES[fmt], reps)
        rec["kernel"] = k["best"]
        rec["ms"] = min(ms, k["best"]["ms"])
    return M, rec


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


def kernel_table(families, dtypes=("f64", "f32"), ks=(1, 2, 4, 8), flags=((0, 0), (2, 0), (1, 0)), reps: int = 5,
                 log=None) -> list[dict]:
    """Times the CSR kernels (stream, merge-path, vector) on the named
    synthetic workloads for k right-hand sides; one record per (workload,
    precision, k, kernel): median ms (L2 flushed), algorithmic GB/s."""
    import numpy as np
    import torch
    from . import synth
    flush = L2Flush("cuda")
    out = []
    for fam in families:
        for dt in dtypes:
            dtype = np.float64 if dt == "f64" else np.float32
            A = synth.load(fam, 1, dtype)
            csr = L.csr_from_host(A)
            for k in ks:
                X = torch.from_numpy(synth.vector(A.num_cols, 0, dtype, k).reshape(A.num_cols, k)).cuda()
                Y = torch.zeros((A.num_rows, k), dtype=X.dtype, device="cuda")
                for flag, param in flags:
                    csr.set_kernel(flag, param)
                    ts = []
                    for i in range(reps + 1):
                        flush()
                        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
                        e0.record()
                        L.spmm(1.0, csr, X, 0.0, Y)
                        e1.record()
                        e1.synchronize()
                        if i:
                            ts.append(e0.elapsed_time(e1))
                    ms = sorted(ts)[len(ts) // 2]
                    rec = {"workload": fam, "dtype": dt, "k": k, "kernel_flag": flag, "param": param,
                           "ms": round(ms, 4), "GBps": round(csr.algorithmic_bytes(k, False) / ms / 1e6, 1)}
                    out.append(rec)
                    if log:
                        log(json.dumps(rec))
            csr.delete()
    return out


def main(argv=None) -> None:
    """python -m sspmv_gb300.autotune table --families powerlaw_4M,uniform_4M [--ks 1,2,4,8]"""
    import argparse
    import sys
    ap = argparse.ArgumentParser(prog="python -m sspmv_gb300.autotune")
    sub = ap.add_subparsers(dest="cmd", required=True)
    t = sub.add_parser("table", help="CSR kernels x k right-hand sides on synthetic workloads")
    t.add_argument("--families", default="powerlaw_4M,uniform_4M,banded_2M,block4_2M")
    t.add_argument("--dtypes", default="f64,f32")
    t.add_argument("--ks", default="1,2,4,8")
    a = ap.parse_args(argv)
    kernel_table(a.families.split(","), a.dtypes.split(","), [int(k) for k in a.ks.split(",")],
                 log=lambda s: print(s, flush=True))
    sys.stdout.flush()


if __name__ == "__main__":
    main()
