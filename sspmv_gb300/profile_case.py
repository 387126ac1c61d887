"""One format on one seeded synthetic family, a few SpMVs: the small, fixed
workload to run under a profiler (ncu) or to time one kernel alone.

    python -m sspmv_gb300.profile_case powerlaw_4M csr f64 [--kernel-flag F] [--param P] [--reps R]

The matrix is built exactly as `bench.py` builds it (same generator, seed,
converter parameters), x is the benchmark's vector, L2 is flushed before every
SpMV (--flush write: a 256 MiB write; write+read: that write, then a 256 MiB
read of another buffer, so L2 holds clean lines and the SpMV pays no
write-back of the flush; none).  After `reps` untimed SpMVs it times five more
with CUDA events and prints the best time, the algorithmic GB/s and the bytes.
"""
from __future__ import annotations

import argparse


def main(argv=None) -> None:
    import numpy as np
    import torch

    from . import lespmv as L
    from . import synth

    ap = argparse.ArgumentParser(prog="python -m sspmv_gb300.profile_case")
    ap.add_argument("family", help="banded_2M, powerlaw_4M, block4_2M, uniform_4M, ...")
    ap.add_argument("format", choices=L.FORMATS)
    ap.add_argument("dtype", choices=["f64", "f32"])
    ap.add_argument("--kernel-flag", type=int, default=-1, help="sspmv_set_kernel flag (-1: library default)")
    ap.add_argument("--param", type=int, default=0, help="sspmv_set_kernel param")
    ap.add_argument("--reps", type=int, default=3, help="untimed SpMVs before the timed ones")
    ap.add_argument("--flush", default="write", choices=["write", "write+read", "none"])
    a = ap.parse_args(argv)
    dtype = np.float64 if a.dtype == "f64" else np.float32
    A = synth.generate(synth.WORKLOADS[a.family](), seed=1, dtype=np.float64)
    if dtype == np.float32:
        A = A.astype(np.float32)
    csr = L.csr_from_host(A)
    M, why = L.build_format(csr, a.format, A)
    if M is None:
        raise SystemExit(f"{a.family}/{a.format}/{a.dtype}: {why}")
    if a.kernel_flag >= 0:
        M.set_kernel(a.kernel_flag, a.param)
    x = torch.from_numpy(synth.vector(A.num_cols, 0, dtype)).cuda()
    y = torch.zeros(A.num_rows, dtype=x.dtype, device="cuda")
    buf = torch.empty(64 << 20, dtype=torch.float32, device="cuda")
    clean = torch.ones(64 << 20, dtype=torch.float32, device="cuda") if a.flush == "write+read" else None

    def flush():
        if a.flush == "none":
            return
        buf.zero_()
        if clean is not None:
            clean.sum()

    for _ in range(a.reps):
        flush()
        L.LeSpMV(1.0, M, x, 0.0, y)
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    ts = []
    for _ in range(5):
        flush()
        e0.record()
        L.LeSpMV(1.0, M, x, 0.0, y)
        e1.record()
        e1.synchronize()
        ts.append(e0.elapsed_time(e1))
    b = M.algorithmic_bytes(1, False)
    print(a.family, a.format, a.dtype, "ms", min(ts), "GB/s", b / min(ts) / 1e6, "bytes", b)


if __name__ == "__main__":
    main()
