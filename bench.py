#!/usr/bin/env python
"""SpMV benchmark: every format on the four seeded synthetic families, FP64
and FP32, one GB300.

A step is one SpMV (y = A*x, alpha=1, beta=0) of every feasible
(family, format, precision) matrix of the workload:
    families  banded_2M, powerlaw_4M, block4_2M, uniform_4M
    formats   the library's formats (infeasible pairs are skipped and listed:
              DIA over 10240 diagonals, ELL/BSR whose padded size exceeds 4x
              the CSR size)
    precision f64, f32
value = sum of algorithmic bytes / sum of kernel time (GB/s), device-resident
inputs, L2 flushed before every SpMV (a 256 MiB write, then a 256 MiB read so
that no dirty line of the flush is left for the SpMV to write back) and the
flush excluded from the timing.  e2e = the same through the C ABI with pinned
host x copied in and y copied out of every SpMV inside the timed region, the
copies on their own streams overlapping the other matrices' SpMVs
(serial_value: copies and SpMV back to back on one stream).

The last line on stdout is the compact result (one JSON object of a few KB);
everything else -- per-format table, sweep points, tuning tables -- goes to
the detail file (--detail, default gpurun_out/bench_detail.json) and to
stderr.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl sspmv|reference]
"""
from __future__ import annotations

import argparse
import json
import os
import random
import statistics
import subprocess
import sys
import tempfile
import threading
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

FAMILIES = ["banded_2M", "powerlaw_4M", "block4_2M", "uniform_4M"]
DTYPES = ["f64", "f32"]
L2_FLUSH_BYTES = 256 << 20
RANDOM_COLUMN_FAMILIES = ("uniform_4M", "powerlaw_4M")


def parse_args(argv=None):
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="sspmv", choices=["sspmv", "reference"])
    ap.add_argument("--families", default=",".join(FAMILIES))
    ap.add_argument("--formats", default="all")
    ap.add_argument("--dtypes", default=",".join(DTYPES))
    ap.add_argument("--scale", type=float, default=1.0, help="row-count scale (testing only)")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-tune", action="store_true", help="skip the autotuner (library defaults)")
    ap.add_argument("--csr-kernel", default="", help="pin the CSR kernel as FLAG:PARAM (implies no tuning of CSR)")
    ap.add_argument("--kernel", action="append", default=[],
                    help="pin a format's kernel as FMT:FLAG:PARAM (repeatable; that format is not tuned)")
    ap.add_argument("--no-cpu", action="store_true", help="skip the CPU baseline (profiling runs)")
    ap.add_argument("--no-large", action="store_true", help="skip the Laplacian and the power-law 16M SELL-c-sigma vs CSR sections")
    ap.add_argument("--no-serving", action="store_true", help="skip the request-server section")
    ap.add_argument("--sections", default="suite,laplacian,large,serving",
                    help="sections to run: suite (the timed line), laplacian (1024^2 from .mtx), large "
                         "(power-law 16M), serving; e.g. --sections laplacian for a profiling run")
    ap.add_argument("--detail", default=str(ROOT / "gpurun_out" / "bench_detail.json"),
                    help="file for the full result (per-format table, sweeps); '' to skip")
    return ap.parse_args(argv)


def sections(args) -> set[str]:
    """The sections a run includes (--sections, less the --no-* ones)."""
    out = {x for x in args.sections.split(",") if x}
    if args.no_large:
        out -= {"laplacian", "large"}
    if args.no_serving:
        out.discard("serving")
    return out


_T0 = time.perf_counter()


def log(msg: str) -> None:
    """Progress line on stderr (stdout carries only the JSON result)."""
    print(f"[bench {time.perf_counter() - _T0:7.1f}s] {msg}", file=sys.stderr, flush=True)


def np_dtype(tag):
    return np.float64 if tag == "f64" else np.float32


L2_NOTE = ("flushed before every SpMV (256 MiB write, then 256 MiB read: no dirty flush lines left), "
           "flush not timed")


def scaled_params(name, scale):
    from sspmv_gb300 import synth
    p = synth.WORKLOADS[name]()
    if scale != 1.0:
        if p.family == synth.LAPLACIAN2D:
            p.grid = max(8, int(p.grid * scale ** 0.5))
        else:
            p.num_rows = max(4096, int(p.num_rows * scale))
            if p.family == synth.BLOCK:
                p.num_blocks = max(16, int(p.num_blocks * scale))
    return p


def host_matrices(families, scale):
    from sspmv_gb300 import synth
    mats = {}
    for fam in families:
        A = synth.generate(scaled_params(fam, scale), seed=1, dtype=np.float64)
        mats[(fam, "f64")] = A
        mats[(fam, "f32")] = A.astype(np.float32)
    return mats


# ------------------------------------------------------------------ clocks --
class ClockSampler:
    QUERY = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index=0):
        self.index = index
        self.proc = None
        self.file = None

    def start(self):
        try:
            self.file = tempfile.NamedTemporaryFile("w+", suffix=".csv", delete=False)
            self.proc = subprocess.Popen(["nvidia-smi", f"--id={self.index}", f"--query-gpu={self.QUERY}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=self.file, stderr=subprocess.DEVNULL)
        except (OSError, FileNotFoundError):
            self.proc = None

    def stop(self):
        if not self.proc:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        time.sleep(0.25)
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        self.file.flush()
        rows = [ln.split(",") for ln in Path(self.file.name).read_text().splitlines() if ln.count(",") >= 8]
        os.unlink(self.file.name)
        sm = [float(r[1]) for r in rows if r[1].strip().replace(".", "").isdigit()]
        mx = [float(r[2]) for r in rows if r[2].strip().replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for r in rows for i in range(4) if "Active" in r[5 + i] and "Not" not in r[5 + i]})
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": reasons, "samples": len(rows)}


# ------------------------------------------------------------ probes ------
class Probes:
    """The benchmark's measurement probes (sspmv_gb300/csrc/probe/calibrate.cu,
    lib/libsspmv_probe.so): the random-gather rate and the FP64 FMA rate of
    the device, the ceilings that bound SpMV on random-column matrices and
    FP64 SpMV where HBM bytes do not."""

    def __init__(self):
        import ctypes as C
        from sspmv_gb300 import _lib  # loads libsspmv.so, which the probe library links
        self.C = C
        self.call = _lib.call
        path = ROOT / "sspmv_gb300" / "lib" / "libsspmv_probe.so"
        if not path.exists():
            raise ImportError(f"{path} is not built; run __graft_entry__.build()")
        h = C.CDLL(str(path))
        h.sspmv_gather_ceiling.restype = C.c_int
        h.sspmv_gather_ceiling.argtypes = [C.c_int32, C.c_int64, C.c_int64, C.POINTER(C.c_double),
                                           C.POINTER(C.c_double), C.c_void_p]
        h.sspmv_fp64_ceiling.restype = C.c_int
        h.sspmv_fp64_ceiling.argtypes = [C.POINTER(C.c_double), C.c_void_p]
        h.sspmv_stream_ceiling.restype = C.c_int
        h.sspmv_stream_ceiling.argtypes = [C.c_int64, C.c_int64, C.POINTER(C.c_double), C.c_void_p]
        self.h = h

    def _check(self, st, what):
        from sspmv_gb300 import _lib
        _lib.check(st, what)

    def gather_ceiling(self, dtype, num_cols, num_gathers):
        """(gathers per second, checksum) of random gathers from a vector of
        num_cols values, num_gathers indices streamed once."""
        C = self.C
        rate, chk = C.c_double(0.0), C.c_double(0.0)
        vt = 1 if np.dtype(dtype) == np.float64 else 0
        self._check(self.h.sspmv_gather_ceiling(vt, int(num_cols), int(num_gathers), C.byref(rate), C.byref(chk),
                                                None), "sspmv_gather_ceiling")
        return rate.value, chk.value

    def stream_ceiling_ms(self, read_bytes, write_bytes):
        """Median ms of a plain stream reading read_bytes and writing
        write_bytes, L2 flushed as the benchmark flushes: the cold time of a
        kernel that only had to move those bytes."""
        C = self.C
        ms = C.c_double(0.0)
        self._check(self.h.sspmv_stream_ceiling(int(read_bytes), int(write_bytes), C.byref(ms), None),
                    "sspmv_stream_ceiling")
        return ms.value

    def fp64_ceiling(self):
        """FP64 FMAs per second (independent chains)."""
        C = self.C
        rate = C.c_double(0.0)
        self._check(self.h.sspmv_fp64_ceiling(C.byref(rate), None), "sspmv_fp64_ceiling")
        return rate.value


def measured_peak():
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        d = json.loads(p.read_text())
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


def traffic_table():
    """Per-launch DRAM bytes of the kernels measured with ncu (profiles/traffic.json)."""
    p = ROOT / "profiles" / "traffic.json"
    return json.loads(p.read_text()) if p.exists() else {}


# ---------------------------------------------------------------- GPU arm --
def run_gpu(args, rank, world):
    """The GPU arm: the timed suite (the result line's value), then the
    Laplacian, large power-law and serving sections (rank 0)."""
    import torch
    secs = sections(args)
    dev = torch.device("cuda", rank % max(1, torch.cuda.device_count()))
    torch.cuda.set_device(dev)
    peak, _ = measured_peak()
    families = [f for f in args.families.split(",") if f]
    dtypes = [d for d in args.dtypes.split(",") if d]
    if "suite" in secs:
        out = run_suite(args, dev, rank, world)
    else:
        out = {"metric": SUITE_METRIC, "value": None, "unit": "GB/s", "n_gpus": world, "steps": args.steps,
               "warmup": args.warmup, "ms_per_step": None, "higher_is_better": True, "scaling": "weak",
               "vs_baseline": None, "dtype": "f64+f32", "data": "synthetic", "config": {"sections": sorted(secs)}}
    lap = large = serving = None
    full = args.scale == 1.0
    if rank == 0 and "laplacian" in secs and full:
        lap = run_laplacian(dev, peak, tuple(int(v) for v in args.csr_kernel.split(":")) if args.csr_kernel else None)
        log("laplacian done")
    if rank == 0 and "large" in secs and full:
        large = run_large(dev, peak)
        log("large done")
    if rank == 0 and "serving" in secs and full:
        serving = run_serving()
        log("serving done")
    out.update({"laplacian_1024": lap, "large_powerlaw_16M": large, "serving": serving})
    del families, dtypes
    return out


SUITE_METRIC = "SpMV GB/s (algorithmic bytes / kernel time), all formats x 4 families x {f64,f32}"


def run_suite(args, dev, rank, world):
    """Every feasible (family, format, precision) of the suite, autotuned,
    one SpMV each per step, timed with CUDA events; parity, e2e, roofline,
    CPU baseline."""
    import torch
    from sspmv_gb300 import _lib
    from sspmv_gb300 import lespmv as L

    families = [f for f in args.families.split(",") if f]
    dtypes = [d for d in args.dtypes.split(",") if d]
    fmts = L.FORMATS if args.formats == "all" else args.formats.split(",")
    hosts = host_matrices(families, args.scale)
    log("host matrices generated")

    cases, skipped = [], []
    for fam in families:
        for dt in dtypes:
            A = hosts[(fam, dt)]
            csr = L.csr_from_host(A)
            for fmt in fmts:
                t_conv = time.perf_counter()
                M, why = L.build_format(csr, fmt, A)
                log(f"convert {fam}/{fmt}/{dt}: {'skipped' if M is None else 'ok'} "
                    f"({time.perf_counter() - t_conv:.2f}s)")
                if M is None:
                    skipped.append(f"{fam}/{fmt}/{dt}: {why}")
                    continue
                x = torch.from_numpy(_x_host(A.num_cols, dt)).to(dev)
                y = torch.zeros(A.num_rows, dtype=x.dtype, device=dev)
                cases.append({"fam": fam, "fmt": fmt, "dt": dt, "M": M, "x": x, "y": y,
                              "bytes": M.algorithmic_bytes(1, False), "csr": csr, "nnz": A.nnz,
                              "rows": A.num_rows, "cols": A.num_cols})
    from sspmv_gb300.autotune import DITHER_CYCLES, L2Flush
    flush = L2Flush(dev)
    stream = torch.cuda.current_stream()
    pinned = {}
    if args.csr_kernel:
        pinned["csr"] = tuple(int(v) for v in args.csr_kernel.split(":"))
    for spec in args.kernel:
        fmt, flag, param = spec.split(":")
        pinned[fmt] = (int(flag), int(param))
    for c in cases:
        if c["fmt"] in pinned:
            c["M"].set_kernel(*pinned[c["fmt"]])
    if not args.no_tune:
        from sspmv_gb300 import autotune
        seen = set()
        for c in cases:
            if id(c["M"]) in seen or c["fmt"] in pinned:
                continue
            seen.add(id(c["M"]))
            if c["fmt"] in ("sell", "sell_c_sigma", "sell_c_R", "csr5", "bsr"):
                M2, rec = autotune.tune_conversion(c["csr"], c["fmt"], c["x"], c["y"])
                if M2 is not None:
                    if c["M"] is not c["csr"]:
                        c["M"].delete()
                    c["M"] = M2
                    c["bytes"] = M2.algorithmic_bytes(1, False)
                    c["tuned"] = {"params": rec["params"], "ms": rec["ms"]}
                    if rec.get("kernel"):
                        c["tuned"]["kernel"] = {k: rec["kernel"][k] for k in ("kernel_flag", "param")}
                log(f"tuned {c['fam']}/{c['fmt']}/{c['dt']}: {c.get('tuned')}")
                continue
            res = autotune.tune_format(c["M"], c["x"], c["y"])
            c["tuned"] = res["best"] if res else None
    for c in cases:
        c.setdefault("tuned", None)
        c["kernel"] = {"kernel_flag": c["M"].kernel_flag}
        # secondary byte counts: the reference benchmark's bytes_per_spmv and
        # the CSR algorithmic bytes of the same matrix (format-independent)
        c["ref_bytes"] = c["M"].reference_bytes()
        c["csr_bytes"] = c["csr"].algorithmic_bytes(1, False)
    log("tuned")

    sleep = getattr(torch.cuda, "_sleep", None)
    dither = random.Random(11)

    def one_step(record):
        for c in cases:
            flush()
            if sleep is not None:  # random start phase against the 2.048 us event-timer step (autotune.time_spmv)
                sleep(dither.randrange(DITHER_CYCLES))
            e0, e1 = record(c)
            e0.record(stream)
            L.LeSpMV(1.0, c["M"], c["x"], 0.0, c["y"], stream)
            e1.record(stream)

    for _ in range(args.warmup):
        one_step(lambda c: (torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)))
    torch.cuda.synchronize()

    events = {id(c): [] for c in cases}

    def rec(c):
        pair = (torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True))
        events[id(c)].append(pair)
        return pair

    sampler = ClockSampler(dev.index)
    _barrier(world)
    torch.cuda.synchronize()
    sampler.start()
    launches0 = _lib.lib.sspmv_launch_count()
    t0 = time.perf_counter()
    torch.cuda.nvtx.range_push("timed_steps")  # profilers select the timed launches by this range
    for _ in range(args.steps):
        one_step(rec)
    torch.cuda.nvtx.range_pop()
    torch.cuda.synchronize()
    wall = time.perf_counter() - t0
    launches = _lib.lib.sspmv_launch_count() - launches0
    clocks = sampler.stop()
    _barrier(world)
    log("timed steps done")

    parity = check_cases(cases, hosts)
    log("parity checked")

    per_case = []
    total_ms = 0.0
    total_bytes = 0.0
    for c in cases:
        ms = [a.elapsed_time(b) for a, b in events[id(c)]]
        avg = sum(ms) / len(ms)
        total_ms += sum(ms)
        total_bytes += c["bytes"] * len(ms)
        per_case.append({"family": c["fam"], "format": c["fmt"], "dtype": c["dt"], "ms": round(avg, 5),
                         "GBps": round(c["bytes"] / avg / 1e6, 1),
                         "ref_model_GBps": round(c["ref_bytes"] / avg / 1e6, 1),
                         "csr_equiv_GBps": round(c["csr_bytes"] / avg / 1e6, 1),
                         "GFLOPs": round(2.0 * c["nnz"] / avg / 1e6, 1),
                         "kernel": c["tuned"] or c["kernel"], "max_norm_err": c["max_norm_err"],
                         "median_norm_err": c["median_norm_err"]})
    step_ms = total_ms / args.steps
    step_ms = _max_over_ranks(step_ms, world)
    value = total_bytes / args.steps * world / (step_ms * 1e6)

    e2e = None
    if not args.no_e2e:
        e2e = run_e2e(args, cases, flush, stream, world)
        log("e2e done")

    dom = max(range(len(cases)), key=lambda i: per_case[i]["ms"])
    dc = cases[dom]
    peak, peak_kind = measured_peak()
    ach = dc["bytes"] / per_case[dom]["ms"] / 1e6
    tt = traffic_table().get(f"{dc['fam']}/{dc['fmt']}/{dc['dt']}")
    roofline = {"bound": "hbm", "achieved": round(ach, 1), "peak": peak, "unit": "GB/s",
                "frac": round(ach / peak, 4), "peak_kind": peak_kind,
                "traffic": tt["bytes_per_launch"] if tt else None,
                "kernel": f"{dc['fam']}/{dc['fmt']}/{dc['dt']}",
                "algorithmic_bytes": dc["bytes"]}
    if rank == 0:
        # random column indices: the x gathers, not HBM, bound the kernels; the
        # gather ceiling is measured live for each such matrix's x size and
        # gather count (one gather per nonzero)
        probes = Probes()
        ceiling = {}
        for c, pc in zip(cases, per_case):
            if c["fam"] not in RANDOM_COLUMN_FAMILIES:
                continue
            key = (c["fam"], c["dt"])
            if key not in ceiling:
                ceiling[key] = probes.gather_ceiling(np_dtype(c["dt"]), c["cols"], min(c["nnz"], 1 << 28))[0]
            pc["gather_frac"] = round(c["nnz"] / (pc["ms"] * 1e-3) / ceiling[key], 4)
        # the same bytes as a plain stream, cold: what a kernel of each case's
        # size reaches when it only moves data (short kernels do not reach
        # the multi-gigabyte copy's bandwidth)
        streams = {}
        for c, pc in zip(cases, per_case):
            yb = c["rows"] * (8 if c["dt"] == "f64" else 4)
            key = (int(c["bytes"]) - yb, yb)
            if key not in streams:
                streams[key] = probes.stream_ceiling_ms(*key)
            pc["stream_same_bytes_ms"] = round(streams[key], 5)
            pc["stream_frac"] = round(streams[key] / pc["ms"], 4)
        # FP64: one FMA per nonzero against the device's measured FP64 FMA rate
        fma_rate = probes.fp64_ceiling()
        for c, pc in zip(cases, per_case):
            if c["dt"] == "f64":
                pc["fp64_frac"] = round(c["nnz"] / (pc["ms"] * 1e-3) / fma_rate, 4)
        key = (dc["fam"], dc["dt"])
        rate = ceiling.get(key) or probes.gather_ceiling(np_dtype(dc["dt"]), dc["cols"], min(dc["nnz"], 1 << 28))[0]
        kernel_rate = dc["nnz"] / (per_case[dom]["ms"] * 1e-3)
        roofline["gather_ceiling"] = {
            "ceiling_gathers_per_s": round(rate, 1), "achieved_gathers_per_s": round(kernel_rate, 1),
            "frac": round(kernel_rate / rate, 4),
            "what": "one x gather per nonzero; ceiling = random gathers from a vector of the same size, "
                    "indices streamed (benchmark probe sspmv_gather_ceiling)"}
        roofline["stream_same_bytes_frac"] = per_case[dom]["stream_frac"]
        if dc["dt"] == "f64":
            roofline["fp64_ceiling"] = {
                "ceiling_fmas_per_s": round(fma_rate, 1), "achieved_fmas_per_s": round(kernel_rate, 1),
                "frac": round(kernel_rate / fma_rate, 4),
                "what": "one FP64 FMA per nonzero; ceiling = independent FMA chains (benchmark probe sspmv_fp64_ceiling)"}
    cpu = None
    if rank == 0 and world == 1 and not args.no_cpu:
        cpu = cpu_baseline(hosts, families, dtypes, fmts, budget_s=15.0)
        log("cpu baseline done")
    for c in cases:
        if c["M"] is not c["csr"]:
            c["M"].delete()
    for c in cases:
        c["csr"].delete()
    del cases, hosts
    return {
        "metric": SUITE_METRIC,
        "value": round(value, 1), "unit": "GB/s", "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": round(step_ms, 4), "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f64+f32", "data": "synthetic (seeded generator, families of the SpMV suite)",
        "config": {"workload": "spmv-suite: " + "+".join(families) + " x " + "+".join(fmts) + " x " + "+".join(dtypes),
                   "l2": L2_NOTE,
                   "alpha": 1.0, "beta": 0.0, "k_rhs": 1, "index": "int32", "parallelism": f"replicas{world}",
                   "skipped": skipped, "scale": args.scale},
        "e2e": e2e, "roofline": roofline, "cpu_baseline": cpu, "clocks": clocks, "gpu_launches": int(launches),
        "parity": parity,
        "wall_s": round(wall, 3), "per_format": per_case,
    }


def _x_host(n, dt):
    from sspmv_gb300 import synth
    return synth.vector(n, 0, np_dtype(dt))


def run_e2e(args, cases, flush, stream, world):
    """The same sweep through the public call with host buffers: pinned x
    copied in, SpMV, y copied out, every step.

    value: the copies run on their own streams (host-to-device, device-to-
    host) and overlap the SpMVs of other matrices: x of matrix i+1 moves while
    matrix i multiplies, y of matrix i while matrix i+1 multiplies.  One event
    bracket per sweep; the sweep's matrices total far more than L2, so there
    is no flush inside it.  The sweep takes the matrices largest first: the
    host enqueues a call in tens of microseconds, and while the large
    matrices' SpMVs run it gets ahead of the GPU, which then never waits for
    the host on the small ones.  serial_value: each SpMV with its own copies
    in one bracket on one stream (L2 flushed before each, flush not timed)."""
    import torch
    from sspmv_gb300 import lespmv as L
    hx = [c["x"].cpu().pin_memory() for c in cases]
    hy = [torch.empty(c["rows"], dtype=c["y"].dtype).pin_memory() for c in cases]
    h2d = sum(t.numel() * t.element_size() for t in hx)
    d2h = sum(t.numel() * t.element_size() for t in hy)
    step_bytes = float(sum(c["bytes"] for c in cases))
    s_in, s_out = torch.cuda.Stream(), torch.cuda.Stream()

    order = sorted(range(len(cases)), key=lambda i: -cases[i]["bytes"])

    def overlapped():
        t0, t1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        t0.record(stream)
        s_in.wait_stream(stream)
        s_out.wait_stream(stream)
        for i in order:
            c = cases[i]
            with torch.cuda.stream(s_in):
                c["x"].copy_(hx[i], non_blocking=True)
            stream.wait_stream(s_in)
            L.LeSpMV(1.0, c["M"], c["x"], 0.0, c["y"], stream)
            s_out.wait_stream(stream)
            with torch.cuda.stream(s_out):
                hy[i].copy_(c["y"], non_blocking=True)
        stream.wait_stream(s_out)
        t1.record(stream)
        torch.cuda.synchronize()
        return t0.elapsed_time(t1)

    def no_copies():
        # the same sweep with x and y left on the device: what the copies add
        t0, t1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        t0.record(stream)
        for i in order:
            L.LeSpMV(1.0, cases[i]["M"], cases[i]["x"], 0.0, cases[i]["y"], stream)
        t1.record(stream)
        torch.cuda.synchronize()
        return t0.elapsed_time(t1)

    def serial():
        pairs = []
        for i, c in enumerate(cases):
            flush()
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            c["x"].copy_(hx[i], non_blocking=True)
            L.LeSpMV(1.0, c["M"], c["x"], 0.0, c["y"], stream)
            hy[i].copy_(c["y"], non_blocking=True)
            e1.record(stream)
            pairs.append((e0, e1))
        torch.cuda.synchronize()
        return sum(a.elapsed_time(b) for a, b in pairs)

    torch.cuda.synchronize()
    with torch.cuda.stream(stream):
        for _ in range(args.warmup):
            overlapped()
        ov = sum(overlapped() for _ in range(args.steps)) / args.steps
        dev_only = sum(no_copies() for _ in range(args.steps)) / args.steps
        for _ in range(args.warmup):
            serial()
        se = sum(serial() for _ in range(args.steps)) / args.steps
    ov = _max_over_ranks(ov, world)
    se = _max_over_ranks(se, world)
    return {"value": round(step_bytes * world / (ov * 1e6), 1), "unit": "GB/s",
            "h2d_bytes_per_step": int(h2d), "d2h_bytes_per_step": int(d2h), "ms_per_step": round(ov, 4),
            "copies": "pinned host x in and y out of every SpMV on two copy streams, overlapping other SpMVs",
            "serial_value": round(step_bytes * world / (se * 1e6), 1), "serial_ms_per_step": round(se, 4),
            "sweep_without_copies_ms": round(dev_only, 4)}


# ------------------------------------------------------- result checking --
def check_cases(cases, hosts):
    """Every timed matrix's last y (= A x) on sampled rows -- every 61st row
    and the 64 longest -- against an FP64 product on the same inputs, in units
    of the per-row bound 8 nnz_i eps sum_j |a_ij x_j| (eps of the value type).
    Sets each case's max_norm_err / median_norm_err and returns the summary:
    max and median per format x precision over the four families."""
    import scipy.sparse as sp
    refs = {}
    per = {}
    for c in cases:
        key = (c["fam"], c["dt"])
        if key not in refs:
            A = hosts[key]
            lens = np.diff(A.row_offset)
            rows = np.union1d(np.arange(0, A.num_rows, 61), np.argsort(lens)[-64:])
            sub_ptr = np.concatenate([[0], np.cumsum(lens[rows])])
            take = np.repeat(A.row_offset[rows] - sub_ptr[:-1], lens[rows]) + np.arange(sub_ptr[-1])
            Asp = sp.csr_matrix((A.values[take].astype(np.float64), A.col_index[take], sub_ptr),
                                shape=(len(rows), A.num_cols))
            x64 = _x_host(A.num_cols, c["dt"]).astype(np.float64)
            eps = np.finfo(A.values.dtype).eps
            bound = 8.0 * np.maximum(lens[rows], 1) * eps * (abs(Asp) @ np.abs(x64)) + np.finfo(np.float64).tiny
            refs[key] = (rows, Asp @ x64, bound)
        rows, y64, bound = refs[key]
        yg = c["y"].cpu().numpy()[rows].astype(np.float64)
        err = np.abs(yg - y64) / bound
        c["max_norm_err"] = round(float(err.max(initial=0.0)), 4)
        c["median_norm_err"] = round(float(np.median(err)) if err.size else 0.0, 5)
        per.setdefault(f"{c['fmt']}/{c['dt']}", []).append(err)
    by_fmt = {}
    worst = 0.0
    for k, errs in per.items():
        e = np.concatenate(errs)
        mx = float(e.max(initial=0.0))
        worst = max(worst, mx)
        by_fmt[k] = [round(mx, 4), round(float(np.median(e)), 5)]
    return {"cases": len(cases), "rows": "every 61st and the 64 longest of each matrix",
            "max_norm_err": round(worst, 4), "within_tolerance": bool(worst <= 1.0),
            "tolerance": "|y - y_fp64| <= 8 nnz_i eps sum_j |a_ij x_j| per row",
            "max_median_by_format": by_fmt}


# ------------------------------------------------ large power-law section --
def fp64_row_check(A, X, Y, rows):
    """Normalised error of GPU rows Y[rows] against an FP64 product on the
    same (possibly FP32-rounded) inputs: |y - y64| / (8 nnz_i eps sum|a x|)."""
    import scipy.sparse as sp
    m = A.num_rows
    Asp = sp.csr_matrix((A.values.astype(np.float64), A.col_index, A.row_offset), shape=(m, A.num_cols))[rows]
    X64 = X.astype(np.float64).reshape(A.num_cols, -1)
    y64 = Asp @ X64
    absum = abs(Asp) @ np.abs(X64)
    nz = np.diff(A.row_offset)[rows].astype(np.float64)[:, None]
    eps = np.finfo(A.values.dtype).eps
    bound = 8.0 * np.maximum(nz, 1.0) * eps * absum + np.finfo(np.float64).tiny
    err = np.abs(Y.reshape(len(rows), -1).astype(np.float64) - y64) / bound
    return float(err.max(initial=0.0)), float(np.median(err))


def run_large(dev, peak):
    """Power-law N=16M (Zipf 2.0, mean 16, cap 50k), FP32 values, int32
    indices: SELL-c-sigma autotuned over C in {8,16,32} x sigma in {256,
    4096, N} against CSR (autotuned kernel), k = 1 and k = 8 right-hand
    sides; GB/s (algorithmic bytes / kernel time, L2 flushed), fraction of the
    measured HBM peak, and FP64 error on every 64th row."""
    import torch
    from sspmv_gb300 import autotune, synth
    from sspmv_gb300 import lespmv as L
    t0 = time.perf_counter()
    A = synth.generate(synth.WORKLOADS["powerlaw_16M"](), 1, np.float32)
    log(f"large: generated N={A.num_rows} nnz={A.nnz} ({time.perf_counter() - t0:.1f}s)")
    csr = L.csr_from_host(A)
    n, m = A.num_cols, A.num_rows
    x1 = torch.from_numpy(synth.vector(n, 0, np.float32)).to(dev)
    y1 = torch.zeros(m, dtype=torch.float32, device=dev)
    from sspmv_gb300.autotune import L2Flush
    flush = L2Flush(dev)
    out = {"workload": "powerlaw_16M f32 (Zipf 2.0, mean 16, cap 50k)", "num_rows": m, "nnz": A.nnz, "formats": {}}
    res_csr = autotune.tune_format(csr, x1, y1)
    sig_n = -(-m // 32) * 32
    cands = [dict(slicewidth=sg, chunkwidth=c, alignment=0) for c in (8, 16, 32) for sg in (256, 4096, sig_n)]
    best = None
    table = []
    for kw in cands:
        M = L.csr_to_sell_c_sigma(csr, **kw)
        ms = autotune.time_spmv(M, x1, y1, reps=5, flush=flush)
        table.append({"C": kw["chunkwidth"], "sigma": kw["slicewidth"], "ms": round(ms, 4)})
        if best is None or ms < best[1]:
            if best:
                best[0].delete()
            best = (M, ms, kw)
        else:
            M.delete()
    scs = best[0]
    out["sell_c_sigma_tuning"] = table
    log(f"large: tuned SELL-c-sigma C={best[2]['chunkwidth']} sigma={best[2]['slicewidth']}")
    rows = np.arange(0, m, 64)
    for name, M, tuned in (("csr", csr, res_csr["best"] if res_csr else None),
                           ("sell_c_sigma", scs, {"C": best[2]["chunkwidth"], "sigma": best[2]["slicewidth"]})):
        rec = {"tuned": tuned}
        for k in (1, 8):
            X = torch.from_numpy(synth.vector(n, 0, np.float32, k).reshape(n, k)).to(dev)
            Y = torch.zeros((m, k), dtype=torch.float32, device=dev)
            ts = []
            for i in range(6):
                flush()
                e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
                e0.record()
                L.spmm(1.0, M, X, 0.0, Y)
                e1.record()
                e1.synchronize()
                if i >= 1:
                    ts.append(e0.elapsed_time(e1))
            ms = statistics.median(ts)
            b = M.algorithmic_bytes(k, False)
            Yh = Y[torch.from_numpy(rows).to(dev)].cpu().numpy()
            mx, med = fp64_row_check(A, X.cpu().numpy(), Yh, rows)
            rec[f"k{k}"] = {"ms": round(ms, 4), "GBps": round(b / ms / 1e6, 1),
                            "GFLOPs": round(2.0 * A.nnz * k / ms / 1e6, 1),
                            "frac_of_measured_peak": round(b / ms / 1e6 / peak, 4),
                            "max_norm_err": round(mx, 4), "median_norm_err": round(med, 4),
                            "within_tolerance": mx <= 1.0}
            del X, Y
        out["formats"][name] = rec
        log(f"large: {name} {rec}")
    scs.delete()
    csr.delete()
    out["sell_vs_csr_speedup"] = {f"k{k}": round(out["formats"]["csr"][f"k{k}"]["ms"] /
                                                 out["formats"]["sell_c_sigma"][f"k{k}"]["ms"], 3) for k in (1, 8)}
    out["wall_s"] = round(time.perf_counter() - t0, 1)
    return out


def time_in_stream(fn, flush, reps: int = 50, rounds: int = 5) -> float:
    """Milliseconds of one cold call of fn inside a stream of work: reps x
    (L2 flush, fn) timed as one CUDA-event bracket, minus reps x (L2 flush)
    timed the same way, per call; the median of `rounds` such pairs.  A
    per-launch event pair around a 20 us kernel also times the launch and the
    two event records (about 3 us on this GPU, and in steps of about 2 us);
    over a bracket of reps calls those steps average out, and what is left
    is the call's cost in a stream of back-to-back work, its launch gap
    included."""
    import torch
    for _ in range(3):
        flush()
        fn()
    out = []
    for _ in range(rounds):
        ev = [torch.cuda.Event(enable_timing=True) for _ in range(3)]
        ev[0].record()
        for _ in range(reps):
            flush()
            fn()
        ev[1].record()
        for _ in range(reps):
            flush()
        ev[2].record()
        ev[2].synchronize()
        out.append((ev[0].elapsed_time(ev[1]) - ev[1].elapsed_time(ev[2])) / reps)
    out.sort()
    return out[len(out) // 2]


def run_laplacian(dev, peak, pin=None):
    """2-D 5-point Laplacian on a 1024 x 1024 grid, FP64 CSR, y = A x: the
    matrix is written as a Matrix Market file and read back through the
    library's reader (the reference CPU build's input path), then timed with
    L2 flushed (cold) and without flushing (the 84 MB working set stays in
    the 129 MB L2: warm).  pin = (kernel_flag, param) skips the tuner."""
    import torch
    from sspmv_gb300 import autotune, synth
    from sspmv_gb300 import lespmv as L
    A0 = synth.load("laplacian_1024", 1, np.float64)
    with tempfile.TemporaryDirectory() as d:
        path = str(Path(d) / "laplacian_1024.mtx")
        L.write_mtx(path, A0)
        A = L.read_csr_matrix(path, 64)
    same = bool(np.array_equal(A.row_offset, A0.row_offset) and np.array_equal(A.col_index, A0.col_index)
                and np.array_equal(A.values, A0.values))
    csr = L.csr_from_host(A)
    x = torch.from_numpy(synth.vector(A.num_cols, 0)).to(dev)
    y = torch.zeros(A.num_rows, dtype=torch.float64, device=dev)
    if pin:
        csr.set_kernel(*pin)
        tuned = {"best": {"kernel_flag": pin[0], "param": pin[1], "pinned": True}}
    else:
        tuned = autotune.tune_format(csr, x, y)
    flush = autotune.L2Flush(dev)
    torch.cuda.nvtx.range_push("laplacian_cold")  # profilers select the cold runs and the stream by this range
    cold = autotune.time_spmv(csr, x, y, reps=50, warmup=5, flush=flush)
    cold_seq = time_in_stream(lambda: L.LeSpMV(1.0, csr, x, 0.0, y), flush)
    ev = [torch.cuda.Event(enable_timing=True) for _ in range(2)]
    for _ in range(5):
        L.LeSpMV(1.0, csr, x, 0.0, y)
    ev[0].record()
    for _ in range(200):
        L.LeSpMV(1.0, csr, x, 0.0, y)
    ev[1].record()
    ev[1].synchronize()
    warm = ev[0].elapsed_time(ev[1]) / 200
    b = csr.algorithmic_bytes(1, False)
    # the same bytes as a plain stream (matrix and x in, y out), cold: what a
    # kernel of this size reaches when it only moves data
    stream_ms = Probes().stream_ceiling_ms(b - A.num_rows * 8, A.num_rows * 8)
    torch.cuda.nvtx.range_pop()
    rows = np.arange(0, A.num_rows, 16)
    mx, med = fp64_row_check(A, x.cpu().numpy(), y[torch.from_numpy(rows).to(dev)].cpu().numpy(), rows)
    csr.delete()
    return {"workload": "laplacian_1024 (N=1,048,576) FP64 CSR, alpha=1 beta=0, read from .mtx",
            "mtx_round_trip_exact": same, "nnz": A.nnz, "algorithmic_bytes": b, "kernel": tuned["best"] if tuned else None,
            "cold_ms": round(cold, 5), "cold_GBps": round(b / cold / 1e6, 1),
            "cold_frac_of_measured_peak": round(b / cold / 1e6 / peak, 4),
            "cold_in_stream_ms": round(cold_seq, 5), "cold_in_stream_GBps": round(b / cold_seq / 1e6, 1),
            "cold_in_stream_frac_of_measured_peak": round(b / cold_seq / 1e6 / peak, 4),
            "stream_same_bytes_ms": round(stream_ms, 5), "cold_frac_of_stream_same_bytes": round(stream_ms / cold, 4),
            "warm_ms": round(warm, 5), "warm_GBps": round(b / warm / 1e6, 1),
            "max_norm_err": round(mx, 4), "median_norm_err": round(med, 4)}


def run_serving():
    """The request server on its serving workload (64 matrices x FP64/FP32),
    pinned-host and device buffers: saturation throughput and p50/p99 under
    Poisson load, batched vs one launch per request."""
    from sspmv_gb300 import serving
    model = ROOT / "sspmv_gb300" / "data" / "selector_model.npz"
    out = {"selector_model": str(model.relative_to(ROOT)) if model.exists() else None}
    for kind, dev_buf in (("host", False), ("device", True)):
        r = serving.serving_benchmark(64, device_buffers=dev_buf, log=log,
                                      selector_model=model if model.exists() else None)
        out[kind] = r
    return out


# ------------------------------------------------------------- CPU legs ----
def cpu_sample(A, frac=0.125):
    """First `frac` of the rows of A (all columns kept)."""
    from sspmv_gb300.synth import HostCSR
    r = max(1, int(A.num_rows * frac))
    nnz = int(A.row_offset[r])
    return HostCSR(r, A.num_cols, A.row_offset[:r + 1].copy(), A.col_index[:nnz], A.values[:nnz])


# The reference's CSR5 SpMV (src/spmv_csr5.cpp) is written with x86 AVX-512
# intrinsics that only ICC accepts: it has no CPU implementation to time on
# the GB300's Arm host, so the CPU legs leave CSR5 out and say so.
CPU_UNAVAILABLE = {"csr5": "unavailable on aarch64 host (reference CSR5 SpMV is x86 AVX-512 only)"}


def _cpu_convert(O, fmt, A):
    """Oracle (CPU restatement) conversion of a sample for the CPU timing; None if infeasible."""
    from sspmv_gb300.formats import feasible_host
    ok, _ = feasible_host(fmt, A)
    if not ok or fmt in CPU_UNAVAILABLE:
        return None
    if fmt == "csr":
        return {}
    if fmt == "coo":
        return O.csr_to_coo(A)
    if fmt == "ell":
        d = O.csr_to_ell(A, 1)
        d["ld"] = 1
        return d
    if fmt == "sell":
        d = O.csr_to_sell(A, 4)
        d["C"] = 4
        return d
    if fmt == "sell_c_sigma":
        d = O.csr_to_sell_c_sigma(A, 16384, 4)
        d["C"] = 4
        return d
    if fmt == "sell_c_R":
        d = O.csr_to_sell_c_R(A, 4)
        d["C"] = 4
        return d
    if fmt == "dia":
        return O.csr_to_dia(A)
    if fmt == "bsr":
        from sspmv_gb300.formats import bsr_block_for
        r, c = bsr_block_for(A)
        return O.csr_to_bsr(A, r, c)
    return None


def _cpu_bytes(fmt, A, d, sv):
    m, n, nnz = A.num_rows, A.num_cols, A.nnz
    xb, yb = n * sv, m * sv
    if fmt == "csr":
        return nnz * (sv + 4) + (m + 1) * 4 + xb + yb
    if fmt == "coo":
        return nnz * (sv + 8) + xb + yb
    if fmt in ("ell", "sell"):
        return nnz * (sv + 4) + xb + yb
    if fmt in ("sell_c_sigma", "sell_c_R"):
        return nnz * (sv + 4) + m * 4 + xb + yb
    if fmt == "dia":
        return nnz * sv + d["complete_ndiags"] * 8 + xb + yb
    if fmt == "bsr":
        return nnz * sv + d["nnzb"] * 4 + (d["mb"] + 1) * 4 + xb + yb
    return nnz * (sv + 4) + xb + yb


def cpu_sweep(hosts, families, dtypes, fmts, budget_s, frac=0.125):
    """Times the oracle port's OpenMP SpMV kernels (all host threads) on the
    first `frac` of the rows of every matrix.  The oracle restates the
    reference's OpenMP kernels (src/spmv_<fmt>.cpp); the reference's own
    sources are not present where the benchmark runs.  Returns (GB/s,
    seconds, threads, sweeps)."""
    sys.path.insert(0, str(ROOT / "oracle"))
    from oracle import Oracle
    O = Oracle()
    threads = O.lib.oracle_max_threads()
    prepared = []
    for fam in families:
        for dt in dtypes:
            A = cpu_sample(hosts[(fam, dt)], frac)
            for fmt in fmts:
                d = _cpu_convert(O, fmt, A)
                if d is None:
                    continue
                x = _x_host(A.num_cols, dt)
                y = np.zeros(A.num_rows, np_dtype(dt))
                prepared.append((fmt, A, d, x, y, _cpu_bytes(fmt, A, d, np.dtype(np_dtype(dt)).itemsize)))
    tot_b, tot_t = 0.0, 0.0
    t_start = time.perf_counter()
    reps = 0
    while True:
        for fmt, A, d, x, y, b in prepared:
            t0 = time.perf_counter()
            O.spmv(fmt, d, A, 1.0, x, 0.0, y)
            tot_t += time.perf_counter() - t0
            tot_b += b
        reps += 1
        if time.perf_counter() - t_start > budget_s or reps >= 50:
            break
    return tot_b / tot_t / 1e9, tot_t, threads, reps


def cpu_baseline(hosts, families, dtypes, fmts, budget_s):
    gbs, secs, threads, reps = cpu_sweep(hosts, families, dtypes, fmts, budget_s)
    return {"value": round(gbs, 2), "unit": "GB/s", "cores": threads, "kind": "port",
            "sample": f"first 1/8 of the rows of every matrix, {reps} sweep(s), {secs:.1f} s of SpMV time; "
                      "oracle restatement of the reference's OpenMP kernels; csr5 " + CPU_UNAVAILABLE["csr5"]}


def run_reference(args, rank, world):
    if rank != 0:
        return None
    families = [f for f in args.families.split(",") if f]
    dtypes = [d for d in args.dtypes.split(",") if d]
    from sspmv_gb300.formats import FORMATS
    fmts = FORMATS if args.formats == "all" else args.formats.split(",")
    hosts = host_matrices(families, args.scale)
    for _ in range(args.warmup):
        cpu_sweep(hosts, families, dtypes, fmts, budget_s=0.0)
    vals = []
    t0 = time.perf_counter()
    for _ in range(args.steps):
        gbs, secs, threads, _ = cpu_sweep(hosts, families, dtypes, fmts, budget_s=0.0)
        vals.append((gbs, secs))
    gbs = sum(v[0] * v[1] for v in vals) / sum(v[1] for v in vals)
    ms = sum(v[1] for v in vals) / len(vals) * 1e3
    return {"impl": "reference",
            "metric": "SpMV GB/s (algorithmic bytes / kernel time), all formats x 4 families x {f64,f32}",
            "value": round(gbs, 2), "unit": "GB/s", "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": round(ms, 3), "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "f64+f32", "data": "synthetic (seeded generator, families of the SpMV suite)",
            "config": {"workload": "spmv-suite: " + "+".join(families) + " x " + "+".join(fmts) + " x " + "+".join(dtypes),
                       "sample": "first 1/8 of the rows of every matrix", "wall_s": round(time.perf_counter() - t0, 2)},
            "cpu_baseline": {"value": round(gbs, 2), "unit": "GB/s", "cores": threads, "kind": "port",
                             "sample": "first 1/8 of the rows of every matrix, one sweep per step; csr5 "
                                       + CPU_UNAVAILABLE["csr5"]},
            "e2e": {"value": round(gbs, 2), "unit": "GB/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}


# ------------------------------------------------------------ distributed --
def _dist():
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    return rank, world


def _barrier(world):
    if world > 1:
        import torch.distributed as dist
        dist.barrier()


def _max_over_ranks(v, world):
    """Max of v over the ranks (NCCL on the GPUs; gloo process groups, as in
    the CPU tests, reduce on the host)."""
    if world == 1:
        return v
    import torch
    import torch.distributed as dist
    dev = "cuda" if dist.get_backend() == "nccl" else "cpu"
    t = torch.tensor([v], dtype=torch.float64, device=dev)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


# ------------------------------------------------------------- output ----
HEADLINE_LIMIT = 4000


def _by_format_GBps(per_case):
    """Algorithmic bytes / kernel time per format x precision over the four
    families (sum of bytes / sum of time)."""
    acc = {}
    for pc in per_case:
        k = f"{pc['format']}/{pc['dtype']}"
        b, t = acc.get(k, (0.0, 0.0))
        acc[k] = (b + pc["GBps"] * pc["ms"], t + pc["ms"])
    return {k: round(b / t, 1) for k, (b, t) in acc.items() if t > 0}


def headline(out: dict) -> dict:
    """The compact result line: the contract keys, the roofline and CPU
    baseline, parity max / median per format x precision, and one-number
    summaries of the Laplacian, 16M power-law and serving sections (their
    full records are in the detail file)."""
    h = {k: out[k] for k in ("metric", "value", "unit", "n_gpus", "steps", "warmup", "ms_per_step",
                             "higher_is_better", "scaling", "vs_baseline", "dtype", "data") if k in out}
    cfg = dict(out.get("config", {}))
    skipped = cfg.pop("skipped", [])
    cfg["skipped"] = len(skipped)
    h["config"] = cfg
    e2e = out.get("e2e")
    if e2e:
        h["e2e"] = {k: e2e[k] for k in ("value", "unit", "h2d_bytes_per_step", "d2h_bytes_per_step",
                                        "ms_per_step", "serial_value") if k in e2e}
    rf = out.get("roofline")
    if rf:
        h["roofline"] = {k: rf.get(k) for k in ("bound", "achieved", "peak", "unit", "frac", "traffic", "kernel",
                                                "algorithmic_bytes", "peak_kind")}
        for extra in ("gather_ceiling", "fp64_ceiling"):
            if rf.get(extra):
                h["roofline"][extra + "_frac"] = rf[extra]["frac"]
        if rf.get("stream_same_bytes_frac") is not None:
            h["roofline"]["stream_same_bytes_frac"] = rf["stream_same_bytes_frac"]
    h["cpu_baseline"] = out.get("cpu_baseline")
    h["clocks"] = out.get("clocks")
    h["gpu_launches"] = out.get("gpu_launches")
    par = out.get("parity") or {}
    h["parity"] = {"within_tolerance": par.get("within_tolerance"), "max_norm_err": par.get("max_norm_err"),
                   "max_median_by_format": par.get("max_median_by_format"), "tolerance": par.get("tolerance")}
    if out.get("per_format"):
        h["GBps_by_format"] = _by_format_GBps(out["per_format"])
    lap = out.get("laplacian_1024")
    if lap:
        h["laplacian_1024"] = {k: lap.get(k) for k in ("cold_GBps", "cold_frac_of_measured_peak", "cold_ms",
                                                       "cold_in_stream_ms", "cold_in_stream_frac_of_measured_peak",
                                                       "stream_same_bytes_ms", "cold_frac_of_stream_same_bytes",
                                                       "warm_GBps", "max_norm_err", "median_norm_err")}
        h["laplacian_1024"]["kernel"] = (lap.get("kernel") or {}).get("kernel_flag"), (lap.get("kernel") or {}).get("param")
    large = out.get("large_powerlaw_16M")
    if large:
        h["large_powerlaw_16M"] = {f"{f}_k{k}_GBps": large["formats"][f][f"k{k}"]["GBps"]
                                   for f in large.get("formats", {}) for k in (1, 8)}
        h["large_powerlaw_16M"]["max_norm_err"] = max(large["formats"][f][f"k{k}"]["max_norm_err"]
                                                      for f in large["formats"] for k in (1, 8))
    srv = out.get("serving")
    if srv:
        h["serving"] = {}
        for kind in ("host", "device"):
            r = srv.get(kind)
            if not r:
                continue
            h["serving"][kind] = {"saturation_ratio": {m: round(v, 3) for m, v in r.get("saturation_ratio", {}).items()},
                                  "equal_p99_ratio": {m: (round(v["throughput_ratio"], 3)
                                                          if v.get("throughput_ratio") is not None else None)
                                                      for m, v in r.get("equal_p99", {}).items()}}
    line = json.dumps(h, separators=(",", ":"))
    # stay within the limit: drop the least important summaries first
    for key in ("serving", "large_powerlaw_16M", "GBps_by_format"):
        if len(line) <= HEADLINE_LIMIT:
            break
        h.pop(key, None)
        line = json.dumps(h, separators=(",", ":"))
    return h


def emit(out: dict, args) -> None:
    """Full record to the detail file, compact line as the last stdout line."""
    if args.detail:
        try:
            Path(args.detail).parent.mkdir(parents=True, exist_ok=True)
            Path(args.detail).write_text(json.dumps(out, indent=1))
            log(f"detail written to {args.detail}")
        except OSError as e:
            log(f"detail not written: {e}")
    h = headline(out)
    if args.detail:
        h["detail"] = str(Path(args.detail).relative_to(ROOT)) if Path(args.detail).is_relative_to(ROOT) else args.detail
    print(json.dumps(h, separators=(",", ":")), flush=True)


def main():
    args = parse_args()
    rank, world = _dist()
    if args.impl == "reference":
        out = run_reference(args, rank, world)
        if out is not None:
            print(json.dumps(out))
        return
    if world > 1:
        import torch
        import torch.distributed as dist
        torch.cuda.set_device(int(os.environ.get("LOCAL_RANK", "0")))
        dist.init_process_group("nccl")
    out = run_gpu(args, rank, world)
    if rank == 0:
        emit(out, args)
    if world > 1:
        import torch.distributed as dist
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
