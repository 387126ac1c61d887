"""Request server over the C ABI (sspmv_server_*), and its serving workload.

A `Server` keeps registered matrices resident in HBM in their serving format
(least-recently-used eviction under a byte budget) and serves SpMV / SpMM
requests y = alpha*A*X + beta*Y with continuous batching: requests that
arrive while batches run on the GPU are gathered into the next batch, whose
CSR requests (k in 1, 2, 4, 8) run in one persistent stream-kernel launch per
(value type, k) group replayed from a CUDA graph.  mode="per_request" serves
each request with its own sspmv_spmm_<fmt> launch instead (the comparison
point).

The reference has no serving layer (its benchmark programs run one matrix per
process); the workload below is the serving configuration the library is
measured on: 64 resident matrices mixed across the synthetic families with N
log-uniform in [1e3, 1e6], requests SpMV or SpMM with k in {1, 2, 4, 8}, FP64
or FP32, Poisson arrivals.
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass

import numpy as np

from . import _lib, synth
from ._lib import ServerConfig, ServerStats, call, lib
from .synth import HostCSR

FORMAT_IDS = {"csr": 0, "coo": 1, "ell": 2, "sell": 3, "sell_c_sigma": 4, "sell_c_R": 5, "dia": 6, "bsr": 7,
              "csr5": 8}
MODES = {"batched": 0, "per_request": 1}
DEVICE_BUFFERS = 1

REQUEST_DTYPE = np.dtype({"names": ["matrix_id", "k", "alpha", "beta", "x", "ldx", "y", "ldy", "flags", "reserved"],
                          "formats": ["<i4", "<i4", "<f8", "<f8", "<u8", "<i8", "<u8", "<i8", "<i4", "<i4"],
                          "offsets": [0, 4, 8, 16, 24, 32, 40, 48, 56, 60], "itemsize": 64})
INFO_DTYPE = np.dtype({"names": ["status", "batch_size", "batch_id", "arrival_ns", "launch_ns", "done_ns"],
                       "formats": ["<i4", "<i4", "<i8", "<i8", "<i8", "<i8"],
                       "offsets": [0, 4, 8, 16, 24, 32], "itemsize": 40})
assert REQUEST_DTYPE.itemsize == C.sizeof(_lib.Request) and INFO_DTYPE.itemsize == C.sizeof(_lib.RequestInfo)


def _vt(dtype) -> int:
    return _lib.F64 if np.dtype(dtype) == np.float64 else _lib.F32


class Server:
    """Owns one sspmv_server.  Registered host arrays are kept referenced
    here for as long as the server lives (the server reads them on load)."""

    def __init__(self, mode: str = "batched", max_batch_requests: int = 0, max_batch_tiles: int = 0,
                 arena_bytes: int = 0, stage_limit_bytes: int = 0, hbm_budget_bytes: int = 0,
                 num_inflight: int = 0, use_graphs: bool = True):
        cfg = ServerConfig()
        cfg.mode = MODES[mode]
        cfg.max_batch_requests = max_batch_requests
        cfg.max_batch_tiles = max_batch_tiles
        cfg.arena_bytes = arena_bytes
        cfg.stage_limit_bytes = stage_limit_bytes
        cfg.hbm_budget_bytes = hbm_budget_bytes
        cfg.num_inflight = num_inflight
        cfg.use_graphs = 1 if use_graphs else 0
        h = C.c_void_p()
        call("sspmv_server_create", C.byref(cfg), C.byref(h))
        self._h = h
        self.mode = mode
        self._keep: dict[int, HostCSR] = {}
        self.shapes: dict[int, tuple[int, int, np.dtype]] = {}

    def close(self) -> None:
        if self._h:
            call("sspmv_server_destroy", self._h)
            self._h = C.c_void_p()

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def add_matrix(self, mid: int, A: HostCSR, fmt: str = "csr", params=None) -> None:
        A = HostCSR(A.num_rows, A.num_cols, np.ascontiguousarray(A.row_offset, np.int32),
                    np.ascontiguousarray(A.col_index, np.int32), np.ascontiguousarray(A.values))
        p = None
        if params:
            p = (C.c_int32 * 4)(*(list(params) + [0] * (4 - len(params))))
        call("sspmv_server_add_matrix", self._h, int(mid), _vt(A.values.dtype), A.num_rows, A.num_cols, A.nnz,
             A.row_offset.ctypes.data, A.col_index.ctypes.data if A.nnz else None,
             A.values.ctypes.data if A.nnz else None, FORMAT_IDS[fmt], p)
        self._keep[mid] = A
        self.shapes[mid] = (A.num_rows, A.num_cols, A.values.dtype)

    def preload(self, mid: int) -> None:
        call("sspmv_server_preload", self._h, int(mid))

    @staticmethod
    def _ld(a, k: int) -> int:
        if a.ndim == 1:
            return k
        return int(a.stride(0)) if callable(getattr(a, "stride", None)) else a.strides[0] // a.itemsize

    @staticmethod
    def _ptr(a) -> int:
        if hasattr(a, "data_ptr"):
            return int(a.data_ptr())
        return int(a.ctypes.data)

    def submit(self, mid: int, x, y, alpha: float = 1.0, beta: float = 0.0, k: int | None = None,
               device: bool = False) -> int:
        """x: num_cols x k (or num_cols) host array (device tensor with
        device=True), y likewise num_rows x k; both must stay alive until
        wait() returns."""
        if k is None:
            k = 1 if x.ndim == 1 else int(x.shape[1])
        r = _lib.Request(int(mid), int(k), float(alpha), float(beta), self._ptr(x), self._ld(x, k), self._ptr(y),
                         self._ld(y, k), DEVICE_BUFFERS if device else 0, 0)
        t = C.c_int64()
        call("sspmv_server_submit", self._h, C.byref(r), C.byref(t))
        return t.value

    def wait(self, ticket: int, timeout: float = -1.0) -> dict:
        info = _lib.RequestInfo()
        st = lib.sspmv_server_wait(self._h, int(ticket), float(timeout), C.byref(info))
        _lib.check(st, "sspmv_server_wait")
        return {f: getattr(info, f) for f, _ in _lib.RequestInfo._fields_}

    def replay(self, reqs: np.ndarray, arrival_ns: np.ndarray) -> np.ndarray:
        """Open-loop load: request i is submitted arrival_ns[i] after the
        call starts; returns one INFO_DTYPE record per request."""
        reqs = np.ascontiguousarray(reqs, REQUEST_DTYPE)
        arrival_ns = np.ascontiguousarray(arrival_ns, np.int64)
        infos = np.zeros(len(reqs), INFO_DTYPE)
        st = lib.sspmv_server_replay(self._h, len(reqs), reqs.ctypes.data, arrival_ns.ctypes.data,
                                     infos.ctypes.data)
        _lib.check(st, "sspmv_server_replay")
        return infos

    def stats(self) -> dict:
        s = ServerStats()
        call("sspmv_server_get_stats", self._h, C.byref(s))
        return {f: getattr(s, f) for f, _ in ServerStats._fields_}


# --------------------------------------------------------------- workload --
FAMILIES = ("banded", "powerlaw", "block", "uniform")


def serving_matrix(family: str, n: int, seed: int) -> HostCSR:
    """One matrix of the serving mix (FP64 values; FP32 copies are rounded)."""
    if family == "banded":
        p = synth.banded(n)
    elif family == "powerlaw":
        p = synth.powerlaw(n, 1.8, 16.0, min(50000, n))
    elif family == "block":
        p = synth.block(n, 4, max(1, n // 4))
    else:
        p = synth.uniform(n, min(32, n))
    return synth.generate(p, seed, np.float64)


def serving_matrices(num: int = 64, n_min: int = 1000, n_max: int = 1_000_000, seed: int = 0) -> list[dict]:
    """`num` matrices cycling over the four families, N log-uniform in
    [n_min, n_max] (seeded)."""
    rng = np.random.default_rng(seed)
    ns = np.exp(rng.uniform(np.log(n_min), np.log(n_max), num)).astype(np.int64)
    out = []
    for i in range(num):
        fam = FAMILIES[i % len(FAMILIES)]
        n = int(ns[i])
        if fam == "block":
            n = max(4, n - n % 4)
        out.append({"family": fam, "n": n, "A": serving_matrix(fam, n, 100 + i)})
    return out


@dataclass
class RequestStream:
    reqs: np.ndarray        # REQUEST_DTYPE
    arrival_ns: np.ndarray  # int64, ascending
    matrix: np.ndarray      # served matrix index per request
    k: np.ndarray
    f64: np.ndarray


def request_stream(num_requests: int, matrix_ids_f64: list[int], matrix_ids_f32: list[int], rate: float,
                   seed: int = 1, ks=(1, 2, 4, 8)) -> RequestStream:
    """Poisson arrivals at `rate` requests/s (rate <= 0: all at time 0);
    each request picks a matrix uniformly, k uniformly from ks and FP64 or
    FP32 with equal odds.  Buffers are filled in by the caller."""
    rng = np.random.default_rng(seed)
    nm = len(matrix_ids_f64)
    mat = rng.integers(0, nm, num_requests)
    k = np.asarray(ks)[rng.integers(0, len(ks), num_requests)]
    f64 = rng.integers(0, 2, num_requests).astype(bool)
    if rate > 0:
        gaps = rng.exponential(1.0 / rate, num_requests)
        arrival = np.cumsum(gaps) * 1e9
        arrival -= arrival[0]
    else:
        arrival = np.zeros(num_requests)
    reqs = np.zeros(num_requests, REQUEST_DTYPE)
    ids64, ids32 = np.asarray(matrix_ids_f64), np.asarray(matrix_ids_f32)
    reqs["matrix_id"] = np.where(f64, ids64[mat], ids32[mat])
    reqs["k"] = k
    reqs["alpha"] = 1.0
    reqs["beta"] = 0.0
    reqs["ldx"] = k
    reqs["ldy"] = k
    return RequestStream(reqs, arrival.astype(np.int64), mat, k, f64)


def latency_summary(infos: np.ndarray) -> dict:
    """p50 / p99 latency (arrival to result in the caller's buffer) and the
    completed-requests throughput of one replay."""
    ok = infos["status"] == 0
    lat = (infos["done_ns"] - infos["arrival_ns"])[ok] / 1e3
    span = (infos["done_ns"].max() - infos["arrival_ns"].min()) / 1e9 if len(infos) else 0.0
    bs = infos["batch_size"][ok]
    return {"requests": int(len(infos)), "failed": int((~ok).sum()),
            "req_per_s": float(ok.sum() / span) if span > 0 else 0.0,
            "p50_us": float(np.percentile(lat, 50)) if len(lat) else None,
            "p99_us": float(np.percentile(lat, 99)) if len(lat) else None,
            "mean_batch": float(bs.mean()) if len(bs) else 0.0}


# -------------------------------------------------------------- benchmark --
class ServingBench:
    """The serving workload on one GPU: `num_matrices` matrices registered in
    FP64 (ids 2i) and FP32 (ids 2i+1), one X and one Y buffer per id holding
    up to 8 right-hand sides (pinned host memory, or device memory with
    device_buffers=True).  Requests on one id share its buffers, so
    overlapping requests write the same Y: the benchmark times the serving
    path, the parity tests check results."""

    def __init__(self, num_matrices: int = 64, seed: int = 0, device_buffers: bool = False, log=None):
        import torch
        self.log = log or (lambda *a: None)
        self.mats = serving_matrices(num_matrices, seed=seed)
        self.device_buffers = device_buffers
        self.host = {}
        self.xbuf, self.ybuf = {}, {}
        for i, d in enumerate(self.mats):
            A64 = d["A"]
            for mid, A in ((2 * i, A64), (2 * i + 1, A64.astype(np.float32))):
                self.host[mid] = A
                tdt = torch.float64 if A.values.dtype == np.float64 else torch.float32
                if device_buffers:
                    x = torch.rand(A.num_cols * 8, dtype=tdt, device="cuda") * 2 - 1
                    y = torch.zeros(A.num_rows * 8, dtype=tdt, device="cuda")
                else:
                    x = torch.empty(A.num_cols * 8, dtype=tdt, pin_memory=True)
                    x.copy_(torch.from_numpy(synth.vector(A.num_cols * 8, mid, A.values.dtype)))
                    y = torch.zeros(A.num_rows * 8, dtype=tdt, pin_memory=True)
                self.xbuf[mid], self.ybuf[mid] = x, y
        self.ids64 = [2 * i for i in range(len(self.mats))]
        self.ids32 = [2 * i + 1 for i in range(len(self.mats))]
        self.total_nnz = sum(d["A"].nnz for d in self.mats)

    def server(self, mode: str, fmt_of=None, **kw) -> Server:
        s = Server(mode=mode, **kw)
        for mid, A in self.host.items():
            fmt, params = fmt_of(mid, A) if fmt_of else ("csr", None)
            s.add_matrix(mid, A, fmt, params)
        for mid in self.host:
            s.preload(mid)
        return s

    def stream(self, num_requests: int, rate: float, seed: int) -> RequestStream:
        rs = request_stream(num_requests, self.ids64, self.ids32, rate, seed)
        mids = rs.reqs["matrix_id"]
        rs.reqs["x"] = [self.xbuf[m].data_ptr() for m in mids]
        rs.reqs["y"] = [self.ybuf[m].data_ptr() for m in mids]
        rs.reqs["flags"] = DEVICE_BUFFERS if self.device_buffers else 0
        return rs

    def run(self, s: Server, num_requests: int, rate: float, seed: int) -> dict:
        rs = self.stream(num_requests, rate, seed)
        infos = s.replay(rs.reqs, rs.arrival_ns)
        out = latency_summary(infos)
        out["offered_per_s"] = float(rate) if rate > 0 else None
        return out


# converter integer arguments in sspmv_server_add_matrix order, from the
# keyword names the Python converters take
_PARAM_ORDER = {"ell": ["ld"], "sell": ["chunkwidth", "alignment"],
                "sell_c_sigma": ["slicewidth", "chunkwidth", "alignment"], "sell_c_R": ["chunkwidth", "alignment"],
                "dia": ["max_diags", "alignment"], "bsr": ["blockDimRow", "blockDimCol"], "csr5": ["sigma", "omega"]}


def server_params(fmt: str, params: dict | None) -> list[int] | None:
    if fmt not in _PARAM_ORDER or not params:
        return None
    return [int(params.get(k, 0)) for k in _PARAM_ORDER[fmt]]


def select_formats(mats: list[dict], model_path, min_nnz: int = 1_000_000, log=None) -> list[tuple[str, list | None]]:
    """Serving format of each matrix: the selector's pick for matrices with
    at least min_nnz nonzeros (their kernel time dwarfs a launch), CSR --
    batched with the other requests -- for the rest."""
    from . import lespmv as L
    from .selector import Selector
    sel = Selector(model_path)
    out = []
    for d in mats:
        A = d["A"]
        if A.nnz < min_nnz:
            out.append(("csr", None))
            continue
        csr = L.csr_from_host(A)
        fmt, prm = sel.pick(csr)
        csr.delete()
        out.append((fmt, server_params(fmt, prm)))
        if log:
            log(f"[serving] {d['family']} n={A.num_rows} nnz={A.nnz}: {fmt} {prm}")
    return out


def _us(v) -> str:
    return "n/a" if v is None else f"{v:.0f} us"


SWEEP_FRACTIONS = (0.2, 0.4, 0.6, 0.8, 1.0, 1.2, 1.5)


def throughput_at_p99(sweep: list[dict], target_us: float) -> float | None:
    """Highest completed-request throughput at which a server's p99 stays
    within target_us, linearly interpolated between its sweep points (p99 as
    a function of throughput, points in offered-rate order).  None if even
    its lightest point is above the target."""
    pts = [(r["req_per_s"], r["p99_us"]) for r in sweep if r.get("p99_us") is not None]
    if not pts or pts[0][1] > target_us:
        return None
    best = pts[0][0]
    for (t0, p0), (t1, p1) in zip(pts, pts[1:]):
        if p1 <= target_us:
            best = max(best, t1)
            continue
        if p0 <= target_us < p1 and p1 > p0:  # crosses the target between these points
            best = max(best, t0 + (t1 - t0) * (target_us - p0) / (p1 - p0))
        break
    return best


def equal_p99(res: dict, batched: str = "batched") -> dict:
    """Throughput of the batched server against each baseline at equal p99.
    The target is the baseline's p99 at its most loaded sweep point that
    still keeps up with the offered rate (completed >= 95% of offered); both
    servers' throughputs at that p99 are interpolated from their sweeps."""
    out = {}
    bsw = res["modes"][batched]["sweep"]
    for base in res["modes"]:
        if base == batched:
            continue
        sw = res["modes"][base]["sweep"]
        kept = [r for r in sw if r["offered_per_s"] and r["req_per_s"] >= 0.95 * r["offered_per_s"]]
        if not kept:
            continue
        ref = kept[-1]
        target = ref["p99_us"]
        tb, tr = throughput_at_p99(bsw, target), throughput_at_p99(sw, target)
        out[base] = {"p99_target_us": target, "baseline_req_per_s": tr, "batched_req_per_s": tb,
                     "throughput_ratio": (tb / tr) if (tb and tr) else None}
    return out


def serving_benchmark(num_matrices: int = 64, device_buffers: bool = False, duration_s: float = 2.0,
                      seed: int = 0, log=None, selector_model=None, fractions=SWEEP_FRACTIONS) -> dict:
    """Saturation throughput of the batched server and of per-request CSR
    launches (8 requests in flight, and 1: the plain serial loop), then every
    server under the same Poisson offered rates -- `fractions` of the 8-deep
    per-request server's saturation, duration_s of arrivals per point (a
    server is not run at rates above 1.2x its own saturation, where its queue
    only grows) -- with p50/p99 per point, and the throughput ratios at
    saturation and at equal p99 (interpolated)."""
    log = log or (lambda *a: None)
    b = ServingBench(num_matrices, seed, device_buffers, log)
    picks = select_formats(b.mats, selector_model, log=log) if selector_model else None
    res = {"matrices": num_matrices, "registered": 2 * num_matrices, "total_nnz_per_precision": b.total_nnz,
           "buffers": "device" if device_buffers else "pinned host", "seconds_per_point": duration_s,
           "modes": {},
           "server_config": {"per_request": {"num_inflight": 8, "arena_bytes": 160 << 20},
                             "per_request_serial": {"num_inflight": 1, "arena_bytes": 160 << 20},
                             "batched": {"num_inflight": 4, "arena_bytes": 512 << 20,
                                         "max_batch_tiles": 1 << 16}}}
    server_kw = res["server_config"]
    if picks:
        res["formats"] = {f"{d['family']}:{d['n']}": pk[0] for d, pk in zip(b.mats, picks) if pk[0] != "csr"}

    def fmt_of(mode):
        # the per-request comparison point is plain CSR; the batched server
        # serves each matrix in its selected format
        if mode != "batched" or not picks:
            return None
        return lambda mid, A: picks[mid // 2]

    modes = ("per_request", "per_request_serial", "batched")
    servers = {}
    try:
        for mode in modes:
            s = b.server("batched" if mode == "batched" else "per_request", fmt_of(mode), **server_kw[mode])
            servers[mode] = s
            b.run(s, 2000, 0.0, seed + 1)  # warm: graphs for the group sets, pools
            sat = b.run(s, {"batched": 20000, "per_request": 8000, "per_request_serial": 3000}[mode], 0.0, seed + 2)
            log(f"[serving] {mode}: saturation {sat['req_per_s']:.0f} req/s, mean batch {sat['mean_batch']:.1f}")
            res["modes"][mode] = {"saturation": sat, "sweep": [], "stats": None}
        base = res["modes"]["per_request"]["saturation"]["req_per_s"]
        res["offered_rates_per_s"] = [f * base for f in fractions]
        for mode in modes:
            m = res["modes"][mode]
            satm = m["saturation"]["req_per_s"]
            for f in fractions:
                rate = f * base
                if rate > 1.2 * satm:
                    m.setdefault("not_run_above_saturation", []).append(f)
                    continue
                n = int(min(max(rate * duration_s, 1000), 400000))
                r = b.run(servers[mode], n, rate, seed + 10 + int(f * 100))
                r["fraction_of_per_request_saturation"] = f
                m["sweep"].append(r)
                log(f"[serving] {mode} @ {rate:.0f}/s: {r['req_per_s']:.0f} req/s p50 {_us(r['p50_us'])} "
                    f"p99 {_us(r['p99_us'])} batch {r['mean_batch']:.1f} failed {r['failed']}")
            m["stats"] = servers[mode].stats()
    finally:
        for s in servers.values():
            s.close()
    res["saturation_ratio"] = {m: res["modes"]["batched"]["saturation"]["req_per_s"] /
                               max(res["modes"][m]["saturation"]["req_per_s"], 1e-9)
                               for m in ("per_request", "per_request_serial")}
    res["equal_p99"] = equal_p99(res)
    return res


def mix_bound(num_matrices: int = 64, seed: int = 0, thresholds=(1e5, 1e6, 4e6), log=None) -> dict:
    """GPU time per request of the serving mix, request kind by request kind
    (matrix x precision x k, each equally likely, as in request_stream): the
    request's CSR SpMM captured 20 times in a CUDA graph, replayed, timed
    with CUDA events (no host launch gaps; warm).  Reports the mean, and the
    share of it spent on requests whose matrix has at least each threshold
    of nonzeros: work that batching cannot remove, which bounds any
    server's throughput at about 1 / (that share)."""
    import torch
    from . import lespmv as L
    mats = serving_matrices(num_matrices, seed=seed)
    recs = []
    for i, d in enumerate(mats):
        for dt in (np.float64, np.float32):
            A = d["A"] if dt == np.float64 else d["A"].astype(np.float32)
            csr = L.csr_from_host(A)
            tdt = torch.float64 if dt == np.float64 else torch.float32
            for k in (1, 2, 4, 8):
                X = torch.rand((A.num_cols, k), dtype=tdt, device="cuda")
                Y = torch.zeros((A.num_rows, k), dtype=tdt, device="cuda")
                for _ in range(3):  # plans built before capture
                    L.spmm(1.0, csr, X, 0.0, Y)
                torch.cuda.synchronize()
                g = torch.cuda.CUDAGraph()
                st = torch.cuda.Stream()
                with torch.cuda.stream(st):
                    with torch.cuda.graph(g, stream=st):
                        for _ in range(20):
                            L.spmm(1.0, csr, X, 0.0, Y)
                g.replay()
                torch.cuda.synchronize()
                e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
                e0.record()
                g.replay()
                e1.record()
                e1.synchronize()
                recs.append({"matrix": i, "nnz": A.nnz, "dtype": np.dtype(dt).name, "k": k,
                             "us": e0.elapsed_time(e1) * 1e3 / 20})
                del g, X, Y
            csr.delete()
        if log:
            log(f"[serving bound] matrix {i}: nnz {d['A'].nnz}")
    n = len(recs)
    mean = sum(r["us"] for r in recs) / n
    out = {"request_kinds": n, "mean_us_per_request": mean, "bound_req_per_s": 1e6 / mean, "split": []}
    for t in thresholds:
        big = sum(r["us"] for r in recs if r["nnz"] >= t) / n
        out["split"].append({"nnz_at_least": t, "kinds": sum(1 for r in recs if r["nnz"] >= t),
                             "mean_us_of_these": big, "mean_us_of_the_rest": mean - big,
                             "bound_req_per_s_from_these": (1e6 / big) if big > 0 else None})
    out["requests"] = recs
    return out


def main(argv=None) -> None:
    """python -m sspmv_gb300.serving sweep [--seconds 5] [--buffers device,host] [--out FILE]
    python -m sspmv_gb300.serving bound [--out FILE]

    sweep: the serving workload's full sweep (longer points than the
    benchmark's default run), one JSON document per buffer kind.
    bound: GPU time per request of the mix (mix_bound)."""
    import argparse
    import json
    import sys
    from pathlib import Path
    ap = argparse.ArgumentParser(prog="python -m sspmv_gb300.serving")
    sub = ap.add_subparsers(dest="cmd", required=True)
    sw = sub.add_parser("sweep")
    sw.add_argument("--seconds", type=float, default=5.0)
    sw.add_argument("--buffers", default="device,host")
    sw.add_argument("--matrices", type=int, default=64)
    sw.add_argument("--out", default="")
    bd = sub.add_parser("bound")
    bd.add_argument("--matrices", type=int, default=64)
    bd.add_argument("--out", default="")
    a = ap.parse_args(argv)
    if a.cmd == "bound":
        res = mix_bound(a.matrices, log=lambda m: print(m, file=sys.stderr, flush=True))
        if a.out:
            Path(a.out).write_text(json.dumps(res, indent=1))
        print(json.dumps({k: v for k, v in res.items() if k != "requests"}))
        return
    model = Path(__file__).resolve().parent / "data" / "selector_model.npz"
    out = {}
    for kind in a.buffers.split(","):
        out[kind] = serving_benchmark(a.matrices, device_buffers=(kind == "device"), duration_s=a.seconds,
                                      log=lambda m: print(m, file=sys.stderr, flush=True),
                                      selector_model=model if model.exists() else None)
    text = json.dumps(out, indent=1)
    if a.out:
        Path(a.out).write_text(text)
    summary = {k: {"saturation_ratio": v["saturation_ratio"], "equal_p99": v["equal_p99"]} for k, v in out.items()}
    print(json.dumps(summary))


if __name__ == "__main__":
    main()
