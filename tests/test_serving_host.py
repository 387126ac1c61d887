"""Host side of the request server (no GPU): the request / info record
layouts match the C ABI, the serving workload generator and the latency
summary."""
import ctypes as C

import numpy as np


def test_record_layouts_match_c_abi():
    from sspmv_gb300 import _lib
    from sspmv_gb300.serving import INFO_DTYPE, REQUEST_DTYPE
    for dt, st in ((REQUEST_DTYPE, _lib.Request), (INFO_DTYPE, _lib.RequestInfo)):
        assert dt.itemsize == C.sizeof(st)
        for name, _ in st._fields_:
            assert dt.fields[name][1] == getattr(st, name).offset, name


def test_request_stream_poisson_and_mix():
    from sspmv_gb300.serving import request_stream
    ids64, ids32 = [0, 2, 4, 6], [1, 3, 5, 7]
    rs = request_stream(40000, ids64, ids32, rate=50000.0, seed=3)
    gaps = np.diff(rs.arrival_ns) / 1e9
    assert rs.arrival_ns[0] == 0 and (gaps >= 0).all()
    assert abs(gaps.mean() * 50000.0 - 1.0) < 0.03
    assert set(np.unique(rs.reqs["k"])) == {1, 2, 4, 8}
    assert (rs.reqs["ldx"] == rs.reqs["k"]).all() and (rs.reqs["ldy"] == rs.reqs["k"]).all()
    mid = rs.reqs["matrix_id"]
    assert np.array_equal(mid % 2 == 0, rs.f64)
    assert abs(rs.f64.mean() - 0.5) < 0.02
    again = request_stream(40000, ids64, ids32, rate=50000.0, seed=3)
    assert np.array_equal(again.reqs, rs.reqs) and np.array_equal(again.arrival_ns, rs.arrival_ns)
    burst = request_stream(100, ids64, ids32, rate=0.0)
    assert (burst.arrival_ns == 0).all()


def test_serving_matrices_mix():
    from sspmv_gb300.serving import FAMILIES, serving_matrices
    mats = serving_matrices(8, n_min=1000, n_max=20000, seed=5)
    assert [d["family"] for d in mats] == list(FAMILIES) * 2
    for d in mats:
        A = d["A"]
        assert 996 <= A.num_rows <= 20000 and A.num_rows == A.num_cols == d["n"]
        assert A.row_offset[-1] == A.nnz and A.nnz > 0
        if d["family"] == "block":
            assert A.num_rows % 4 == 0


def test_latency_summary():
    from sspmv_gb300.serving import INFO_DTYPE, latency_summary
    infos = np.zeros(100, INFO_DTYPE)
    infos["arrival_ns"] = np.arange(100) * 1000
    infos["done_ns"] = infos["arrival_ns"] + (np.arange(100) + 1) * 1000
    infos["batch_size"] = 4
    infos["status"][-1] = 4
    s = latency_summary(infos)
    assert s["failed"] == 1 and s["requests"] == 100
    assert abs(s["p50_us"] - 50.0) < 1.0 and s["p99_us"] <= 99.0
    assert s["mean_batch"] == 4.0



def test_throughput_at_p99_interpolates():
    from sspmv_gb300.serving import throughput_at_p99
    sw = [{"req_per_s": 1000.0, "p99_us": 100.0}, {"req_per_s": 2000.0, "p99_us": 200.0},
          {"req_per_s": 2900.0, "p99_us": 1000.0}]
    assert throughput_at_p99(sw, 150.0) == 1500.0   # halfway between the first two points
    assert throughput_at_p99(sw, 600.0) == 2450.0
    assert throughput_at_p99(sw, 5000.0) == 2900.0  # every point within the target
    assert throughput_at_p99(sw, 50.0) is None      # even the lightest point is above it


def test_equal_p99_uses_the_baselines_last_sustained_point():
    from sspmv_gb300.serving import equal_p99

    def pt(off, got, p99):
        return {"offered_per_s": off, "req_per_s": got, "p99_us": p99}
    res = {"modes": {
        "batched": {"sweep": [pt(1000, 1000, 50), pt(2000, 2000, 60), pt(3000, 3000, 80), pt(4000, 3990, 400)]},
        "per_request": {"sweep": [pt(1000, 1000, 100), pt(2000, 1990, 300), pt(3000, 2500, 9000)]},
    }}
    eq = equal_p99(res)["per_request"]
    assert eq["p99_target_us"] == 300            # 3000 offered, 2500 done: not sustained
    assert eq["baseline_req_per_s"] == 1990
    assert abs(eq["batched_req_per_s"] - (3000 + 990 * 220 / 320)) < 1e-6
    assert abs(eq["throughput_ratio"] - eq["batched_req_per_s"] / 1990) < 1e-12
