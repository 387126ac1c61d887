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

