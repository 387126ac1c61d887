"""Request server on the GPU: results of requests batched together equal the
same requests served alone (bit for bit) and the single-request entry points
(bit for bit, batched CSR path), and lie within the FP64 oracle's tolerance;
least-recently-used eviction under a small HBM budget; device-buffer
requests; argument errors.

Tolerance (per row): |y_i - y_ref_i| <= 8*nnz_i*eps*|alpha|*sum_j|a_ij x_j|
+ 2*eps*|beta*y0_i|, y_ref the FP64 CSR result on the same inputs."""
import numpy as np
import pytest

from gpu_util import to_dev, to_host
from oracle import tolerance_ok

pytestmark = pytest.mark.gpu

ALPHA, BETA = 0.8, 0.7


def _matrices():
    from sspmv_gb300 import synth
    g = synth.generate
    empty = synth.HostCSR(10, 10, np.zeros(11, np.int32), np.zeros(0, np.int32), np.zeros(0))
    tiny = synth.HostCSR(1, 1, np.array([0, 1], np.int32), np.array([0], np.int32), np.array([2.5]))
    return {
        0: (g(synth.powerlaw(30000, 1.8, 16.0, 20000, 0.02), 3, np.float64), "csr", None),
        1: (g(synth.powerlaw(30000, 1.8, 16.0, 20000, 0.02), 3, np.float32), "csr", None),
        2: (g(synth.uniform(5000, 8), 4, np.float32), "sell_c_sigma", (256, 8, 0)),
        3: (g(synth.banded(20000), 5, np.float64), "csr", None),
        4: (tiny, "csr", None),
        5: (empty, "csr", None),
        6: (g(synth.block(4000, 4, 800), 6, np.float64), "coo", None),
        7: (g(synth.uniform(3000, 24, 0.1, num_cols=7000), 8, np.float32), "csr", None),
    }


def _requests(mats):
    """(matrix id, k, beta) for every matrix and k in 1, 2, 3, 4, 8."""
    out = []
    for mid in mats:
        for i, k in enumerate((1, 2, 3, 4, 8)):
            out.append((mid, k, BETA if (mid + i) % 2 else 0.0))
    return out


def _buffers(mats, reqs, seed=0):
    from sspmv_gb300 import synth
    xs, y0s = [], []
    for j, (mid, k, beta) in enumerate(reqs):
        A = mats[mid][0]
        dt = A.values.dtype
        xs.append(synth.vector(A.num_cols, seed + j, dt, k).reshape(A.num_cols, k))
        y0s.append(synth.vector(A.num_rows, 1000 + j, dt, k).reshape(A.num_rows, k))
    return xs, y0s


def _server(mats, **kw):
    from sspmv_gb300.serving import Server
    s = Server(**kw)
    for mid, (A, fmt, params) in mats.items():
        s.add_matrix(mid, A, fmt, params)
    return s


def _alone(s, reqs, xs, y0s):
    ys = []
    for (mid, k, beta), x, y0 in zip(reqs, xs, y0s):
        y = y0.copy()
        t = s.submit(mid, x, y, ALPHA, beta)
        info = s.wait(t, 60.0)
        assert info["status"] == 0
        ys.append(y)
    return ys


def _mixed(s, reqs, xs, y0s):
    from sspmv_gb300.serving import REQUEST_DTYPE
    ys = [y0.copy() for y0 in y0s]
    rq = np.zeros(len(reqs), REQUEST_DTYPE)
    for j, ((mid, k, beta), x, y) in enumerate(zip(reqs, xs, ys)):
        rq[j] = (mid, k, ALPHA, beta, x.ctypes.data, k, y.ctypes.data, k, 0, 0)
    infos = s.replay(rq, np.zeros(len(reqs), np.int64))
    assert (infos["status"] == 0).all()
    return ys, infos


def _check_oracle(oracle_lib, mats, reqs, xs, y0s, ys):
    for (mid, k, beta), x, y0, y in zip(reqs, xs, y0s, ys):
        A = mats[mid][0]
        y64, absum = oracle_lib.spmm_ref(A, x, ALPHA, beta, y0)
        ok, mx, _ = tolerance_ok(y, y64.reshape(y.shape), absum.reshape(y.shape), np.diff(A.row_offset),
                                 A.values.dtype, ALPHA, beta, y0)
        assert ok, f"matrix {mid} k={k} beta={beta}: max normalised error {mx}"


def test_batched_equals_alone_and_oracle(oracle_lib):
    mats = _matrices()
    reqs = _requests(mats)
    xs, y0s = _buffers(mats, reqs)
    with _server(mats) as s:
        ys_alone = _alone(s, reqs, xs, y0s)
        ys_mix, infos = _mixed(s, reqs, xs, y0s)
        st = s.stats()
    assert infos["batch_size"].max() > 1, "requests arriving together were not batched"
    assert st["batched_requests"] > 0 and st["graph_launches"] > 0
    for (mid, k, beta), a, b in zip(reqs, ys_alone, ys_mix):
        assert np.array_equal(a, b), f"matrix {mid} k={k}: result differs alone vs in the mix"
    _check_oracle(oracle_lib, mats, reqs, xs, y0s, ys_mix)


def test_batched_csr_equals_single_request_entry_point():
    from sspmv_gb300.lespmv import csr_from_host, spmm
    mats = {m: v for m, v in _matrices().items() if v[1] == "csr"}
    reqs = [(m, k, b) for (m, k, b) in _requests(mats) if k in (1, 2, 4, 8)]
    xs, y0s = _buffers(mats, reqs, seed=50)
    with _server(mats) as s:
        ys, _ = _mixed(s, reqs, xs, y0s)
    dev = {m: csr_from_host(v[0]) for m, v in mats.items()}
    for (mid, k, beta), x, y0, y in zip(reqs, xs, y0s, ys):
        Y = to_dev(y0)
        spmm(ALPHA, dev[mid], to_dev(x), beta, Y)
        assert np.array_equal(to_host(Y), y), f"matrix {mid} k={k}: batched differs from sspmv_spmm_csr"


def _long_row_matrix(seed, m=600, long_len=3000):
    """A small CSR matrix whose row 7 spans more than ten 256-nonzero chunks
    (its other rows 1..12 nonzeros), so rows crossing many chunks of different
    matrices meet in one warp of the batched fix-up."""
    from sspmv_gb300 import synth
    rng = np.random.default_rng(seed)
    lens = rng.integers(1, 13, m)
    lens[7] = long_len
    rp = np.concatenate([[0], np.cumsum(lens)]).astype(np.int32)
    cols = np.concatenate([np.sort(rng.choice(8000, size=l, replace=False)) for l in lens]).astype(np.int32)
    vals = rng.uniform(-1, 1, rp[-1])
    return synth.HostCSR(m, 8000, rp, cols, vals)


def test_batched_long_rows_across_many_small_matrices(oracle_lib):
    """Dozens of small matrices in one batch, each with a row spanning many
    chunks: equal to the single-request entry point bit for bit."""
    from sspmv_gb300.lespmv import csr_from_host, spmm
    mats = {m: (_long_row_matrix(m, long_len=1500 + 97 * m), "csr", None) for m in range(40)}
    reqs = [(m, 1 + (m % 2), BETA if m % 3 else 0.0) for m in mats]
    xs, y0s = _buffers(mats, reqs, seed=70)
    with _server(mats) as s:
        ys, infos = _mixed(s, reqs, xs, y0s)
    assert infos["batch_size"].max() > 1
    dev = {m: csr_from_host(v[0]) for m, v in mats.items()}
    for (mid, k, beta), x, y0, y in zip(reqs, xs, y0s, ys):
        Y = to_dev(y0)
        spmm(ALPHA, dev[mid], to_dev(x), beta, Y)
        assert np.array_equal(to_host(Y), y), f"matrix {mid} k={k}: batched differs from sspmv_spmm_csr"
    _check_oracle(oracle_lib, mats, reqs, xs, y0s, ys)


@pytest.mark.parametrize("graphs", [True, False], ids=["graphs", "direct"])
def test_per_request_mode_and_direct_launches_match(graphs):
    mats = _matrices()
    reqs = _requests(mats)
    xs, y0s = _buffers(mats, reqs, seed=90)
    with _server(mats, use_graphs=graphs, num_inflight=3) as s:
        ys_b, _ = _mixed(s, reqs, xs, y0s)
    with _server(mats, mode="per_request") as s:
        ys_p, infos = _mixed(s, reqs, xs, y0s)
    assert (infos["batch_size"] == 1).all()
    for (mid, k, beta), a, b in zip(reqs, ys_b, ys_p):
        assert np.array_equal(a, b), f"matrix {mid} k={k}: batched and per-request results differ"


def test_lru_eviction_under_budget(oracle_lib):
    from sspmv_gb300 import synth
    mats = {i: (synth.generate(synth.uniform(20000, 16), 20 + i, np.float64), "csr", None) for i in range(4)}
    one = 20001 * 4 + 320000 * 12
    reqs = [(i % 4, 1 + (i % 2), 0.0) for i in range(16)]
    xs, y0s = _buffers(mats, reqs, seed=7)
    with _server(mats, hbm_budget_bytes=int(2.6 * one)) as s:
        ys = _alone(s, reqs, xs, y0s)
        st1 = s.stats()
        ys_mix, _ = _mixed(s, reqs, xs, y0s)
        st2 = s.stats()
    assert st1["evictions"] >= 12 and st1["resident_matrices"] <= 2
    assert st2["resident_bytes"] <= int(2.6 * one)
    for a, b in zip(ys, ys_mix):
        assert np.array_equal(a, b)
    _check_oracle(oracle_lib, mats, reqs, xs, y0s, ys_mix)


def test_device_buffer_requests_match_host_requests():
    mats = _matrices()
    reqs = _requests(mats)
    xs, y0s = _buffers(mats, reqs, seed=31)
    with _server(mats) as s:
        ys_host, _ = _mixed(s, reqs, xs, y0s)
        dx = [to_dev(x) for x in xs]
        dy = [to_dev(y0) for y0 in y0s]
        ts = [s.submit(mid, x, y, ALPHA, beta, device=True) for (mid, k, beta), x, y in zip(reqs, dx, dy)]
        for t in ts:
            assert s.wait(t, 60.0)["status"] == 0
    for (mid, k, beta), a, b in zip(reqs, ys_host, dy):
        assert np.array_equal(a, to_host(b)), f"matrix {mid} k={k}: device-buffer result differs"


def test_server_errors():
    from sspmv_gb300 import synth
    from sspmv_gb300._lib import SSPMVError
    A = synth.generate(synth.uniform(50000, 4), 1, np.float64)
    with _server({0: (A, "csr", None)}, arena_bytes=1 << 16, hbm_budget_bytes=64 << 20) as s:
        x = np.zeros(A.num_cols)
        y = np.zeros(A.num_rows)
        with pytest.raises(SSPMVError):
            s.submit(99, x, y)
        with pytest.raises(SSPMVError):
            s.submit(0, x, y, k=0)
        t = s.submit(0, x, y)  # 400 KB of x does not fit a 64 KB staging arena
        with pytest.raises(SSPMVError) as e:
            s.wait(t, 60.0)
        assert e.value.status == 1
    big = synth.generate(synth.uniform(200000, 16), 1, np.float64)
    with _server({0: (big, "csr", None)}, hbm_budget_bytes=1 << 20) as s:
        t = s.submit(0, np.zeros(big.num_cols), np.zeros(big.num_rows))
        with pytest.raises(SSPMVError) as e:
            s.wait(t, 60.0)
        assert e.value.status == 4
