"""Host-side Matrix Market and CSR utilities against the reference's
semantics (utils/sparse_io.cpp, include/sparse_operation.h), no GPU."""

def test_read_mtx_coo_file_order(tmp_path):
    """read_coo_matrix order: triplets as they appear in the file, 1-based to
    0-based, each symmetric off-diagonal entry followed by its mirror."""
    from sspmv_gb300 import lespmv as L
    p = tmp_path / "s.mtx"
    p.write_text("%%MatrixMarket matrix coordinate real symmetric\n% c\n3 3 4\n3 1 2.5\n1 1 1.0\n2 1 -4\n3 3 7\n")
    m, n, r, c, v = L.read_coo_triplets(str(p))
    assert (m, n) == (3, 3)
    assert r.tolist() == [2, 0, 0, 1, 0, 2]
    assert c.tolist() == [0, 2, 0, 0, 1, 2]
    assert v.tolist() == [2.5, 2.5, 1.0, -4.0, -4.0, 7.0]
    A = L.read_csr_matrix(str(p))
    assert A.row_offset.tolist() == [0, 3, 4, 6]
    assert A.col_index.tolist() == [2, 0, 1, 0, 0, 2]


def _sum_duplicates_reference_order(rp, ci, cv, n):
    """Plain restatement of sum_csr_duplicates (include/sparse_operation.h:
    22-73) for the check: head-first chain of first appearances."""
    out_rp, out_ci, out_cv = [0], [], []
    for i in range(len(rp) - 1):
        sums, order = {}, []
        for jj in range(rp[i], rp[i + 1]):
            j = int(ci[jj])
            if j not in sums:
                sums[j] = 0.0
                order.append(j)
            sums[j] += float(cv[jj])
        for j in reversed(order):
            if sums[j] != 0:
                out_ci.append(j)
                out_cv.append(sums[j])
        out_rp.append(len(out_ci))
    return out_rp, out_ci, out_cv


def test_sum_csr_duplicates():
    import numpy as np
    from sspmv_gb300 import lespmv as L
    from sspmv_gb300.synth import HostCSR
    A = HostCSR(2, 5, np.array([0, 5, 7], np.int32), np.array([3, 1, 3, 2, 1, 4, 4], np.int32),
                np.array([1.0, 2.0, 3.0, 4.0, -2.0, 0.5, 0.25]))
    B = L.sum_csr_duplicates(A)
    assert B.row_offset.tolist() == [0, 2, 3]
    assert B.col_index.tolist() == [2, 3, 4]
    assert B.values.tolist() == [4.0, 4.0, 0.75]
    rng = np.random.default_rng(5)
    m, n = 200, 40
    lens = rng.integers(0, 30, m)
    rp = np.concatenate([[0], np.cumsum(lens)]).astype(np.int32)
    ci = rng.integers(0, n, rp[-1]).astype(np.int32)
    cv = rng.integers(-3, 4, rp[-1]).astype(np.float64)  # small integers: exact sums, some zero
    B = L.sum_csr_duplicates(HostCSR(m, n, rp, ci, cv))
    r_rp, r_ci, r_cv = _sum_duplicates_reference_order(rp, ci, cv, n)
    assert B.row_offset.tolist() == r_rp and B.col_index.tolist() == r_ci and B.values.tolist() == r_cv
