"""Selector host logic (no GPU): the seeded dataset mix, model inputs,
training targets and the regret arithmetic."""
import numpy as np


def test_dataset_spec_ranges_and_determinism():
    from sspmv_gb300.selector import dataset_spec
    specs = [dataset_spec(i, 0) for i in range(400)]
    assert specs[17] == dataset_spec(17, 0) and specs[17] != dataset_spec(17, 1)
    fams = {s["family"] for s in specs}
    assert fams == {"banded", "powerlaw", "block", "uniform", "mix"}
    for s in specs:
        assert 10_000 <= s["n"] <= 2_000_000 and 1.0 <= s["r"] <= 1000.0


def test_dataset_matrices_are_valid_csr():
    from sspmv_gb300.selector import dataset_matrix, dataset_spec
    for i in range(40):
        spec = dict(dataset_spec(i, 3))
        spec["n"] = min(spec["n"], 20000)
        A = dataset_matrix(spec)
        rp = A.row_offset
        assert rp[0] == 0 and rp[-1] == A.nnz and (np.diff(rp) >= 0).all()
        assert A.nnz == len(A.col_index) == len(A.values)
        assert A.col_index.min(initial=0) >= 0 and A.col_index.max(initial=0) < A.num_cols
        for r in range(0, A.num_rows, max(1, A.num_rows // 50)):
            c = A.col_index[rp[r]:rp[r + 1]]
            assert (np.diff(c) > 0).all()


def test_mixture_stacks_two_families():
    from sspmv_gb300.selector import dataset_matrix
    spec = {"i": 5, "family": "mix", "n": 8000, "r": 12.0, "seed": 0}
    A = dataset_matrix(spec)
    assert A.num_rows == A.num_cols == 8000
    top = np.diff(A.row_offset[:4001]).mean()
    bot = np.diff(A.row_offset[4000:]).mean()
    assert top > 0 and bot > 0


def test_model_inputs_and_targets():
    from sspmv_gb300.selector import CSR_LABEL, model_inputs, targets_from_times
    raw = np.array([[1.0, -2.0, 0.0], [10.0, 0.5, -1.0]])
    X = model_inputs(raw)
    assert X.shape == (2, 6)
    assert np.allclose(X[:, 3:], np.sign(raw) * np.log1p(np.abs(raw)))
    times = np.full((2, 9), np.inf)
    times[:, CSR_LABEL] = 2.0
    times[0, 0] = 1.0
    t, mask = targets_from_times(times)
    assert mask[0, 0] == 1 and mask[1, 0] == 0 and mask[:, CSR_LABEL].all()
    assert np.isclose(t[0, 0], np.log(0.5)) and t[0, CSR_LABEL] == 0.0


def test_regret_arithmetic():
    from sspmv_gb300.selector import CSR_LABEL, regret
    times = np.array([[1.0, 2.0, np.inf, 4.0, 5.0, 6.0, 7.0, 8.0, 9.0],
                      [3.0, 1.5, 1.0, 4.0, 5.0, 6.0, 7.0, 8.0, 9.0]])
    r = regret(times, np.array([0, 2]))
    assert r["mean_regret"] == 0.0 and r["exact_pick_rate"] == 1.0
    r = regret(times, np.array([2, CSR_LABEL]))  # infeasible pick falls back to CSR
    assert np.isclose(r["mean_regret"], ((2.0 / 1.0 - 1) + (1.5 / 1.0 - 1)) / 2)
    assert np.isclose(r["csr_mean_regret"], r["mean_regret"])


def test_feasibility_from_features_and_server_params():
    from sspmv_gb300.selector import LABELS, NUM_DIAGS, feasible_from_features
    from sspmv_gb300.serving import server_params
    raw = np.zeros((3, 66))
    raw[:, 0] = 1000           # rows
    raw[:, 2] = 10000          # nonzeros
    raw[:, 7] = [10, 41, 10]   # longest row: ELL pads 1x, 4.1x, 1x
    raw[:, NUM_DIAGS] = [9, 9, 20000]
    f = feasible_from_features(raw)
    ell, dia = LABELS.index("ell"), LABELS.index("dia")
    assert f[0, ell] and not f[1, ell] and f[2, ell]
    assert f[0, dia] and f[1, dia] and not f[2, dia]
    assert f[:, LABELS.index("csr")].all()
    assert server_params("sell_c_sigma", {"slicewidth": 256, "chunkwidth": 8, "alignment": 0}) == [256, 8, 0]
    assert server_params("bsr", {"blockDimRow": 2, "blockDimCol": 4}) == [2, 4]
    assert server_params("csr", {"kernel_flag": 1, "param": 4}) is None


def test_packaged_dataset_is_consistent():
    from sspmv_gb300 import selector as S
    ds = S.load_dataset(S.PACKAGE_DATA / "selector_dataset.npz")
    assert ds.raw.shape == (2000, 66) and ds.times.shape == (2000, 9)
    assert np.isfinite(ds.times[:, S.CSR_LABEL]).all() and (ds.times > 0).all()
    assert set(np.unique(ds.labels)) <= set(range(S.NUM_CLASSES))
    hist = np.bincount(ds.labels, minlength=S.NUM_CLASSES)
    assert hist[S.CSR_LABEL] < 0.6 * len(ds.ids)  # CSR is often, not always, fastest
