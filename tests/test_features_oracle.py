"""Pins the oracle's restatement of the reference's MTX feature extractor
(oracle/oracle_features.c) to the reference's own output stored in the
golden fixtures: per-tile counts bit-exact, features per features_util."""
import numpy as np
import pytest

from features_util import compare
from golden_util import digest, files, load

CASES = [p for p in files() if "empty" not in p.stem]


@pytest.mark.parametrize("path", CASES, ids=[p.stem for p in CASES])
def test_oracle_features_match_reference(path, oracle_lib):
    z, meta, A = load(path)
    F, arrs = oracle_lib.features(A, 256)
    bad = compare(F, z["features"])
    assert not bad, f"features differ (index, oracle, reference): {bad[:5]}"
    for k, d in meta["feature_arrays"].items():
        assert digest(arrs[k]) == d, k


def _rows_csr(m, n, rows, values=None):
    from sspmv_gb300.synth import HostCSR
    rp, ci = [0], []
    for r in rows:
        ci += r
        rp.append(len(ci))
    v = np.ones(len(ci)) if values is None else np.asarray(values, np.float64)
    return HostCSR(m, n, np.array(rp, np.int32), np.array(ci, np.int32), v)


def test_oracle_grx_known_answers(oracle_lib):
    """GrX features worked by hand from the reference's loops
    (AnalyzeTile_Group and the potReuse flags, src/sparse_features.cpp:884-1042):
    16 x 16 with T = 2 gives 8 x 8 tiles."""
    empty = [[] for _ in range(15)]
    # one row, columns 0..7: X = 4 counts the group at 0, resumes at 5 where
    # 5 + 4 > 8 ends the row -> 1 group; 1 of 4 (row group, tile col) pairs;
    # column groups 0, 1 of tile col 0 -> 2 of 4.
    A = _rows_csr(16, 16, [list(range(8))] + empty)
    assert np.allclose(oracle_lib.grx(A, T=2, X=4), [0.0, 1 / 8, 1 / 4, 2 / 4])
    # X = 3: groups at 0 and 4 (resume after the skipped column 3) -> 2.
    assert np.allclose(oracle_lib.grx(A, T=2, X=3), [0.0, 2 / 8, 1 / 6, 3 / 6])
    # columns 0..8 cross into the second tile: 1 group; row group 0 in both tiles.
    B = _rows_csr(16, 16, [list(range(9))] + empty)
    assert np.allclose(oracle_lib.grx(B, T=2, X=4), [0.0, 1 / 9, 2 / 4, 3 / 4])
    # the same runs down a column count for GrX_uniqR
    Ct = _rows_csr(16, 16, [[3]] * 8 + [[] for _ in range(8)])
    assert np.allclose(oracle_lib.grx(Ct, T=2, X=4), [1 / 8, 0.0, 2 / 4, 1 / 4])
    # an explicit zero breaks a run: columns 0..7 with column 2 zero -> run 3..7 (L = 5) -> 1 group
    D = _rows_csr(16, 16, [list(range(8))] + empty, values=[1, 1, 0, 1, 1, 1, 1, 1])
    assert np.allclose(oracle_lib.grx(D, T=2, X=4)[1], 1 / 8)
    # tiles narrower than X leave the features at -1
    assert np.allclose(oracle_lib.grx(A, T=2, X=9), [-1, -1, -1, -1])
