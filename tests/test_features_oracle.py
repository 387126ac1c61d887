"""Pins the oracle's restatement of the reference's MTX feature extractor
(oracle/oracle_features.c) to the reference's own output stored in the
golden fixtures: per-tile counts bit-exact, features per features_util."""
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
