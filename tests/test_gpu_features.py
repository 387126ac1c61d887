"""GPU feature extraction (sspmv_csr_features) against the reference's own
MTX output (golden fixtures) and the oracle on larger seeded matrices:
per-tile counts bit-exact, integer features equal, floating ones within
1e-9 relative (features_util)."""
import numpy as np
import pytest

from features_util import compare
from golden_util import digest, files, load

pytestmark = pytest.mark.gpu

CASES = [p for p in files() if "empty" not in p.stem]


@pytest.mark.parametrize("path", CASES, ids=[p.stem for p in CASES])
def test_gpu_features_match_reference(path):
    from sspmv_gb300 import lespmv as L
    z, meta, A = load(path)
    F, arrs = L.features(L.csr_from_host(A), 256, arrays=True)
    bad = compare(F, z["features"])
    assert not bad, f"features differ (index, gpu, reference): {bad[:5]}"
    for k, d in meta["feature_arrays"].items():
        assert digest(arrs[k]) == d, k


@pytest.mark.parametrize("T", [256, 2048])
@pytest.mark.parametrize("fam", ["powerlaw", "uniform", "banded", "block", "wide"])
def test_gpu_features_families(fam, T, oracle_lib):
    from sspmv_gb300 import lespmv as L
    from sspmv_gb300 import synth
    p = {"powerlaw": synth.powerlaw(40000, 1.8, 16.0, 20000, 0.05), "uniform": synth.uniform(30000, 24, 0.02),
         "banded": synth.banded(50000), "block": synth.block(30000, 4, 6000),
         "wide": synth.uniform(7000, 10, 0.1, num_cols=20000)}[fam]
    A = synth.generate(p, 5)
    F, arrs = L.features(L.csr_from_host(A), T, arrays=True)
    Fo, ao = oracle_lib.features(A, T)
    bad = compare(F, Fo)
    assert not bad, f"features differ (index, gpu, oracle): {bad[:5]}"
    for k in ao:
        assert np.array_equal(arrs[k], ao[k]), k


@pytest.mark.parametrize("T,X", [(256, 8), (64, 4), (2048, 4), (16, 8)])
@pytest.mark.parametrize("fam", ["powerlaw", "banded", "block", "wide", "zeros"])
def test_gpu_grx_features_match_oracle(fam, T, X, oracle_lib):
    from sspmv_gb300 import lespmv as L
    from sspmv_gb300 import synth
    p = {"powerlaw": synth.powerlaw(6000, 1.8, 16.0, 3000, 0.05), "banded": synth.banded(8000, (0, 1, -1, 2, 5, -9)),
         "block": synth.block(6000, 4, 1500), "wide": synth.uniform(3000, 10, 0.1, num_cols=9000),
         "zeros": synth.block(4000, 8, 300)}[fam]
    A = synth.generate(p, 5)
    if fam == "zeros":
        A.values[::7] = 0.0  # explicit zeros are absent entries
    g = L.grx_features(L.csr_from_host(A), T, X)
    o = oracle_lib.grx(A, T, X)
    assert np.array_equal(g, o), f"gpu {g} oracle {o}"
