"""The benchmark's measurement probes (lib/libsspmv_probe.so): the random-
gather kernel's checksum equals the same sum taken on the host, and the FP64
FMA rate is positive."""
import sys
from pathlib import Path

import numpy as np
import pytest

sys.path.insert(0, str(Path(__file__).resolve().parents[1]))
import bench  # noqa: E402

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("dt", [np.float64, np.float32])
def test_gather_ceiling_checksum(dt):
    """The gather-ceiling kernel gathers x[h(i) mod n] for a splitmix64 mix h
    of i: its checksum equals the same sum taken on the host."""
    n, count = 1000, 256 * 4000
    rate, chk = bench.Probes().gather_ceiling(dt, n, count)
    z = np.arange(count, dtype=np.uint64) + np.uint64(12345) + np.uint64(0x9E3779B97F4A7C15)
    z = (z ^ (z >> np.uint64(30))) * np.uint64(0xBF58476D1CE4E5B9)
    z = (z ^ (z >> np.uint64(27))) * np.uint64(0x94D049BB133111EB)
    z ^= z >> np.uint64(31)
    idx = (z % np.uint64(n)).astype(np.int64)
    x = (1.0 + (np.arange(n) % 7) * 0.125).astype(dt)
    ref = float(x[idx].astype(np.float64).sum())
    assert rate > 0
    assert abs(chk - ref) <= 1e-6 * ref


def test_fp64_ceiling_positive():
    assert bench.Probes().fp64_ceiling() > 1e9


def test_stream_ceiling_scales_with_bytes():
    """A plain stream of 4x the bytes takes longer, and no stream beats the
    measured HBM peak by more than the burst margin."""
    import json
    p = bench.Probes()
    small = p.stream_ceiling_ms(64 << 20, 8 << 20)
    large = p.stream_ceiling_ms(256 << 20, 32 << 20)
    assert 0 < small < large
    peak = json.loads((bench.ROOT / "MEASURED_PEAKS.json").read_text())["hbm_gbs"] \
        if (bench.ROOT / "MEASURED_PEAKS.json").exists() else 6800.0
    assert (288 << 20) / (large * 1e-3) / 1e9 < 1.3 * peak
