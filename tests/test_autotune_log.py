"""The autotuner's append-only result log: a restarted tuning run reads the
records already written and skips their keys (no GPU needed)."""
import json
import sys
from pathlib import Path

ROOT = Path(__file__).resolve().parents[1]
sys.path.insert(0, str(ROOT))


def test_append_and_resume(tmp_path):
    from sspmv_gb300 import autotune
    log = tmp_path / "tune.jsonl"
    assert autotune.load_log(log) == {}
    autotune.append_log(log, "banded_2M/csr/f64", {"best": {"kernel_flag": 1, "param": 2, "ms": 0.06}})
    autotune.append_log(log, "powerlaw_4M/csr/f64", {"best": {"kernel_flag": 0, "param": 0, "ms": 0.4}})
    done = autotune.load_log(log)
    assert set(done) == {"banded_2M/csr/f64", "powerlaw_4M/csr/f64"}
    assert done["banded_2M/csr/f64"]["best"]["param"] == 2
    # a resumed run tunes only the keys not in the log
    todo = [k for k in ("banded_2M/csr/f64", "uniform_4M/csr/f64", "powerlaw_4M/csr/f64") if k not in done]
    assert todo == ["uniform_4M/csr/f64"]
    autotune.append_log(log, todo[0], {"best": {"kernel_flag": 1, "param": 8, "ms": 0.58}})
    lines = [json.loads(s) for s in log.read_text().splitlines()]
    assert [r["key"] for r in lines] == ["banded_2M/csr/f64", "powerlaw_4M/csr/f64", "uniform_4M/csr/f64"]
    # a later record of the same key wins
    autotune.append_log(log, "banded_2M/csr/f64", {"best": {"kernel_flag": 3, "param": 1024, "ms": 0.05}})
    assert autotune.load_log(log)["banded_2M/csr/f64"]["best"]["kernel_flag"] == 3


def test_candidates_cover_the_reference_macros():
    """The candidate sets include the reference's compile-time defaults."""
    from sspmv_gb300 import autotune
    cs = autotune.conversion_candidates("sell_c_sigma", 1 << 20)
    assert dict(slicewidth=0, chunkwidth=0, alignment=0) in cs  # SELL_SIGMA / CHUNK_SIZE defaults
    assert any(c["chunkwidth"] == 32 and c["slicewidth"] == 1 << 20 for c in cs)
    assert dict(sigma=0, omega=0) in autotune.conversion_candidates("csr5", 1000)  # CSR5_SIGMA default
    assert (0, 0) in autotune.CSR_CANDIDATES


def test_csr_candidates_cover_every_kernel_and_param():
    """The CSR candidates the tuner times cover every kernel_flag the library
    has (0 stream, 1 vector, 2 merge-path, 3 row-block, 4 pipelined) and, for
    the pipelined kernel, every param (bit 0 value-load point, bits 1-2 lanes
    per row, bit 3 CTA size); each (flag, param) once."""
    from sspmv_gb300 import autotune
    cands = autotune.CSR_CANDIDATES
    assert len(cands) == len(set(cands))
    assert {f for f, _ in cands} == {0, 1, 2, 3, 4}
    assert {p for f, p in cands if f == 4} == set(range(16))
    assert {p for f, p in cands if f == 1} == {1, 2, 4, 8, 16, 32}
    assert {p for f, p in cands if f == 3} == {512, 1024, 2048, 4096}
    assert autotune.KERNEL_CANDIDATES["csr"] is cands
