"""bench.py's result line: the compact headline stays a few KB whatever the
size of the detail record, keeps the contract keys, and summarises parity
per format x precision (max and median normalised error)."""
import json
import sys
from pathlib import Path

ROOT = Path(__file__).resolve().parents[1]
sys.path.insert(0, str(ROOT))


def _fake_out():
    fmts = ["csr", "coo", "ell", "sell", "sell_c_sigma", "sell_c_R", "dia", "bsr", "csr5"]
    fams = ["banded_2M", "powerlaw_4M", "block4_2M", "uniform_4M"]
    per = [{"family": f, "format": m, "dtype": d, "ms": 0.1 + i * 1e-3, "GBps": 3000.0 + i, "ref_model_GBps": 1.0,
            "csr_equiv_GBps": 1.0, "GFLOPs": 1.0, "kernel": {"kernel_flag": 0}, "max_norm_err": 0.1,
            "median_norm_err": 0.01}
           for i, (f, m, d) in enumerate((f, m, d) for f in fams for m in fmts for d in ("f64", "f32"))]
    sweep = [{"requests": 1000, "failed": 0, "req_per_s": 1e4 * i, "p50_us": 100.0, "p99_us": 900.0 + i,
              "mean_batch": 1.0, "offered_per_s": 1e4 * i} for i in range(30)]
    srv = {"saturation_ratio": {"per_request": 1.01, "per_request_serial": 2.4},
           "equal_p99": {"per_request": {"throughput_ratio": 0.5}, "per_request_serial": {"throughput_ratio": None}},
           "modes": {m: {"sweep": sweep} for m in ("batched", "per_request", "per_request_serial")},
           "formats": {f"m{i}": "csr" for i in range(64)}}
    return {
        "metric": "SpMV GB/s", "value": 2665.2, "unit": "GB/s", "n_gpus": 1, "steps": 20, "warmup": 5,
        "ms_per_step": 13.35, "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64+f32",
        "data": "synthetic", "config": {"workload": "spmv-suite", "skipped": ["x"] * 14, "l2": "flushed"},
        "e2e": {"value": 2500.0, "unit": "GB/s", "h2d_bytes_per_step": 1, "d2h_bytes_per_step": 2, "ms_per_step": 1.0,
                "copies": "a long description " * 10, "serial_value": 1400.0, "serial_ms_per_step": 2.0},
        "roofline": {"bound": "hbm", "achieved": 3530.7, "peak": 6692.8, "unit": "GB/s", "frac": 0.52,
                     "traffic": 123, "kernel": "uniform_4M/coo/f64", "algorithmic_bytes": 1, "peak_kind": "measured",
                     "gather_ceiling": {"frac": 0.74, "what": "w" * 300}},
        "cpu_baseline": {"value": 32.0, "unit": "GB/s", "cores": 16, "kind": "port", "sample": "s"},
        "clocks": {"sm_mhz": 2070, "sm_max_mhz": 2070, "reasons": []}, "gpu_launches": 565,
        "parity": {"within_tolerance": True, "max_norm_err": 0.06, "tolerance": "t",
                   "max_median_by_format": {f"{m}/{d}": [0.06, 0.001] for m in fmts for d in ("f64", "f32")}},
        "per_format": per,
        "laplacian_1024": {"cold_GBps": 3000.0, "cold_frac_of_measured_peak": 0.45, "cold_ms": 0.027,
                           "cold_in_stream_ms": 0.0185, "cold_in_stream_frac_of_measured_peak": 0.67,
                           "warm_GBps": 3700.0, "max_norm_err": 0.1, "median_norm_err": 0.01,
                           "kernel": {"kernel_flag": 4, "param": 8}},
        "large_powerlaw_16M": {"formats": {f: {f"k{k}": {"GBps": 2000.0, "max_norm_err": 0.05} for k in (1, 8)}
                                           for f in ("csr", "sell_c_sigma")}},
        "serving": {"host": srv, "device": srv},
    }


def test_headline_is_compact_and_complete():
    import bench
    out = _fake_out()
    assert len(json.dumps(out)) > 8000
    h = bench.headline(out)
    line = json.dumps(h, separators=(",", ":"))
    assert len(line) <= bench.HEADLINE_LIMIT
    for k in ("metric", "value", "unit", "n_gpus", "steps", "warmup", "ms_per_step", "higher_is_better",
              "dtype", "config", "e2e", "roofline", "cpu_baseline", "clocks", "gpu_launches", "parity"):
        assert k in h, k
    assert h["parity"]["max_median_by_format"]["csr/f64"] == [0.06, 0.001]
    assert h["e2e"]["h2d_bytes_per_step"] == 1
    assert h["serving"]["device"]["equal_p99_ratio"]["per_request"] == 0.5
    lap = h["laplacian_1024"]
    assert lap["cold_in_stream_frac_of_measured_peak"] == 0.67 and list(lap["kernel"]) == [4, 8]
    assert h["config"]["skipped"] == 14


def test_emit_prints_one_line_last_and_writes_detail(tmp_path, capsys):
    import argparse
    import bench
    out = _fake_out()
    args = argparse.Namespace(detail=str(tmp_path / "d.json"))
    bench.emit(out, args)
    lines = capsys.readouterr().out.strip().splitlines()
    assert len(lines) == 1 and lines[0].startswith("{")
    assert json.loads(lines[0])["value"] == 2665.2
    assert json.loads((tmp_path / "d.json").read_text())["per_format"][0]["family"] == "banded_2M"
