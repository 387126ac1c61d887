"""The benchmark_spmv_<fmt> programs: command line and output compatible
with the reference's test/benchmark_spmv_<fmt>.cpp (usage, argument errors
on the CPU; a run per format on the GPU appends the reference's
mat_perf.txt line)."""
import re
import subprocess

import numpy as np
import pytest

from sspmv_gb300 import build as B

# (format, mat_perf line pattern) -- the reference's fprintf layouts
NUM = r"-?\d+\.\d+"
LINES = {
    "csr": rf"^7 m CSR 2 0 +{NUM} {NUM} $",
    "coo": rf"^7 m COO 1 0 +{NUM} {NUM} {NUM} $",
    "ell": rf"^7 m ELL 2 0 +{NUM} {NUM} {NUM} $",
    "sell": rf"^7 m S-ELL 2 0 4 +{NUM} {NUM} {NUM} $",
    "sell_c_sigma": rf"^7 m S-ELL-sigma 2 0 4 16384 +{NUM} {NUM} {NUM} $",
    "sell_c_R": rf"^7 m S-ELL-R 2 0 4 +{NUM} {NUM} $",
    "dia": rf"^7 m DIA 1 0 +{NUM} {NUM} {NUM} $",
    "bsr": rf"^7 m BSR 2 0 +{NUM} {NUM} {NUM} $",
    "csr5": rf"^7 m CSR5 +{NUM} {NUM} $",
}


def _exe(fmt: str):
    B.build_library()
    B.build_cli()
    return str(B.BINDIR / f"benchmark_spmv_{fmt}")


def test_cli_help_and_argument_errors(tmp_path):
    r = subprocess.run([_exe("csr"), "--help"], capture_output=True, text=True)
    assert r.returncode == 0 and "Usage:" in r.stdout and "--precision" in r.stdout
    r = subprocess.run([_exe("csr"), "m.mtx", "--Index=1"], capture_output=True, text=True)
    assert r.returncode != 0 and "not supported" in r.stderr
    r = subprocess.run([_exe("csr"), "--precision=64"], capture_output=True, text=True)
    assert r.returncode != 0 and "You need to input a matrix file!" in r.stdout
    r = subprocess.run([str(B.BINDIR / "benchmark_spmv"), "m.mtx"], capture_output=True, text=True)
    assert r.returncode != 0 and "unknown format" in r.stderr


@pytest.mark.gpu
@pytest.mark.parametrize("precision", [64, 32])
@pytest.mark.parametrize("fmt", list(LINES))
def test_cli_runs_and_appends_reference_line(tmp_path, fmt, precision):
    from sspmv_gb300 import synth
    from sspmv_gb300.lespmv import write_mtx
    A = synth.generate(synth.banded(3000, (0, 1, -1, 7, -7)), 3, np.float64)
    mtx = tmp_path / "m.mtx"
    write_mtx(str(mtx), A)
    (tmp_path / "performance").mkdir()
    r = subprocess.run([_exe(fmt), str(mtx), "--matID=7", f"--precision={precision}", "--iters=30"],
                       capture_output=True, text=True, cwd=tmp_path, timeout=300)
    assert r.returncode == 0, r.stdout + r.stderr
    assert f"Using 3000-by-3000 matrix with {A.nnz} nonzero values" in r.stdout
    # the reference's own verdict thresholds: 5 sqrt(eps) "small round-error", 0.005 "failure"
    err = float(re.search(r"\[max error +([0-9.eE+-]+)\]", r.stdout).group(1))
    assert err < 5 * np.sqrt(np.finfo(np.float64 if precision == 64 else np.float32).eps)
    assert "FAILURE" not in r.stdout and "Round-Error" not in r.stdout
    assert "Performing 30 iterations" in r.stdout
    line = (tmp_path / "performance" / "mat_perf.txt").read_text().splitlines()[-1] + "\n"
    assert re.match(LINES[fmt], line.rstrip("\n")), repr(line)


def test_bench_selects_one_case():
    """One case of the benchmark (the profiling command of profiles/) is
    selected by arguments alone: family, format, precision, sections."""
    import sys
    from pathlib import Path
    sys.path.insert(0, str(Path(__file__).resolve().parents[1]))
    import bench
    a = bench.parse_args(["--families", "banded_2M", "--formats", "csr", "--dtypes", "f32", "--steps", "1",
                          "--warmup", "3", "--sections", "suite", "--no-cpu", "--no-e2e"])
    assert (a.families, a.formats, a.dtypes, a.steps) == ("banded_2M", "csr", "f32", 1)
    assert bench.sections(a) == {"suite"}
    assert bench.sections(bench.parse_args([])) == {"suite", "laplacian", "large", "serving"}
    assert bench.sections(bench.parse_args(["--no-serving", "--no-large"])) == {"suite"}
