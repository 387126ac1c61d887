"""CPU-only checks of the C ABI: the library loads, exports every entry point
include/sspmv.h declares, and its host utilities (Matrix Market IO, seeded
generator) behave as the reference's do.  No device calls."""
import ctypes as C
import re
from pathlib import Path

import numpy as np
import pytest

from sspmv_gb300 import _lib, synth
from sspmv_gb300.lespmv import read_csr_matrix, write_mtx

ROOT = Path(__file__).resolve().parents[1]


def declared_functions():
    names = set()
    for h in (ROOT / "include").glob("*.h"):
        text = re.sub(r"/\*.*?\*/", "", h.read_text(), flags=re.S)
        for m in re.finditer(r"\b(sspmv_\w+)\s*\(", text):
            names.add(m.group(1))
    return sorted(names)


def test_every_declared_symbol_is_exported():
    names = declared_functions()
    assert len(names) > 10
    missing = [n for n in names if not hasattr(_lib.lib, n)]
    assert not missing, f"declared but not exported: {missing}"


def test_status_strings():
    assert _lib.lib.sspmv_status_string(0) == b"SSPMV_OK"
    assert _lib.lib.sspmv_status_string(2) == b"SSPMV_INFEASIBLE"
    assert b"sm_103a" in _lib.lib.sspmv_version()


def test_synth_deterministic_and_sorted():
    for p in (synth.powerlaw(5000, 1.8, 16, 3000, 0.05), synth.uniform(3000, 32), synth.block(2000, 4, 300),
              synth.banded(5000), synth.laplacian2d(20)):
        a = synth.generate(p, 9)
        b = synth.generate(p, 9)
        assert np.array_equal(a.row_offset, b.row_offset) and np.array_equal(a.col_index, b.col_index)
        assert np.array_equal(a.values, b.values)
        for i in range(0, a.num_rows, max(1, a.num_rows // 50)):
            c = a.col_index[a.row_offset[i]:a.row_offset[i + 1]]
            assert np.all(np.diff(c) > 0), "columns must be strictly ascending"
        f32 = synth.generate(p, 9, np.float32)
        assert np.array_equal(f32.values, a.values.astype(np.float32))


def test_laplacian_shape():
    a = synth.generate(synth.laplacian2d(1024))
    assert a.num_rows == 1_048_576 and a.nnz == 5_238_784


def test_mtx_round_trip(tmp_path):
    a = synth.generate(synth.powerlaw(2000, 1.8, 16, 500, 0.1), 3)
    path = tmp_path / "m.mtx"
    write_mtx(path, a)
    b = read_csr_matrix(path, 64)
    assert np.array_equal(a.row_offset, b.row_offset) and np.array_equal(a.col_index, b.col_index)
    assert np.array_equal(a.values, b.values)
    b32 = read_csr_matrix(path, 32)
    assert np.array_equal(b32.values, a.values.astype(np.float32))


def test_mtx_symmetric_and_pattern_match_reference(tmp_path):
    ref = pytest.importorskip("oracle").Reference
    try:
        R = ref()
    except ImportError:
        pytest.skip("reference harness not built (no reference sources on this host)")
    p = tmp_path / "s.mtx"
    p.write_text("%%MatrixMarket matrix coordinate pattern symmetric\n% c\n5 5 6\n1 1\n2 1\n3 2\n5 5\n4 2\n5 3\n")
    mine = read_csr_matrix(p, 64)
    theirs = R.read_csr(p, np.float64)
    assert np.array_equal(mine.row_offset, theirs["row_offset"])
    assert np.array_equal(mine.col_index, theirs["col"])
    assert np.array_equal(mine.values, theirs["val"])


def test_mtx_errors_are_statuses(tmp_path):
    p = tmp_path / "bad.mtx"
    p.write_text("%%MatrixMarket matrix array real general\n2 2\n1\n2\n3\n4\n")
    with pytest.raises(_lib.SSPMVError) as e:
        read_csr_matrix(p)
    assert e.value.status == 7
    with pytest.raises(_lib.SSPMVError):
        read_csr_matrix(tmp_path / "missing.mtx")


def test_torch_operator_is_registered():
    import torch
    import sspmv_gb300.torch_ops  # noqa: F401
    assert hasattr(torch.ops.sspmv, "spmv_csr")
