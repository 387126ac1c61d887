"""Helpers shared by the tests that read tests/golden/*.npz."""
from __future__ import annotations

import hashlib
import json
from pathlib import Path

import numpy as np

from sspmv_gb300.synth import HostCSR

GOLDEN = Path(__file__).resolve().parent / "golden"
ALPHA, BETA = 0.8, 0.7


def digest(a: np.ndarray) -> str:
    return hashlib.sha256(np.ascontiguousarray(a).tobytes()).hexdigest()


def load(path: Path):
    z = np.load(path)
    meta = json.loads(bytes(z["meta"]).decode())
    A = HostCSR(meta["num_rows"], meta["num_cols"], z["row_offset"], z["col_index"], z["values"])
    return z, meta, A


def files():
    return sorted(GOLDEN.glob("*.npz"))
