import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parents[1]
for p in (ROOT, ROOT / "oracle"):
    if str(p) not in sys.path:
        sys.path.insert(0, str(p))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")
    # Build the in-tree library and the oracle when they are missing.
    from sspmv_gb300 import build as _b
    if not _b.LIB.exists():
        _b.build_library()
    if not _b.SYNTH_LIB.exists():
        _b.build_synth()
    if not (ROOT / "oracle" / "liboracle.so").exists():
        _b.build_oracle(with_reference=False)


GOLDEN = ROOT / "tests" / "golden"


def golden_files():
    return sorted(GOLDEN.glob("*.npz"))


@pytest.fixture(scope="session")
def oracle_lib():
    from oracle import Oracle
    return Oracle()
