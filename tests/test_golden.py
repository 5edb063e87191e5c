"""The CPU oracle reproduces its committed golden vectors (tests/golden/)."""
from pathlib import Path

import numpy as np
import pytest

GOLDEN = Path(__file__).resolve().parent / "golden" / "oracle_small.npz"


def test_oracle_matches_golden():
    import importlib.util
    spec = importlib.util.spec_from_file_location("make_golden", GOLDEN.parent / "make_golden.py")
    mg = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mg)
    ref = np.load(GOLDEN)
    got = mg.cases()
    assert set(got) == set(ref.files)
    for k in ref.files:
        a, b = got[k], ref[k]
        scale = max(1.0, float(np.max(np.abs(b))))
        assert np.max(np.abs(a - b)) <= 1e-13 * scale, k
