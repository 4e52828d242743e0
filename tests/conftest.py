import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

GOLDEN = os.path.join(ROOT, "tests", "golden")
CASES = ("loop", "east", "cfg1")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")


def _lists(off, flat):
    return [flat[off[i]:off[i + 1]].astype(np.int32) for i in range(len(off) - 1)]


def load_golden(name: str) -> dict:
    z = np.load(os.path.join(GOLDEN, f"{name}.npz"))
    d = {k: z[k] for k in z.files}
    for k in ("op_cutset", "op_prev", "op_children"):
        d[k] = _lists(d.pop(k + "_off"), d.pop(k + "_flat"))
    for k in ("N", "F", "M", "K", "n_lod"):
        d[k] = int(d[k])
    return d


def golden_names():
    return [c for c in CASES if os.path.exists(os.path.join(GOLDEN, f"{c}.npz"))]


@pytest.fixture(params=CASES)
def golden(request):
    return load_golden(request.param)
