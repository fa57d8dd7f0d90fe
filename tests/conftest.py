import json
import sys
from pathlib import Path

import numpy as np
import pytest

ROOT = Path(__file__).resolve().parents[1]
if str(ROOT) not in sys.path:
    sys.path.insert(0, str(ROOT))

GOLDEN = ROOT / "tests" / "golden"


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA device (GB300); runs through the C ABI")


def load_golden(name: str):
    return np.load(GOLDEN / f"{name}.npz")


def params_from_json(js):
    from axions_gb300.params import make_params
    d = json.loads(str(js))
    p = make_params(d["model"])
    for k, v in d.items():
        setattr(p, k, v)
    return p


@pytest.fixture(scope="session")
def oracle_mod():
    from oracle import oracle as O
    O.lib()
    return O
