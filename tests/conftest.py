import json
import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

GOLDEN_DIR = os.path.join(ROOT, "tests", "golden")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (sm_103a); parity tests proper")
    config.addinivalue_line("markers", "slow: large sizes")


def pytest_collection_modifyitems(config, items):
    try:
        import torch

        has_gpu = torch.cuda.is_available()
    except Exception:  # pragma: no cover
        has_gpu = False
    if has_gpu:
        return
    skip = pytest.mark.skip(reason="no CUDA device")
    for item in items:
        if "gpu" in item.keywords:
            item.add_marker(skip)


@pytest.fixture(scope="session")
def golden():
    with open(os.path.join(GOLDEN_DIR, "golden.json")) as f:
        return json.load(f)


@pytest.fixture(scope="session")
def small_cases(golden):
    z = np.load(os.path.join(GOLDEN_DIR, "small_cases.npz"))
    out = {}
    for meta in golden["small_cases"]:
        name = meta["name"]
        case = dict(meta)
        for key in z.files:
            if key.startswith(name + "__"):
                case[key.split("__", 1)[1]] = z[key]
        out[name] = case
    return out
