import importlib
import json
import sys
from pathlib import Path

import numpy as np
import pytest

ROOT = Path(__file__).resolve().parents[1]
if str(ROOT) not in sys.path:
    sys.path.insert(0, str(ROOT))

GOLD = ROOT / "tests" / "golden"


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300); runs the CUDA library")


@pytest.fixture(scope="session")
def srn():
    pkg = importlib.import_module("stimuli-responsive-nanodroplets_gb300")
    from importlib import import_module
    build = import_module("stimuli-responsive-nanodroplets_gb300.build")
    build.build()
    return pkg


@pytest.fixture(scope="session")
def oracle_mod():
    from oracle import oracle
    return oracle


def load_golden(name):
    g = dict(np.load(GOLD / f"{name}.npz", allow_pickle=False))
    return g


def surface_from_json(srn, text):
    d = json.loads(str(text))
    s = srn.Surface()
    for k, v in d.items():
        setattr(s, k, v)
    return s


@pytest.fixture(scope="session")
def golden(srn):
    def get(name):
        g = load_golden(name)
        g["S"] = surface_from_json(srn, g["surface"])
        return g
    return get
