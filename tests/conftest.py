import json
import pathlib
import sys

import numpy as np
import pytest

ROOT = pathlib.Path(__file__).resolve().parents[1]
sys.path.insert(0, str(ROOT))
import __graft_entry__ as ge  # noqa: E402

GOLDEN = ROOT / "tests" / "golden"


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300); run with -m gpu")


@pytest.fixture(scope="session")
def pkg():
    return ge.load_package()


@pytest.fixture(scope="session")
def abi(pkg):
    return pkg.abi


@pytest.fixture(scope="session")
def O():
    mod = ge.load_oracle_module()
    if not mod.ORACLE_SO.exists():
        mod.build()
    return mod


@pytest.fixture(scope="session")
def oracle(O, abi):
    return O.Oracle(abi)


def model_from_dict(abi, d):
    m = abi.GbfModel()
    for k, v in d.items():
        if isinstance(v, list):
            getattr(m, k)[:] = v
        else:
            setattr(m, k, v)
    return m


def load_golden(abi, name):
    z = np.load(GOLDEN / name)
    return model_from_dict(abi, json.loads(str(z["model"]))), z


@pytest.fixture(scope="session")
def gpu_lib(pkg):
    """libgbflow.so on a CUDA device; skips (never falls back) without a GPU."""
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    return pkg.load_library(required=True)
