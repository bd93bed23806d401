import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parent.parent
if str(ROOT) not in sys.path:
    sys.path.insert(0, str(ROOT))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (runs the engine's kernels)")


@pytest.fixture(scope="session")
def oracle_lib():
    from oracle import pm_oracle
    pm_oracle.build()
    return pm_oracle


@pytest.fixture(scope="session")
def engine_lib():
    from patchmatch_cuda_gb300 import _native
    return _native.load_engine()


@pytest.fixture(scope="session")
def parity_log():
    """Records measured parity figures; written as JSON to $PM_PARITY_LOG when set."""
    import json
    import os
    records = {}

    def log(name, **values):
        records[name] = values

    yield log
    path = os.environ.get("PM_PARITY_LOG")
    if path and records:
        with open(path, "w") as f:
            json.dump(records, f, indent=1, sort_keys=True)
