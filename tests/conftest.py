import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300); runs the kernels through the C ABI")


@pytest.fixture(scope="session")
def golden_solar():
    import json
    with open(os.path.join(ROOT, "tests", "golden", "solar_tester.json")) as f:
        return json.load(f)


@pytest.fixture(scope="session")
def golden_obsgeo():
    import json
    with open(os.path.join(ROOT, "tests", "golden", "obsgeo_lpcs.json")) as f:
        return json.load(f)


@pytest.fixture(scope="session")
def golden_iqu():
    import json
    with open(os.path.join(ROOT, "tests", "golden", "solar_tester_iqu.json")) as f:
        return json.load(f)
