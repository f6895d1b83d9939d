import json
import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
PKG = os.path.join(ROOT, "erdos-selfridge_gb300")
ORACLE = os.path.join(ROOT, "oracle")
GOLDEN = os.path.join(ROOT, "tests", "golden")
for p in (PKG, ORACLE):
    if p not in sys.path:
        sys.path.insert(0, p)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a GB300 (sm_103a) GPU and the built engine library")


def golden(name: str):
    with open(os.path.join(GOLDEN, name)) as f:
        return json.load(f)


@pytest.fixture(scope="session")
def bfile():
    g = golden("bfile.json")
    return {int(k): int(v) for k, v in g["g"].items()}


def gpu_available() -> bool:
    try:
        import es_native
        es_native.device_info()
        return True
    except Exception:
        return False


@pytest.fixture(scope="session")
def native():
    import es_native
    info = es_native.device_info()          # raises if the library or device is missing
    assert info["cc"] == (10, 3), f"expected an sm_103 device, got {info}"
    return es_native
