import os
import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parents[1]
if str(ROOT) not in sys.path:
    sys.path.insert(0, str(ROOT))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA device (GB300, sm_103a)")
    config.addinivalue_line("markers", "slow: longer CPU oracle runs")


@pytest.fixture(scope="session")
def golden():
    import json
    base = ROOT / "tests" / "golden"
    return {p.stem: json.loads(p.read_text()) for p in base.glob("*.json")}


def oracle_threads():
    return min(8, os.cpu_count() or 1)
