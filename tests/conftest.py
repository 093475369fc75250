import gzip
import os
import sys
import tempfile

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
GOLDEN = os.path.join(ROOT, "tests", "golden")
for p in (ROOT, os.path.join(ROOT, "oracle")):
    if p not in sys.path:
        sys.path.insert(0, p)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (sm_103a) and the built engine library")


def load_golden(name):
    """Load tests/golden/<name>.snap.gz as a State."""
    from code_mpm_gb300 import snapshot

    with gzip.open(os.path.join(GOLDEN, name + ".snap.gz"), "rb") as f:
        raw = f.read()
    with tempfile.NamedTemporaryFile(suffix=".snap") as t:
        t.write(raw)
        t.flush()
        return snapshot.load(t.name)


@pytest.fixture
def golden():
    return load_golden
