import json
import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (sm_103a) and the built extension")


@pytest.fixture(scope="session")
def reference_cases():
    """The reference's own unit-case inputs, read from its test sources at run time
    (skipped where the reference tree is absent)."""
    sys.path.insert(0, os.path.join(ROOT, "tests", "golden"))
    try:
        import make_reference_fixtures as mrf
    finally:
        sys.path.pop(0)
    root = os.environ.get("MEDYAN_REFERENCE_ROOT", mrf.DEFAULT_ROOT)
    if not mrf.available(root):
        pytest.skip("reference tree not present: its unit cases are read from its sources at test time")
    return json.loads(json.dumps(mrf.extract(root)))
