import os
import sys

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
# The reference checkout only exists where fixtures are regenerated; tests that
# need it are skipped elsewhere.
REFERENCE_DIR = os.environ.get("VISOR_REFERENCE_DIR", "/root/reference")

if REPO not in sys.path:
    sys.path.insert(0, REPO)
TESTS = os.path.dirname(os.path.abspath(__file__))
if TESTS not in sys.path:
    sys.path.insert(0, TESTS)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")
