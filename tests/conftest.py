import os
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden"))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (run with -m gpu)")
    # temporary files of the tests stay inside the repository
    if not config.option.basetemp:
        config.option.basetemp = os.path.join(ROOT, "tests", ".tmp")
    config.addinivalue_line("markers", "slow: long-running (large sizes)")
