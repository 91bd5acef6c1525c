"""Shared test configuration.

Tests marked ``gpu`` need a CUDA device and the built library; everything
else runs on the CPU.  The oracle (oracle/) is the checker for parity tests.
"""
import sys
from pathlib import Path

ROOT = Path(__file__).resolve().parents[1]
if str(ROOT) not in sys.path:
    sys.path.insert(0, str(ROOT))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA device (GB300) and the built CUDA library")
    # Build the product library and the oracle before test modules are
    # collected (they import the package); a no-op when up to date.
    import __graft_entry__

    __graft_entry__.build()
