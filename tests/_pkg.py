"""Loads the engine package (directory qiskit-aer_gb300/) for the tests."""
import sys
from pathlib import Path

ROOT = Path(__file__).resolve().parents[1]
if str(ROOT) not in sys.path:
    sys.path.insert(0, str(ROOT))

import __graft_entry__ as _entry  # noqa: E402


def pkg():
    return _entry.load_package()
