"""pytest configuration: the `gpu` marker and the import path.

Tests marked `gpu` need a GB300 (sm_103) and the in-tree libpsdgb.so; the
rest run on any CPU host."""
import os
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a GB300 GPU and the built libpsdgb.so")
