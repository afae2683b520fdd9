"""Loads tests/golden/make_golden.py (the fixture recipe) as a module so the
tests regenerate exactly the fixture inputs."""
import importlib.util
import os

_spec = importlib.util.spec_from_file_location(
    "make_golden", os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "make_golden.py"))
make_golden = importlib.util.module_from_spec(_spec)
_spec.loader.exec_module(make_golden)

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
