"""Access to the case table of tests/golden/make_golden.py for the tests."""
import importlib.util
from pathlib import Path

_spec = importlib.util.spec_from_file_location("make_golden", Path(__file__).resolve().parent / "golden" / "make_golden.py")
_mod = importlib.util.module_from_spec(_spec)
_spec.loader.exec_module(_mod)

CASES = _mod.CASES
build = _mod.build
