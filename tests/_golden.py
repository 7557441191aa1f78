"""Loads tests/golden/golden.json and the helper functions of make_golden.py."""
import importlib.util
import json
from pathlib import Path

HERE = Path(__file__).resolve().parent
GOLDEN = json.loads((HERE / "golden" / "golden.json").read_text())
_spec = importlib.util.spec_from_file_location("make_golden", HERE / "golden" / "make_golden.py")
mg = importlib.util.module_from_spec(_spec)
_spec.loader.exec_module(mg)
