"""Regenerates the inputs of the golden cases (same generators as make_golden.py)."""
from __future__ import annotations

import json
import sys
from pathlib import Path

HERE = Path(__file__).resolve().parent
sys.path.insert(0, str(HERE / "golden"))

from make_golden import inputs as golden_inputs  # noqa: E402,F401


def golden_cases() -> list[dict]:
    return json.loads((HERE / "golden" / "golden.json").read_text())
