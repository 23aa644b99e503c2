"""Shared test set-up: the ``gpu`` marker, the repository on ``sys.path``, golden fixtures."""

from __future__ import annotations

import json
import sys
from pathlib import Path

import numpy as np
import pytest

ROOT = Path(__file__).resolve().parents[1]
if str(ROOT) not in sys.path:
    sys.path.insert(0, str(ROOT))
GOLDEN = Path(__file__).resolve().parent / "golden"


def pytest_configure(config: pytest.Config) -> None:
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU and the built engine library")


@pytest.fixture(scope="session")
def golden() -> dict:
    return json.loads((GOLDEN / "golden.json").read_text())["cases"]


@pytest.fixture(scope="session")
def golden_arrays() -> dict:
    with np.load(GOLDEN / "golden.npz") as data:
        return {k: data[k] for k in data.files}
