"""Dynamic Clifford circuits, one tableau per shot (``stabilizer.py:653-694``)."""

from __future__ import annotations

from typing import Any

import numpy as np

from lucivant_sim_gb300._lib import SimulationError


def per_shot(circuit: Any, shots: int, noise: Any, rng: np.random.Generator) -> dict[int, int]:
    raise SimulationError("dynamic Clifford circuits are not on the device engine yet; use method='trajectories'")
