"""Readout-error branching for exact outcome probabilities (``simulator.py:445-486``).

The probabilities come from the device; the marginal over measured qubits and the expansion
over every combination of readout flips (2^pairs branches per outcome at most) are host work on
a vector of 2^m entries.
"""

from __future__ import annotations

from typing import Any

import numpy as np


def marginal(probs: np.ndarray, n: int, qubits: list[int]) -> np.ndarray:
    """Probabilities of ``qubits`` alone; index bit i is the i-th smallest (``engines.py:267-275``)."""
    keep = sorted(qubits)
    if n == 0:
        return probs
    drop = tuple(n - 1 - q for q in range(n) if q not in keep)
    t = probs.reshape([2] * n)
    return np.asarray(t.sum(axis=drop) if drop else t).reshape(-1)


def branch_outcomes(probs: np.ndarray, n: int, measured: list[int], pairs: list[tuple[int, int]], noise: Any,
                    threshold: float) -> dict[int, float]:  # fmt: skip
    position = {q: i for i, q in enumerate(measured)}
    dist = marginal(probs, n, measured)
    out: dict[int, float] = {}
    for index in np.flatnonzero(dist > threshold):
        branches = [(0, float(dist[index]))]
        for q, c in pairs:
            bit = (int(index) >> position[q]) & 1
            err = noise.readout_error(q) if noise else None
            flip = (err.p10 if bit else err.p01) if err is not None else 0.0
            grown = []
            for bits, w in branches:
                if flip < 1:
                    grown.append((bits | (bit << c), w * (1 - flip)))
                if flip > 0:
                    grown.append((bits | ((bit ^ 1) << c), w * flip))
            branches = grown
        for bits, w in branches:
            out[bits] = out.get(bits, 0.0) + w
    return out
