"""Comparison helpers shared by the test modules."""
from __future__ import annotations

import numpy as np


def rel_l2(a, b) -> float:
    a = np.asarray(a, dtype=np.float64)
    b = np.asarray(b, dtype=np.float64)
    den = np.linalg.norm(b)
    return float(np.linalg.norm(a - b) / (den if den > 0 else 1.0))


def copy_arrays(arrays: dict) -> dict:
    return {k: v.copy() for k, v in arrays.items()}
