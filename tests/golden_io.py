"""Loading helpers for the golden vectors in tests/golden/ (made by tests/golden/make_golden.py)."""
from __future__ import annotations

import glob
import os

import numpy as np

from lettuce_simulate_physics_gb300.bodies import Bodies

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def names(prefix: str = "") -> list[str]:
    return sorted(os.path.basename(p)[:-4] for p in glob.glob(os.path.join(GOLDEN, f"{prefix}*.npz")))


class Golden:
    def __init__(self, name: str):
        self.name = name
        self.z = dict(np.load(os.path.join(GOLDEN, f"{name}.npz")))

    def inputs(self) -> Bodies:
        z = self.z
        return Bodies(z["in_x"], z["in_y"], z["in_z"], z["in_vx"], z["in_vy"], z["in_vz"], z["in_m"], z["in_id"])

    def param(self, k):
        return self.z[f"param_{k}"].item()

    def cases(self) -> list[str]:
        return sorted({k.split("__")[0] for k in self.z if "__" in k})

    def case(self, c: str) -> dict:
        p = f"{c}__"
        return {k[len(p):]: v for k, v in self.z.items() if k.startswith(p)}


def by_id(order_id: np.ndarray, a: np.ndarray) -> np.ndarray:
    """Rows of a (k, n) array, in body order, re-indexed by id."""
    out = np.zeros_like(a)
    out[:, order_id] = a
    return out


def rel_rms(a: np.ndarray, ref: np.ndarray) -> float:
    num = float(((a.astype(np.float64) - ref) ** 2).sum())
    den = float((ref.astype(np.float64) ** 2).sum())
    return (num / den) ** 0.5 if den > 0 else num ** 0.5
