"""Host-side body storage, struct of arrays (mirrors the reference's Bodies, src/bodies.hpp:7-35).

Positions, velocities and masses are float32 at this boundary, as in the reference; the engine
widens positions to FP64 on upload. ``id`` is the stable identity: the engine reorders bodies (the
tree method sorts them by Morton key), so anything that tracks a body goes through ``id``.
"""
from __future__ import annotations

from dataclasses import dataclass, field

import numpy as np

_FIELDS = ("x", "y", "z", "vx", "vy", "vz", "m")


@dataclass
class Bodies:
    x: np.ndarray = field(default_factory=lambda: np.zeros(0, np.float32))
    y: np.ndarray = field(default_factory=lambda: np.zeros(0, np.float32))
    z: np.ndarray = field(default_factory=lambda: np.zeros(0, np.float32))
    vx: np.ndarray = field(default_factory=lambda: np.zeros(0, np.float32))
    vy: np.ndarray = field(default_factory=lambda: np.zeros(0, np.float32))
    vz: np.ndarray = field(default_factory=lambda: np.zeros(0, np.float32))
    m: np.ndarray = field(default_factory=lambda: np.zeros(0, np.float32))
    id: np.ndarray = field(default_factory=lambda: np.zeros(0, np.uint32))

    def __post_init__(self) -> None:
        for f in _FIELDS:
            setattr(self, f, np.ascontiguousarray(getattr(self, f), dtype=np.float32))
        self.id = np.ascontiguousarray(self.id, dtype=np.uint32)
        n = self.x.shape[0]
        for f in _FIELDS + ("id",):
            if getattr(self, f).shape != (n,):
                raise ValueError(f"Bodies.{f} must have shape ({n},)")

    def __len__(self) -> int:
        return int(self.x.shape[0])

    size = __len__

    @classmethod
    def empty(cls, n: int) -> "Bodies":
        z = lambda: np.zeros(n, np.float32)  # noqa: E731
        return cls(z(), z(), z(), z(), z(), z(), z(), np.zeros(n, np.uint32))

    @classmethod
    def from_arrays(cls, pos, vel, m, ids=None) -> "Bodies":
        """Rounds FP64 columns to float32, numbering ids 0..n-1 unless given (Bodies::push)."""
        pos = np.asarray(pos, dtype=np.float64)
        vel = np.asarray(vel, dtype=np.float64)
        n = pos.shape[0]
        ids = np.arange(n, dtype=np.uint32) if ids is None else ids
        return cls(pos[:, 0], pos[:, 1], pos[:, 2], vel[:, 0], vel[:, 1], vel[:, 2],
                   np.broadcast_to(np.asarray(m, np.float64), (n,)), ids)

    def subset(self, sel) -> "Bodies":
        """The bodies a boolean mask or index array selects, ids kept."""
        return Bodies(*(getattr(self, f)[sel] for f in _FIELDS), self.id[sel])

    def copy(self) -> "Bodies":
        return Bodies(*(getattr(self, f).copy() for f in _FIELDS + ("id",)))

    def append(self, other: "Bodies", renumber: bool = True) -> "Bodies":
        out = Bodies(*(np.concatenate([getattr(self, f), getattr(other, f)]) for f in _FIELDS + ("id",)))
        if renumber:
            out.id = np.arange(len(out), dtype=np.uint32)
        return out

    def pos64(self) -> np.ndarray:
        return np.stack([self.x, self.y, self.z], axis=1).astype(np.float64)

    def vel64(self) -> np.ndarray:
        return np.stack([self.vx, self.vy, self.vz], axis=1).astype(np.float64)
