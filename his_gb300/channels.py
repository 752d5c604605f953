"""1-D channel network description, with the reference's vocabulary
(hydrointel/domain/channels.py:19-91, :172-193).

A network is a set of reaches, each ordered upstream -> downstream, joined at
junction nodes.  A reach end is ``("inflow",)``, ``("stage",)``, ``("closed",)``
or ``("junction", j)``.  This is the input format of the 1-D network kernel.
"""
from __future__ import annotations

import copy
from dataclasses import dataclass, field

import numpy as np


@dataclass
class Reach:
    reach_id: str
    x: np.ndarray
    y: np.ndarray
    bed: np.ndarray
    width: np.ndarray
    side_slope: np.ndarray
    manning: np.ndarray
    z_bank: np.ndarray
    up: tuple = ("inflow",)
    down: tuple = ("stage",)

    @property
    def n(self) -> int:
        return len(self.x)

    @property
    def spacing(self) -> np.ndarray:
        """Cell length per node: half the distance to each neighbour; ends use one side."""
        if self.n == 1:
            return np.array([1.0])
        d = np.hypot(np.diff(self.x), np.diff(self.y))
        ds = np.empty(self.n)
        ds[0], ds[-1] = d[0], d[-1]
        ds[1:-1] = 0.5 * (d[:-1] + d[1:])
        return ds

    @property
    def chainage(self) -> np.ndarray:
        return np.concatenate([[0.0], np.cumsum(np.hypot(np.diff(self.x), np.diff(self.y)))])


@dataclass
class Junction:
    x: float
    y: float
    bed: float
    width: float
    side_slope: float
    manning: float
    z_bank: float
    length: float


@dataclass
class ChannelNetwork:
    reaches: list = field(default_factory=list)
    junctions: list = field(default_factory=list)
    inflow_reach: str | None = None

    @property
    def n_reaches(self) -> int:
        return len(self.reaches)

    def validate(self) -> None:
        for r in self.reaches:
            for name in ("bed", "width", "side_slope", "manning", "z_bank"):
                a = np.asarray(getattr(r, name))
                if a.shape != np.asarray(r.x).shape or not np.all(np.isfinite(a)):
                    raise ValueError(f"reach {r.reach_id}: field '{name}' has bad shape or non-finite values")
            if np.any(r.width <= 0) or np.any(r.side_slope < 0) or np.any(r.manning <= 0):
                raise ValueError(f"reach {r.reach_id}: width/manning must be > 0 and side_slope >= 0")
            if np.any(r.z_bank - r.bed < 0.2):
                raise ValueError(f"reach {r.reach_id}: bank crest must be at least 0.2 m above bed")
            for end in (r.up, r.down):
                if end[0] not in ("inflow", "stage", "closed", "junction"):
                    raise ValueError(f"reach {r.reach_id}: unknown boundary kind {end[0]}")
                if end[0] == "junction" and not 0 <= end[1] < len(self.junctions):
                    raise ValueError(f"reach {r.reach_id}: junction index {end[1]} out of range")


def apply_gamma(net: ChannelNetwork, gamma) -> ChannelNetwork:
    """Per-reach conveyance scale: bottom width and bankfull depth both times sqrt(gamma),
    the bed moved about the fixed bank crest; a junction takes the factor of each reach
    that ends at it."""
    g = np.asarray(gamma, dtype=float).reshape(-1)
    if g.size != net.n_reaches:
        raise ValueError(f"channel_gamma has {g.size} entries, network has {net.n_reaches} reaches")
    if np.any(g <= 0):
        raise ValueError("channel_gamma must be positive")
    out = copy.deepcopy(net)
    for r, gi in zip(out.reaches, g):
        s = np.sqrt(gi)
        r.width = r.width * s
        r.bed = r.z_bank - (r.z_bank - r.bed) * s
        if r.down[0] == "junction":
            j = out.junctions[r.down[1]]
            j.width *= s
            j.bed = j.z_bank - (j.z_bank - j.bed) * s
    out.validate()
    return out
