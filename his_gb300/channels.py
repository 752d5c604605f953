"""1-D channel network description, with the reference's vocabulary
(hydrointel/domain/channels.py:19-91, :172-193).

A network is a set of reaches, each ordered upstream -> downstream, joined at
junction nodes.  A reach end is ``("inflow",)``, ``("stage",)``, ``("closed",)``
or ``("junction", j)``.  This is the input format of the 1-D network kernel.
"""
from __future__ import annotations

import dataclasses
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

    def problems(self):
        """Yield a message for every rule the network breaks: per-node fields of each
        reach with the node count and finite; positive width and roughness, side
        slopes >= 0; bank crest >= bed + 0.2 m; reach ends of a known kind, naming an
        existing junction (hydrointel/domain/channels.py:77-94)."""
        end_kinds = ("inflow", "stage", "closed", "junction")
        for r in self.reaches:
            nodes = np.shape(r.x)
            fields = {name: np.asarray(getattr(r, name), dtype=float) for name in _NODE_FIELDS}
            broken = [n for n, a in fields.items() if a.shape != nodes or not np.isfinite(a).all()]
            for name in broken:
                yield f"reach {r.reach_id}: field '{name}' has bad shape or non-finite values"
            if broken:
                continue
            if (fields["width"] <= 0).any() or (fields["manning"] <= 0).any() or (fields["side_slope"] < 0).any():
                yield f"reach {r.reach_id}: width/manning must be > 0 and side_slope >= 0"
            if ((fields["z_bank"] - fields["bed"]) < 0.2).any():
                yield f"reach {r.reach_id}: bank crest must be at least 0.2 m above bed"
            for end in (r.up, r.down):
                if end[0] not in end_kinds:
                    yield f"reach {r.reach_id}: unknown boundary kind {end[0]}"
                elif end[0] == "junction" and not 0 <= end[1] < len(self.junctions):
                    yield f"reach {r.reach_id}: junction index {end[1]} out of range"

    def validate(self) -> None:
        """Raise ValueError with the first problem found (``problems``)."""
        for msg in self.problems():
            raise ValueError(msg)


_NODE_FIELDS = ("bed", "width", "side_slope", "manning", "z_bank")


def apply_gamma(net: ChannelNetwork, gamma) -> ChannelNetwork:
    """A copy of ``net`` with each reach's conveyance scaled by its gamma: with
    s = sqrt(gamma), the bottom width becomes s times wider and the depth below the
    fixed bank crest s times deeper, so a rectangular bankfull area scales by gamma
    while the 2-D terrain is untouched.  A junction is rescaled the same way by every
    reach that ends at it, in reach order (hydrointel/domain/channels.py:172-193)."""
    g = np.asarray(gamma, dtype=float).reshape(-1)
    if g.size != net.n_reaches:
        raise ValueError(f"channel_gamma has {g.size} entries, network has {net.n_reaches} reaches")
    if (g <= 0).any():
        raise ValueError("channel_gamma must be positive")
    s = np.sqrt(g)
    deepen = lambda crest, bed, f: crest - (crest - bed) * f
    reaches = [dataclasses.replace(r, width=r.width * f, bed=deepen(r.z_bank, r.bed, f))
               for r, f in zip(net.reaches, s)]
    junctions = [dataclasses.replace(j) for j in net.junctions]
    for r, f in zip(net.reaches, s):
        if r.down[0] == "junction":
            j = junctions[r.down[1]]
            j.width, j.bed = j.width * f, deepen(j.z_bank, j.bed, f)
    out = ChannelNetwork(reaches, junctions, net.inflow_reach)
    out.validate()
    return out
