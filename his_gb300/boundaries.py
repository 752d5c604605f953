"""Edge boundary conditions of the 2-D grid, with the reference's vocabulary
(hydrointel/solver/boundaries.py:25-53).

Edges are ``("west", "east", "south", "north")``; row 0 is the south edge and
column 0 the west edge.  Kinds:

* ``closed``        wall: mirrored ghost layers, normal velocity reversed
* ``transmissive``  zero gradient: mirrored ghost layers
* ``stage``         imposed water level eta(t); outgoing Riemann invariant,
                    zero-gradient when the outflow is supercritical
* ``discharge``     imposed inflow per unit width q(t) [m^2/s], positive into
                    the domain, at critical depth over a dry edge

The ghost construction itself runs inside the CUDA stencil kernels; this module
only carries the edge kinds and evaluates their values on the host.
"""
from __future__ import annotations

from dataclasses import dataclass
from typing import Callable

import numpy as np

EDGES = ("west", "east", "south", "north")
KINDS = ("closed", "transmissive", "stage", "discharge")
KIND_CODE = {k: i for i, k in enumerate(KINDS)}


@dataclass
class EdgeBC:
    kind: str = "transmissive"
    value: float | Callable[[float], float] | None = None

    def __post_init__(self):
        if self.kind not in KINDS:
            raise ValueError(f"unknown boundary kind '{self.kind}'")
        if self.kind in ("stage", "discharge") and self.value is None:
            raise ValueError(f"boundary kind '{self.kind}' needs a value")

    def at(self, t: float):
        """Value at time t: a float, or one value per batch member."""
        v = self.value(t) if callable(self.value) else self.value
        if hasattr(v, "detach"):
            v = v.detach().cpu().numpy()
        return v if hasattr(v, "shape") else float(v)


def edge_values(bcs: dict[str, EdgeBC], t: float) -> list:
    return [bcs[e].at(t) if bcs[e].kind in ("stage", "discharge") else 0.0 for e in EDGES]


def all_edges(kind: str = "closed", **overrides) -> dict[str, EdgeBC]:
    bcs = {e: EdgeBC(kind) for e in EDGES}
    for k, v in overrides.items():
        if k not in EDGES:
            raise ValueError(f"unknown edge '{k}'")
        bcs[k] = v if isinstance(v, EdgeBC) else EdgeBC(v)
    return bcs


def bc_codes(bcs: dict[str, EdgeBC]) -> np.ndarray:
    missing = [e for e in EDGES if e not in bcs]
    if missing:
        raise ValueError(f"boundary conditions missing for edges {missing}")
    return np.array([KIND_CODE[bcs[e].kind] for e in EDGES], dtype=np.int32)
