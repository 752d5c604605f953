"""Assemble the drop-in solvers for one storm (the role of the reference's
hydrointel/engine.py:206-238 build_engine): 2-D solver with its fields and edges,
1-D network at max(normal depth, tide), bank-cell weir links and the coupled loop.
"""
from __future__ import annotations

import numpy as np
import torch

from .boundaries import EdgeBC
from .config import SolverConfig
from .coupling import CoupledEngine, links_from_cells
from .infiltration import Horton
from .swe1d import SWE1D
from .swe2d import SWE2D
from .topology import build_topology, sections
from .workloads import BatchForcing, Storm, bank_links, normal_depth


def storm_bcs(storm: Storm) -> dict:
    f = storm.forcing
    out = {}
    for e, kind in zip(("west", "east", "south", "north"), storm.bc):
        out[e] = EdgeBC(kind, f.tide if kind == "stage" else (0.0 if kind == "discharge" else None))
    return out


def build_engine_batch(storms: list[Storm], cfg: SolverConfig | None = None, dtype=torch.float64, device=None,
                       tile=None) -> CoupledEngine:
    """B storms on one shared terrain as one batched drop-in engine (the role of the
    reference's build_engine_batch, hydrointel/engine.py:169-203): per-member fields,
    networks (same discretisation, own bed and width), rain, tide and inflow; one
    shared CFL step, as in the reference."""
    ter = storms[0].terrain
    if any(s.terrain is not ter for s in storms):
        raise ValueError("batched storms must share the terrain")
    B = len(storms)
    cfg = cfg or SolverConfig(slot_width_frac=storms[0].slot_width_frac)
    stack = lambda xs: np.stack([np.broadcast_to(np.asarray(x, float), (ter.ny, ter.nx)) for x in xs])
    horton = None
    if storms[0].horton is not None:
        horton = Horton(stack([s.horton[0] for s in storms]), stack([s.horton[1] for s in storms]),
                        stack([s.horton[2] for s in storms]), storms[0].horton[3])
    bf = BatchForcing([s.forcing for s in storms])
    tide = bf.tide
    bcs = {e: EdgeBC(k, tide if k == "stage" else None) for e, k in zip(("west", "east", "south", "north"),
                                                                          storms[0].bc)}
    two = SWE2D(ter.z, stack([s.manning for s in storms]), ter.dx, cfg, bcs, device=device, dtype=dtype,
                storage=stack([s.storage for s in storms]) if storms[0].storage is not None else None,
                horton=horton, batch=B, tile=tile)
    two.set_state(np.stack([s.h0() for s in storms]))
    inflow = bf.inflow
    one = SWE1D([s.network for s in storms], cfg, device=device, inflow=inflow, stage=tide)
    levels = []
    for s in storms:
        tp = build_topology(s.network)
        yn = normal_depth(tp, sections(tp, cfg.slot_width_frac), s.forcing.inflow(0.0))
        levels.append(np.maximum(tp.z + yn, s.forcing.tide(0.0)))
    one.set_level(torch.as_tensor(np.stack(levels)))
    tp0 = build_topology(storms[0].network)
    cell1d, cells2d, length = bank_links(ter, tp0)
    links = links_from_cells(one, two, cell1d, cells2d, length)
    rain = bf.rain_rate
    return CoupledEngine(two, one, cfg, rain=rain, links=links)


def build_engine(storm: Storm, cfg: SolverConfig | None = None, dtype=torch.float64, device=None,
                 tile=None) -> CoupledEngine:
    cfg = cfg or SolverConfig(slot_width_frac=storm.slot_width_frac)
    cfg.slot_width_frac = storm.slot_width_frac
    ter = storm.terrain
    horton = Horton(*storm.horton) if storm.horton is not None else None
    two = SWE2D(ter.z, storm.manning, ter.dx, cfg, storm_bcs(storm), device=device, dtype=dtype,
                storage=storm.storage, horton=horton, tile=tile)
    two.set_state(storm.h0())
    if storm.network is None:
        return CoupledEngine(two, None, cfg, rain=storm.forcing.rain_rate)
    f = storm.forcing
    one = SWE1D(storm.network, cfg, device=device, inflow=f.inflow, stage=f.tide)
    tp = build_topology(storm.network)
    yn = normal_depth(tp, sections(tp, cfg.slot_width_frac), f.inflow(0.0))
    one.set_level(torch.as_tensor(np.maximum(tp.z + yn, f.tide(0.0))))
    cell1d, cells2d, length = bank_links(ter, tp)
    links = links_from_cells(one, two, cell1d, cells2d, length)
    return CoupledEngine(two, one, cfg, rain=f.rain_rate, links=links)
