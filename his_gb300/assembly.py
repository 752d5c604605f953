"""Assemble the drop-in solvers into a coupled engine: the role of the reference's
hydrointel/engine.py:169-238 (build_engine, build_engine_batch).

Two call forms each:

* the reference's own argument lists, for code that keeps the reference's run
  configuration, domain and scenario forcing and swaps only the solver imports:
  ``build_engine(cfg, domain, forcing, storage, kappa, manning, gamma, landuse=None,
  device=None, closed=False)`` and ``build_engine_batch(cfg, domain, forcings,
  storages, kappas, mannings, gammas, landuses, device=None) -> (engine, forcing)``.
  The objects are read by attribute (``cfg.solver``, ``cfg.dtype``; ``domain.dem2d``,
  ``dx``, ``sea``, ``landuse``, ``network``; a forcing's ``rain``, ``inflow``,
  ``tide``, ``storm_start`` and ``ssp.drainage_investment_factor``), so the
  reference's classes or any stand-ins with those fields work.  Every solver lives on
  the CUDA device; a CPU device given for the 1-D model is not used.
* ``build_engine(storm)`` / ``build_engine_batch(storms)`` for the seeded synthetic
  storms of ``workloads`` (their own terrain, network, bank links and forcing).

Either way: sea cells start at the tide level, the channel network at the larger of
the Manning normal depth of the initial inflow and the initial tide, and the rain,
tide and inflow are evaluated from closed-form tables (``workloads.Forcing``).
"""
from __future__ import annotations

import numpy as np
import torch

from .boundaries import EdgeBC
from .channels import apply_gamma
from .config import SolverConfig
from .coupling import CoupledEngine, links_from_cells
from .infiltration import Horton
from .swe1d import SWE1D
from .swe2d import SWE2D
from .topology import build_topology, sections
from .workloads import MMH, BatchForcing, Forcing, Storm, bank_links, normal_depth

EDGES = ("west", "east", "south", "north")


# ----------------------------------------------------------------- forcing
def forcing_tables(forcing) -> Forcing:
    """The closed-form tables of a scenario forcing (the reference's engine.Forcing:
    a Hyetograph ``rain`` in mm/h blocks, an InflowHydrograph ``inflow`` and a
    harmonic ``Tide``; hydrointel/forcing/hyetograph.py:23-46, tide.py:15-31,
    catchment.py:26-40): rain blocks in m/s from the same start and step, the tide's
    constituents, mean level plus sea-level rise, phase shift and on/off switch, and
    the inflow table.  Evaluated with the same floor, clamp and interpolation steps."""
    rain, tide, inflow = forcing.rain, forcing.tide, forcing.inflow
    cons = list(tide.cfg.constituents.values())
    return Forcing(rain_t0=float(rain.t_start), rain_step=float(rain.step_s),
                   rain=np.asarray(rain.intensity_mmh, dtype=np.float64) * MMH,
                   tide_base=float(tide.cfg.msl_offset_m + tide.slr_m), tide_shift=float(tide.shift_s),
                   tide_on=bool(tide.on),
                   tide_amp=tuple(float(c["amp_m"]) for c in cons),
                   tide_w=tuple(2 * np.pi / (float(c["period_h"]) * 3600.0) for c in cons),
                   tide_phase=tuple(float(np.radians(c["phase_deg"])) for c in cons),
                   q_t0=float(inflow.t0), q_step=float(inflow.step_s),
                   q=np.asarray(inflow.q_m3s, dtype=np.float64))


def _effective_gamma(gamma, forcing):
    """Channel conveyance scale of a scenario: the member's gamma times the scenario's
    drainage-investment factor, kept in [0.5, 3] (engine.py:182, :213)."""
    return np.clip(np.asarray(gamma, float) * forcing.ssp.drainage_investment_factor, 0.5, 3.0)


def initial_channel_level(net, cfg: SolverConfig, q0: float, eta0: float | None) -> np.ndarray:
    """Initial 1-D water level per cell: the Manning normal depth of discharge q0 above
    the bed, and not below the sea level eta0 (None: no floor) (engine.py:233-236)."""
    tp = build_topology(net)
    level = tp.z + normal_depth(tp, sections(tp, cfg.slot_width_frac), q0)
    return level if eta0 is None else np.maximum(level, eta0)


def _sea_state(dem, sea, eta0):
    """Depth of the sea cells at level eta0 (per member when eta0 is an array)."""
    eta = np.asarray(eta0, dtype=np.float64)
    if eta.ndim:
        eta = eta[:, None, None]
    return np.where(np.asarray(sea, bool), np.maximum(eta - np.asarray(dem, np.float64), 0.0), 0.0)


def _host(a):
    if torch.is_tensor(a):
        return a.detach().to("cpu").double().numpy()
    return np.asarray(a, dtype=np.float64)


# ------------------------------------------------- reference argument lists
def _engine_for_run(cfg, domain, forcing, storage, kappa, manning, gamma, landuse=None, device=None,
                    closed: bool = False) -> CoupledEngine:
    sv = SolverConfig.coerce(cfg.solver)
    dtype = cfg.dtype
    net = apply_gamma(domain.network, _effective_gamma(gamma, forcing))
    tables = forcing_tables(forcing)
    if closed:
        for r in net.reaches:
            r.up = r.up if r.up[0] == "junction" else ("closed",)
            r.down = r.down if r.down[0] == "junction" else ("closed",)
        bcs = {e: EdgeBC("closed") for e in EDGES}
        inflow = None
    else:
        bcs = {e: EdgeBC("transmissive") for e in EDGES}
        bcs["north"] = EdgeBC("stage", tables.tide)
        inflow = tables.inflow
    lu = domain.landuse if landuse is None else landuse
    horton = Horton.from_landuse(lu, _host(kappa), None, dtype, t0=forcing.storm_start)
    two = SWE2D(domain.dem2d, _host(manning), domain.dx, sv, bcs, device, dtype, storage=_host(storage),
                horton=horton)
    one = SWE1D(net, sv, device, dtype, inflow=inflow, stage=tables.tide)
    eta0 = tables.tide(0.0)
    two.set_state(_sea_state(domain.dem2d, domain.sea, eta0))
    q0 = tables.inflow(0.0)
    one.set_level(torch.as_tensor(initial_channel_level(net, sv, q0, None if closed else eta0)))
    return CoupledEngine(two, one, sv, rain=tables.rain_rate)


def _batch_for_run(cfg, domain, forcings, storages, kappas, mannings, gammas, landuses, device=None):
    b = len(forcings)
    if not (len(storages) == len(kappas) == len(mannings) == len(gammas) == len(landuses) == b):
        raise ValueError(f"batched inputs disagree in length: {b} forcings but "
                         f"{len(storages)}/{len(kappas)}/{len(mannings)}/{len(gammas)}/{len(landuses)} fields")
    sv = SolverConfig.coerce(cfg.solver)
    dtype = cfg.dtype
    starts = {float(f.storm_start) for f in forcings}
    if len(starts) != 1:
        raise ValueError("batched forcings must share the storm start (the infiltration clock)")
    bf = BatchForcing([forcing_tables(f) for f in forcings])
    nets = [apply_gamma(domain.network, _effective_gamma(g, f)) for g, f in zip(gammas, forcings)]
    bcs = {e: EdgeBC("transmissive") for e in EDGES}
    bcs["north"] = EdgeBC("stage", bf.tide)
    t0 = starts.pop()
    parts = [Horton.from_landuse(lu, _host(k), None, dtype, t0=t0) for lu, k in zip(landuses, kappas)]
    horton = Horton(*(torch.stack([getattr(h, f) for h in parts]) for f in ("f0", "fc", "k")), t0)
    stack = lambda xs: np.stack([_host(x) for x in xs])
    two = SWE2D(domain.dem2d, stack(mannings), domain.dx, sv, bcs, device, dtype, storage=stack(storages),
                horton=horton, batch=b)
    one = SWE1D(nets, sv, device, dtype, inflow=bf.inflow, stage=bf.tide)
    eta0 = bf.tide(0.0)
    two.set_state(_sea_state(domain.dem2d, domain.sea, eta0))
    q0 = bf.inflow(0.0)
    one.set_level(torch.as_tensor(np.stack([initial_channel_level(n, sv, float(q), float(e))
                                            for n, q, e in zip(nets, q0, eta0)])))
    return CoupledEngine(two, one, sv, rain=bf.rain_rate), bf


# ------------------------------------------------------- synthetic storms
def storm_bcs(storm: Storm) -> dict:
    f = storm.forcing
    out = {}
    for e, kind in zip(EDGES, storm.bc):
        out[e] = EdgeBC(kind, f.tide if kind == "stage" else (0.0 if kind == "discharge" else None))
    return out


def _engine_for_storm(storm: Storm, cfg: SolverConfig | None = None, dtype=torch.float64, device=None,
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
    one.set_level(torch.as_tensor(initial_channel_level(storm.network, cfg, f.inflow(0.0), f.tide(0.0))))
    cell1d, cells2d, length = bank_links(ter, build_topology(storm.network))
    links = links_from_cells(one, two, cell1d, cells2d, length)
    return CoupledEngine(two, one, cfg, rain=f.rain_rate, links=links)


def _batch_for_storms(storms: list[Storm], cfg: SolverConfig | None = None, dtype=torch.float64, device=None,
                      tile=None) -> CoupledEngine:
    ter = storms[0].terrain
    if any(s.terrain is not ter for s in storms):
        raise ValueError("batched storms must share the terrain")
    B = len(storms)
    cfg = cfg or SolverConfig(slot_width_frac=storms[0].slot_width_frac)
    stack = lambda xs: np.stack([np.broadcast_to(np.asarray(x, float), (ter.ny, ter.nx)) for x in xs])
    horton = None
    if storms[0].horton is not None:
        horton = Horton(*(stack([s.horton[j] for s in storms]) for j in range(3)), storms[0].horton[3])
    bf = BatchForcing([s.forcing for s in storms])
    bcs = {e: EdgeBC(k, bf.tide if k == "stage" else None) for e, k in zip(EDGES, storms[0].bc)}
    two = SWE2D(ter.z, stack([s.manning for s in storms]), ter.dx, cfg, bcs, device=device, dtype=dtype,
                storage=stack([s.storage for s in storms]) if storms[0].storage is not None else None,
                horton=horton, batch=B, tile=tile)
    two.set_state(np.stack([s.h0() for s in storms]))
    one = SWE1D([s.network for s in storms], cfg, device=device, inflow=bf.inflow, stage=bf.tide)
    one.set_level(torch.as_tensor(np.stack([initial_channel_level(s.network, cfg, s.forcing.inflow(0.0),
                                                                  s.forcing.tide(0.0)) for s in storms])))
    cell1d, cells2d, length = bank_links(ter, build_topology(storms[0].network))
    links = links_from_cells(one, two, cell1d, cells2d, length)
    return CoupledEngine(two, one, cfg, rain=bf.rain_rate, links=links)


# ------------------------------------------------------------ entry points
def build_engine(*args, **kwargs) -> CoupledEngine:
    """``build_engine(storm, cfg=None, dtype=float64, device=None, tile=None)`` for a
    synthetic storm, or the reference's ``build_engine(cfg, domain, forcing, storage,
    kappa, manning, gamma, landuse=None, device=None, closed=False)``."""
    if (args and isinstance(args[0], Storm)) or "storm" in kwargs:
        return _engine_for_storm(*args, **kwargs)
    return _engine_for_run(*args, **kwargs)


def build_engine_batch(*args, **kwargs):
    """``build_engine_batch(storms, cfg=None, dtype=float64, device=None, tile=None)``
    for synthetic storms on one terrain (returns the engine), or the reference's
    ``build_engine_batch(cfg, domain, forcings, storages, kappas, mannings, gammas,
    landuses, device=None)`` (returns the engine and the batch forcing)."""
    first = args[0] if args else kwargs.get("storms")
    if isinstance(first, (list, tuple)) and first and isinstance(first[0], Storm):
        return _batch_for_storms(*args, **kwargs)
    return _batch_for_run(*args, **kwargs)


__all__ = ["build_engine", "build_engine_batch", "forcing_tables", "initial_channel_level", "storm_bcs"]
