"""Test harness: builds oracle objects (and, on a GPU, the CUDA engine's objects) for the
golden cases, from the committed fixtures and the shared case definitions."""
from __future__ import annotations

from pathlib import Path
from types import SimpleNamespace

import numpy as np

import golden_cases as GC
from his_gb300.boundaries import EdgeBC
from his_gb300.config import SolverConfig

GOLDEN = Path(__file__).resolve().parent / "golden"


def load(name: str) -> dict:
    with np.load(GOLDEN / f"{name}.npz") as f:
        return {k: f[k] for k in f.files}


def swe2d_cfg(spec) -> SolverConfig:
    return SolverConfig(spatial_order=spec["order"], flux=spec["flux"])


def swe2d_bcs(spec) -> dict:
    return {e: EdgeBC(k, GC.bc_value(spec, e)) for e, k in zip(GC.EDGES, spec["bc"])}


def swe2d_inputs(name: str, fx: dict) -> dict:
    g = lambda k: fx.get(f"in_{k}")
    return {k: g(k) for k in ("z", "n", "S", "f0", "fc", "k", "rain_weight", "h0", "hu0", "hv0")}


def oracle_swe2d(name: str, fx: dict | None = None):
    from oracle.oracle import OracleSWE2D
    spec = GC.SWE2D_CASES[name]
    fx = fx if fx is not None else load(name)
    inp = swe2d_inputs(name, fx)
    horton = (inp["f0"], inp["fc"], inp["k"], spec["t0"]) if inp["f0"] is not None else None
    sim = OracleSWE2D(inp["z"], inp["n"], spec["dx"], swe2d_cfg(spec), swe2d_bcs(spec), storage=inp["S"],
                      horton=horton, rain_weight=inp["rain_weight"], dy=spec.get("dy"), batch=spec.get("batch"))
    sim.set_state(inp["h0"], inp["hu0"], inp["hv0"])
    return sim, spec, fx


def topo_from(fx: dict) -> SimpleNamespace:
    keys = ("kind", "reach_of", "ghost_src", "ghost_sign", "face_l", "face_r", "z", "b", "m", "zbank", "n", "dx",
            "x", "y", "chain")
    t = SimpleNamespace(**{k: fx[f"topo_{k}"] for k in keys})
    t.n_cells = int(fx["n_cells"])
    return t


def oracle_swe1d(name: str, fx: dict | None = None):
    from oracle.oracle import OracleSWE1D
    spec = GC.SWE1D_CASES[name]
    fx = fx if fx is not None else load(name)
    cfg = SolverConfig(slot_width_frac=spec["slot_width_frac"])
    topo = topo_from(fx)
    one = OracleSWE1D(topo, cfg, batch=spec.get("batch"), z=fx["z_members"], b=fx["sec_b"],
                      inflow=GC.inflow_fn(spec), stage=GC.stage_fn(spec))
    one.A = np.ascontiguousarray(fx["A0"].reshape(one.A.shape))
    one.Q = np.ascontiguousarray(fx["Q0"].reshape(one.Q.shape))
    return one, spec, fx


def overtop_parts(fx: dict, cfg: SolverConfig | None = None):
    """The reference's overtopping case (benchmarks/suite.py:406-431) rebuilt from the exchange fixture:
    1-D topology, 2-D bed and roughness, links and forcing."""
    cfg = cfg or SolverConfig()
    topo = topo_from(fx)
    zb_last = float(fx["topo_zbank"][fx["topo_kind"] == 0][-1])
    return SimpleNamespace(cfg=cfg, topo=topo, z2d=fx["z2d"], n2d=fx["n2d"], dx=float(np.sqrt(fx["area2"])),
                           inflow=GC.overtop_inflow, stage=lambda t: zb_last - 1.0,
                           links={k: fx[f"links_{k}"] for k in ("cell1d", "zbank", "length", "z2", "inv", "uniq")})


def oracle_overtop(fx: dict, cfg: SolverConfig | None = None):
    from oracle.oracle import OracleLinks, OracleSWE1D, OracleSWE2D
    from his_gb300.boundaries import all_edges
    p = overtop_parts(fx, cfg)
    two = OracleSWE2D(p.z2d, p.n2d, p.dx, p.cfg, all_edges("closed"))
    one = OracleSWE1D(p.topo, p.cfg, inflow=p.inflow, stage=p.stage)
    links = OracleLinks(**p.links)
    return one, two, links, p


def max_abs(a, b) -> float:
    a, b = np.asarray(a, dtype=np.float64), np.asarray(b, dtype=np.float64)
    return float(np.max(np.abs(a - b))) if a.size else 0.0


def overtop_network(mod):
    """The channel of the reference's overtopping case (benchmarks/suite.py:410-418)."""
    xs = np.arange(20.0, 2000.0, 40.0)
    zb = 5.0 - 0.001 * xs
    n = len(xs)
    r = mod.Reach("ch", xs, np.full(n, 500.0), zb - 2.0, np.full(n, 15.0), np.full(n, 1.0), np.full(n, 0.03), zb,
                  ("inflow",), ("stage",))
    return mod.ChannelNetwork([r], [], "ch")


def cuda_swe2d(name: str, fx: dict | None = None, dtype=None, tile=None):
    import torch
    from his_gb300.infiltration import Horton
    from his_gb300.swe2d import SWE2D
    spec = GC.SWE2D_CASES[name]
    fx = fx if fx is not None else load(name)
    inp = swe2d_inputs(name, fx)
    horton = Horton(inp["f0"], inp["fc"], inp["k"], spec["t0"]) if inp["f0"] is not None else None
    sim = SWE2D(inp["z"], inp["n"], spec["dx"], swe2d_cfg(spec), swe2d_bcs(spec), dtype=dtype or torch.float64,
                storage=inp["S"], horton=horton, rain_weight=inp["rain_weight"], dy=spec.get("dy"),
                batch=spec.get("batch"), tile=tile)
    sim.set_state(inp["h0"], inp["hu0"], inp["hv0"])
    return sim, spec, fx


def cuda_overtop(fx: dict, dtype=None, cfg: SolverConfig | None = None):
    """The overtopping case on the CUDA solvers, built from the exchange fixture's bed."""
    import torch
    import his_gb300.channels as CH
    from his_gb300.boundaries import all_edges
    from his_gb300.coupling import build_links
    from his_gb300.swe1d import SWE1D
    from his_gb300.swe2d import SWE2D
    p = overtop_parts(fx, cfg)
    two = SWE2D(p.z2d, p.n2d, p.dx, p.cfg, all_edges("closed"), dtype=dtype or torch.float64)
    one = SWE1D(overtop_network(CH), p.cfg, inflow=p.inflow, stage=p.stage)
    links = build_links(one, two)
    return one, two, links, p


def oracle_from_storm(storm, cfg: SolverConfig | None = None):
    """The oracle's coupled engine for a synthetic storm (same fields, network, links, forcing)."""
    from oracle.oracle import OracleCoupled, OracleLinks, OracleSWE1D, OracleSWE2D
    from his_gb300.assembly import storm_bcs
    from his_gb300.topology import build_topology, sections
    from his_gb300.workloads import bank_links, normal_depth
    cfg = cfg or SolverConfig(slot_width_frac=storm.slot_width_frac)
    ter = storm.terrain
    two = OracleSWE2D(ter.z, np.broadcast_to(np.asarray(storm.manning, float), ter.z.shape), ter.dx, cfg,
                      storm_bcs(storm), storage=storm.storage, horton=storm.horton)
    two.set_state(storm.h0())
    f = storm.forcing
    if storm.network is None:
        return OracleCoupled(two, None, None, cfg, rain=f.rain_rate)
    tp = build_topology(storm.network)
    one = OracleSWE1D(tp, cfg, inflow=f.inflow, stage=f.tide)
    sec = sections(tp, cfg.slot_width_frac)
    y = np.maximum(np.maximum(tp.z + normal_depth(tp, sec, f.inflow(0.0)), f.tide(0.0)) - tp.z, 0.0)
    yt = np.minimum(y, sec["yb"])
    one.A[0] = yt * (sec["b"] + sec["m"] * yt) + sec["ts"] * np.maximum(y - sec["yb"], 0.0)
    cell1d, cells2d, length = bank_links(ter, tp)
    uniq, inv = np.unique(cells2d, return_inverse=True)
    links = OracleLinks(cell1d, tp.zbank[cell1d], np.full(len(cell1d), length), ter.z.reshape(-1)[cells2d], inv,
                        uniq)
    return OracleCoupled(two, one, links, cfg, rain=f.rain_rate)


def assembly_inputs(fx: dict):
    """The inputs of the reference's engine assembly (hydrointel/engine.py:169-238),
    rebuilt from the assembly fixture as plain stand-ins with the attributes the
    assembly reads: run configuration, domain (bed, sea mask, land use, channel
    network) and per member the scenario forcing and fields (storage, kappa,
    roughness, channel gamma).  Returns (cfg, domain, members, landuse table)."""
    import torch
    from his_gb300.channels import ChannelNetwork, Junction, Reach
    from his_gb300.config import SolverConfig
    NS = SimpleNamespace
    reaches = []
    for i in range(int(fx["n_reaches"])):
        g = lambda k: fx[f"reach{i}_{k}"]
        end = lambda a: tuple(int(v) if v.lstrip("-").isdigit() else str(v) for v in a)
        reaches.append(Reach(str(g("id")), g("x"), g("y"), g("bed"), g("width"), g("side_slope"), g("manning"),
                             g("z_bank"), end(g("up")), end(g("down"))))
    junctions = [Junction(*(float(v) for v in fx[f"junction{j}"])) for j in range(int(fx["n_junctions"]))]
    net = ChannelNetwork(reaches, junctions, str(fx["inflow_reach"]))
    domain = NS(dem2d=fx["dem2d"], dx=float(fx["dx"]), sea=fx["sea"], landuse=fx["landuse"], network=net)
    cfg = NS(solver=SolverConfig(), dtype=torch.float64)
    members = []
    m = 0
    while f"m{m}_rain_mmh" in fx:
        g = lambda k: fx[f"m{m}_{k}"]
        cons = {f"c{j}": {"amp_m": float(a), "period_h": float(p), "phase_deg": float(ph)}
                for j, (a, p, ph) in enumerate(zip(g("tide_amp_m"), g("tide_period_h"), g("tide_phase_deg")))}
        forcing = NS(rain=NS(step_s=float(g("rain_step")), intensity_mmh=g("rain_mmh"), t_start=float(g("rain_t0"))),
                     inflow=NS(step_s=float(g("q_step")), q_m3s=g("q"), t0=float(g("q_t0"))),
                     tide=NS(cfg=NS(constituents=cons, msl_offset_m=float(g("tide_msl"))), slr_m=float(g("tide_slr")),
                             on=bool(g("tide_on")), shift_s=float(g("tide_shift"))),
                     storm_start=float(g("storm_start")), t_end=float(g("t_end")),
                     ssp=NS(drainage_investment_factor=float(g("drainage"))))
        members.append(NS(forcing=forcing, storage=g("storage"), kappa=g("kappa"), manning=g("manning"),
                          gamma=g("gamma"), landuse=fx["landuse"]))
        m += 1
    table = {k: fx[f"lu_{k}"] for k in ("f0_mmh", "fc_mmh", "k_per_h")}
    return cfg, domain, members, table
