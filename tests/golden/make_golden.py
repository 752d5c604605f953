"""Generate golden vectors by running the reference solver itself (float64, CPU).

Run in a container where the reference project is checked out:

    python tests/golden/make_golden.py <reference checkout> [group ...]

It imports ``hydrointel`` from the given checkout, drives the reference's own
SWE2D / SWE1D / exchange / CoupledEngine on small seeded cases and writes
``tests/golden/*.npz``.  The cases are defined in ``golden_cases.py`` (shared with
the tests, so that forcing callables are rebuilt identically).  The fixtures are
committed; nothing at test time reads the reference.
"""
from __future__ import annotations

import math
import sys
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
sys.path.insert(0, str(HERE))
import golden_cases as GC  # noqa: E402


def _t(x):
    import torch
    return x.detach().cpu().numpy().astype(np.float64) if torch.is_tensor(x) else np.asarray(x, dtype=np.float64)


def make_swe2d(name: str, ref):
    import torch
    from hydrointel.config import SolverConfig
    from hydrointel.solver.boundaries import EdgeBC
    from hydrointel.solver.infiltration import Horton
    from hydrointel.solver.swe2d import SWE2D
    spec = GC.SWE2D_CASES[name]
    inp = GC.swe2d_inputs(spec)
    cfg = SolverConfig(spatial_order=spec["order"], flux=spec["flux"], compile=False)
    bcs = {e: EdgeBC(k, GC.bc_value(spec, e)) for e, k in zip(GC.EDGES, spec["bc"])}
    horton = None
    if inp.get("f0") is not None:
        horton = Horton(torch.as_tensor(inp["f0"]), torch.as_tensor(inp["fc"]), torch.as_tensor(inp["k"]),
                        spec["t0"])
    sim = SWE2D(inp["z"], inp["n"], spec["dx"], cfg, bcs, torch.device("cpu"), torch.float64,
                storage=inp.get("S"), horton=horton, rain_weight=inp.get("rain_weight"), dy=spec.get("dy"),
                batch=spec.get("batch"))
    sim.set_state(inp["h0"], inp["hu0"], inp["hv0"])
    rec = {k: [] for k in ("dt", "t", "rate", "bnd_in", "bnd_out", "rain", "infil", "clip")}
    snaps = {}
    t = 0.0
    for k in range(spec["steps"]):
        rate = float(sim._max_rate(sim.h, sim.hu, sim.hv))
        dt = min(sim.max_dt(), spec.get("dt_cap", 1e9))
        vol = sim.step(dt, t, GC.rain_value(spec, t))
        rec["dt"].append(dt); rec["t"].append(t); rec["rate"].append(rate)
        for key, val in zip(("bnd_in", "bnd_out", "rain", "infil", "clip"),
                            (vol.bnd_in, vol.bnd_out, vol.rain, vol.infil, vol.clip)):
            rec[key].append(_t(val).reshape(-1))
        t += dt
        if k + 1 in spec["snap_at"]:
            for f in ("h", "hu", "hv", "s_filled", "infil_cum"):
                snaps[f"{f}_{k + 1}"] = _t(getattr(sim, f))
    out = {k: np.asarray(v) for k, v in rec.items()}
    out.update(snaps)
    out.update({f"in_{k}": np.asarray(v) for k, v in inp.items() if v is not None})
    np.savez_compressed(HERE / f"{name}.npz", **out)
    print(name, "steps", spec["steps"], "final t", t)


def make_swe1d(name: str):
    import torch
    from hydrointel.config import SolverConfig
    from hydrointel.domain.channels import apply_gamma
    from hydrointel.solver.swe1d import SWE1D
    spec = GC.SWE1D_CASES[name]
    cfg = SolverConfig(compile=False, slot_width_frac=spec["slot_width_frac"])
    net = GC.network(spec)
    B = spec.get("batch")
    nets = [apply_gamma(net, np.asarray(g)) for g in spec["gammas"]] if B else net
    one = SWE1D(nets, cfg, torch.device("cpu"), torch.float64, inflow=GC.inflow_fn(spec), stage=GC.stage_fn(spec))
    one.set_level(torch.maximum(one.z + spec["init_depth"], torch.full_like(one.z, GC.stage_fn(spec)(0.0)
                                                                           if B is None else -1e9)))
    tp = one.topo
    out = {f"topo_{k}": np.asarray(getattr(tp, k)) for k in ("kind", "reach_of", "ghost_src", "ghost_sign",
                                                              "face_l", "face_r", "z", "b", "m", "zbank", "n",
                                                              "dx", "x", "y", "chain")}
    out["n_cells"] = np.asarray(tp.n_cells)
    for k in ("b", "m", "yb", "ts"):
        out[f"sec_{k}"] = _t(getattr(one.sec, k))
        out[f"fsec_{k}"] = _t(getattr(one.fsec, k))
    out["z_members"] = _t(one.z)
    out["A0"], out["Q0"] = _t(one.A), _t(one.Q)
    rec = {k: [] for k in ("dt", "t", "max_dt", "bnd_in", "bnd_out", "clip")}
    t = 0.0
    for k in range(spec["steps"]):
        mdt = one.max_dt()
        dt = mdt * spec.get("dt_frac", 1.0)
        v = one.step(dt, t)
        rec["dt"].append(dt); rec["t"].append(t); rec["max_dt"].append(mdt)
        rec["bnd_in"].append(_t(v.bnd_in).reshape(-1)); rec["bnd_out"].append(_t(v.bnd_out).reshape(-1))
        rec["clip"].append(_t(v.clip).reshape(-1))
        t += dt
        if k + 1 in spec["snap_at"]:
            out[f"A_{k + 1}"], out[f"Q_{k + 1}"] = _t(one.A), _t(one.Q)
    out.update({k: np.asarray(v) for k, v in rec.items()})
    np.savez_compressed(HERE / f"{name}.npz", **out)
    print(name, "cells", tp.n_cells, "final t", t)


def make_exchange(name: str):
    import torch
    from hydrointel.benchmarks.suite import _overtopping_case
    from hydrointel.solver.coupling import exchange
    spec = GC.EXCHANGE_CASES[name]
    eng, one, two = _overtopping_case(torch.device("cpu"), dx=spec["dx"])
    L = eng.links
    out = {"links_cell1d": _t(L.cell1d).astype(np.int64), "links_zbank": _t(L.zbank),
           "links_length": _t(L.length), "links_z2": _t(L.z2), "links_inv": _t(L.inv).astype(np.int64),
           "links_uniq": _t(L.uniq_dev).astype(np.int64), "z2d": _t(two.z), "z1d": _t(one.z),
           "dx1": _t(one.dx), "area2": np.asarray(two.area)}
    for k in ("b", "m", "yb", "ts"):
        out[f"sec_{k}"] = _t(getattr(one.sec, k))
    for k in ("kind", "reach_of", "ghost_src", "ghost_sign", "face_l", "face_r", "z", "b", "m", "zbank", "n",
              "dx", "x", "y", "chain"):
        out[f"topo_{k}"] = np.asarray(getattr(one.topo, k))
    out["n_cells"] = np.asarray(one.topo.n_cells)
    out["n2d"] = _t(two.n)
    g = torch.Generator().manual_seed(spec["seed"])
    for i in range(spec["calls"]):
        two.set_state(torch.rand(two.z.shape, generator=g, dtype=torch.float64) * 1.5)
        two.hu = torch.rand(two.z.shape, generator=g, dtype=torch.float64) - 0.5
        two.hv = torch.rand(two.z.shape, generator=g, dtype=torch.float64) - 0.5
        one.A = one.sec.area(torch.rand(one.z.shape, generator=g, dtype=torch.float64) * 4.0)
        out[f"h_in_{i}"], out[f"hu_in_{i}"], out[f"hv_in_{i}"] = _t(two.h), _t(two.hu), _t(two.hv)
        out[f"A_in_{i}"] = _t(one.A)
        V = exchange(one, two, L, spec["dt"], eng.cfg)
        out[f"V_{i}"] = _t(V)
        out[f"h_out_{i}"], out[f"hu_out_{i}"], out[f"hv_out_{i}"] = _t(two.h), _t(two.hu), _t(two.hv)
        out[f"A_out_{i}"] = _t(one.A)
    np.savez_compressed(HERE / f"{name}.npz", **out)
    print(name, "links", len(L.cell1d))


def make_coupled(name: str):
    import torch
    from hydrointel.benchmarks.suite import _overtopping_case
    spec = GC.COUPLED_CASES[name]
    eng, one, two = _overtopping_case(torch.device("cpu"), dx=spec["dx"])
    eng.rain = GC.rain_fn_coupled(spec)
    two.set_state(np.asarray(GC.coupled_h0(spec, _t(two.z))))
    eng.mb = type(eng.mb)(two.device, eng.total_volume())
    rec = {k: [] for k in ("dt", "n_sub", "t")}
    t = 0.0
    out = {"h0": _t(two.h), "A0": _t(one.A), "Q0": _t(one.Q)}
    for k in range(spec["steps"]):
        dt = min(two.max_dt(), spec["t_end"] - t)
        n_sub = max(1, math.ceil(dt / one.max_dt() - 1e-9))
        rec["dt"].append(dt); rec["n_sub"].append(n_sub); rec["t"].append(t)
        t = eng.step(t, spec["t_end"], dt=dt, n_sub=n_sub)
        if k + 1 in spec["snap_at"]:
            out[f"h_{k + 1}"], out[f"hu_{k + 1}"], out[f"hv_{k + 1}"] = _t(two.h), _t(two.hu), _t(two.hv)
            out[f"A_{k + 1}"], out[f"Q_{k + 1}"] = _t(one.A), _t(one.Q)
    src = eng.mb.sources()
    for k, v in src.items():
        out[f"src_{k}"] = np.asarray(v, dtype=np.float64)
    out["mass_err"] = np.asarray(eng.mb.check(eng.total_volume(), t, record=False))
    out.update({k: np.asarray(v) for k, v in rec.items()})
    np.savez_compressed(HERE / f"{name}.npz", **out)
    print(name, "steps", spec["steps"], "final t", t, "mass err", float(out["mass_err"]))


def make_coupled_batch(name: str):
    """Two members of the overtopping case in one batched reference CoupledEngine,
    stepped with the reference's own shared CFL choice."""
    import torch
    from hydrointel.benchmarks.suite import _overtopping_case
    from hydrointel.domain.channels import apply_gamma
    from hydrointel.solver.boundaries import all_edges
    from hydrointel.solver.coupling import CoupledEngine
    from hydrointel.solver.swe1d import SWE1D
    from hydrointel.solver.swe2d import SWE2D
    spec = GC.COUPLED_BATCH_CASES[name]
    cpu = torch.device("cpu")
    eng0, one0, two0 = _overtopping_case(cpu, dx=spec["dx"])
    cfg = eng0.cfg
    B = len(spec["gamma"])
    z = _t(two0.z)
    n_b = np.stack([np.full(z.shape, m) for m in spec["manning"]])
    two = SWE2D(z, n_b, spec["dx"], cfg, all_edges("closed"), cpu, torch.float64, batch=B)
    nets = [apply_gamma(one0.net, [g]) for g in spec["gamma"]]
    one = SWE1D(nets, cfg, cpu, inflow=GC.inflow_batch(spec), stage=one0.stage)
    off = torch.as_tensor(spec["level_offset"], dtype=torch.float64)[:, None]
    one.set_level(one.z + off)
    eng = CoupledEngine(two, one, cfg, rain=GC.rain_fn_batch(spec))
    two.set_state(torch.as_tensor(GC.coupled_h0_batch(spec, z)))
    eng.mb = type(eng.mb)(two.device, eng.total_volume())
    rec = {k: [] for k in ("dt", "n_sub", "t")}
    t = 0.0
    out = {"h0": _t(two.h), "A0": _t(one.A), "Q0": _t(one.Q)}
    for k in range(spec["steps"]):
        dt = min(two.max_dt(), spec["t_end"] - t)
        n_sub = max(1, math.ceil(dt / one.max_dt() - 1e-9))
        rec["dt"].append(dt); rec["n_sub"].append(n_sub); rec["t"].append(t)
        t = eng.step(t, spec["t_end"], dt=dt, n_sub=n_sub)
        if k + 1 in spec["snap_at"]:
            out[f"h_{k + 1}"], out[f"hu_{k + 1}"], out[f"hv_{k + 1}"] = _t(two.h), _t(two.hu), _t(two.hv)
            out[f"A_{k + 1}"], out[f"Q_{k + 1}"] = _t(one.A), _t(one.Q)
    src = eng.mb.sources()
    for k, v in src.items():
        out[f"src_{k}"] = np.asarray(v, dtype=np.float64)
    out["mass_err"] = np.asarray(eng.mb.check(eng.total_volume(), t, record=False))
    out.update({k: np.asarray(v) for k, v in rec.items()})
    np.savez_compressed(HERE / f"{name}.npz", **out)
    print(name, "steps", spec["steps"], "final t", t, "n_sub max", max(rec["n_sub"]), "mass err", out["mass_err"])


ASSEMBLY = {"lx_m": 4000.0, "ly_m": 3200.0, "cell_m": 80.0, "seed": 7, "steps": 800,
            # (return period, rcp, ssp, horizon year, tide on, storm-tide offset h) per member
            "scenarios": [(25, "RCP4.5", "SSP2", 2050, True, 0.0), (100, "RCP8.5", "SSP5", 2080, True, -2.0)]}


def _store_forcing(out: dict, tag: str, fo) -> None:
    out[f"{tag}rain_step"], out[f"{tag}rain_t0"] = fo.rain.step_s, fo.rain.t_start
    out[f"{tag}rain_mmh"] = np.asarray(fo.rain.intensity_mmh, np.float64)
    out[f"{tag}q_step"], out[f"{tag}q_t0"] = fo.inflow.step_s, fo.inflow.t0
    out[f"{tag}q"] = np.asarray(fo.inflow.q_m3s, np.float64)
    cons = list(fo.tide.cfg.constituents.values())
    for k in ("amp_m", "period_h", "phase_deg"):
        out[f"{tag}tide_{k}"] = np.array([c[k] for c in cons], np.float64)
    out[f"{tag}tide_msl"], out[f"{tag}tide_slr"] = fo.tide.cfg.msl_offset_m, fo.tide.slr_m
    out[f"{tag}tide_on"], out[f"{tag}tide_shift"] = float(fo.tide.on), fo.tide.shift_s
    out[f"{tag}storm_start"], out[f"{tag}t_end"] = fo.storm_start, fo.t_end
    out[f"{tag}drainage"] = fo.ssp.drainage_investment_factor
    ts = np.linspace(0.0, fo.t_end, 97)
    out[f"{tag}sample_t"] = ts
    out[f"{tag}sample_rain"] = np.array([fo.rain.rate_ms(t) for t in ts])
    out[f"{tag}sample_tide"] = np.array([fo.tide(t) for t in ts])
    out[f"{tag}sample_inflow"] = np.array([fo.inflow(t) for t in ts])


def _run_recorded(eng, t_end: float, steps: int, out: dict, tag: str) -> None:
    """Drive a reference CoupledEngine on its own CFL choice, recording dt and n_sub."""
    dts, subs = [], []
    t = 0.0
    for _ in range(steps):
        dt = min(eng.two.max_dt(), t_end - t)
        n_sub = max(1, math.ceil(dt / eng.one.max_dt() - 1e-9))
        dts.append(dt)
        subs.append(n_sub)
        t = eng.step(t, t_end, dt=dt, n_sub=n_sub)
    out[f"{tag}dt"], out[f"{tag}n_sub"] = np.array(dts), np.array(subs)
    for f in ("h", "hu", "hv", "s_filled", "infil_cum"):
        out[f"{tag}{f}_end"] = _t(getattr(eng.two, f))
    out[f"{tag}A_end"], out[f"{tag}Q_end"] = _t(eng.one.A), _t(eng.one.Q)
    for k, v in eng.mb.sources().items():
        out[f"{tag}src_{k}"] = np.asarray(v, np.float64)


def make_assembly():
    """The reference's own engine assembly (hydrointel/engine.py:169-238) on a small
    generated domain: build_engine for one scenario and build_engine_batch for two, each
    run 800 steps (past the storm start at 1800 s); the inputs are stored as plain arrays so the assembly can be rebuilt
    without the reference."""
    import dataclasses
    import torch
    from hydrointel.config import DomainConfig, RunConfig
    from hydrointel.domain import landuse as LU
    from hydrointel.domain.synthetic import generate
    from hydrointel.engine import build_engine, build_engine_batch, build_forcing
    A = ASSEMBLY
    cfg = RunConfig()
    cfg.solver.compile = False
    cfg.domain = dataclasses.replace(cfg.domain, lx_m=A["lx_m"], ly_m=A["ly_m"], cell_m=A["cell_m"])
    dom = generate(cfg.domain, A["seed"])
    area = dom.nx * dom.ny * dom.dx ** 2 / 1e6
    out = {"dem2d": dom.dem2d.astype(np.float64), "dx": dom.dx, "sea": dom.sea.astype(bool),
           "landuse": dom.landuse.astype(np.int64), "inflow_reach": str(dom.network.inflow_reach)}
    for k in ("f0_mmh", "fc_mmh", "k_per_h"):
        out[f"lu_{k}"] = LU.table_array(k)
    out["n_reaches"], out["n_junctions"] = dom.network.n_reaches, len(dom.network.junctions)
    for i, r in enumerate(dom.network.reaches):
        for k in ("x", "y", "bed", "width", "side_slope", "manning", "z_bank"):
            out[f"reach{i}_{k}"] = np.asarray(getattr(r, k), np.float64)
        out[f"reach{i}_id"] = str(r.reach_id)
        out[f"reach{i}_up"] = np.array([str(v) for v in r.up])
        out[f"reach{i}_down"] = np.array([str(v) for v in r.down])
    for j, jn in enumerate(dom.network.junctions):
        out[f"junction{j}"] = np.array([jn.x, jn.y, jn.bed, jn.width, jn.side_slope, jn.manning, jn.z_bank,
                                        jn.length])
    members = []
    for m, sc in enumerate(A["scenarios"]):
        rng = np.random.default_rng(100 + m)
        lu = dom.landuse
        storage = LU.lookup(lu, "storage_m") * rng.uniform(0.5, 1.5)
        kappa = np.full(dom.shape, rng.uniform(0.7, 1.3))
        manning = LU.lookup(lu, "manning") * rng.uniform(0.8, 1.2)
        gamma = rng.uniform(0.8, 1.2, dom.network.n_reaches)
        fo = build_forcing(cfg, sc[0], sc[1], sc[2], sc[3], sc[4], sc[5], area)
        members.append((fo, storage, kappa, manning, gamma, lu))
        out[f"m{m}_storage"], out[f"m{m}_kappa"], out[f"m{m}_manning"], out[f"m{m}_gamma"] = \
            storage, kappa, manning, gamma
        _store_forcing(out, f"m{m}_", fo)
    cpu = torch.device("cpu")
    # one scenario
    fo, storage, kappa, manning, gamma, lu = members[0]
    eng = build_engine(cfg, dom, fo, storage, kappa, manning, gamma, landuse=lu, device=cpu)
    out["single_h0"], out["single_A0"] = _t(eng.two.h), _t(eng.one.A)
    out["single_level0"] = _t(eng.one.level())
    out["single_f0"], out["single_fc"], out["single_k"] = (_t(getattr(eng.two.horton, f)) for f in ("f0", "fc",
                                                                                                   "k"))
    _run_recorded(eng, fo.t_end, A["steps"], out, "single_")
    # both scenarios as one batch
    cols = list(zip(*members))
    engb, _ = build_engine_batch(cfg, dom, list(cols[0]), list(cols[1]), list(cols[2]), list(cols[3]),
                                 list(cols[4]), list(cols[5]), device=cpu)
    out["batch_h0"], out["batch_A0"] = _t(engb.two.h), _t(engb.one.A)
    _run_recorded(engb, members[0][0].t_end, A["steps"], out, "batch_")
    np.savez_compressed(HERE / "assembly_run.npz", **out)
    print("assembly_run", dom.ny, "x", dom.nx, "reaches", dom.network.n_reaches, "junctions",
          len(dom.network.junctions), "dt", out["single_dt"][[0, -1]], "n_sub max", out["single_n_sub"].max())


def reference_checkout(argv) -> Path:
    """The reference checkout: the first argument, else $HIS_REFERENCE; required."""
    import os
    root = argv[1] if len(argv) > 1 else os.environ.get("HIS_REFERENCE")
    if not root:
        raise SystemExit("usage: make_golden.py <reference checkout> [group ...]  (or set HIS_REFERENCE); "
                         "groups: swe2d swe1d exchange coupled coupled_batch assembly")
    root = Path(root)
    if not (root / "hydrointel").is_dir():
        raise SystemExit(f"{root} is not a checkout of the reference (no hydrointel/ package)")
    return root


def main(argv):
    ref = reference_checkout(argv)
    sys.path.insert(0, str(ref))
    import torch
    torch.set_num_threads(1)
    groups = {
        "swe2d": lambda: [make_swe2d(n, ref) for n in GC.SWE2D_CASES],
        "swe1d": lambda: [make_swe1d(n) for n in GC.SWE1D_CASES],
        "exchange": lambda: [make_exchange(n) for n in GC.EXCHANGE_CASES],
        "coupled": lambda: [make_coupled(n) for n in GC.COUPLED_CASES],
        "coupled_batch": lambda: [make_coupled_batch(n) for n in GC.COUPLED_BATCH_CASES],
        "assembly": make_assembly,
    }
    chosen = argv[2:] or list(groups)
    for g in chosen:
        if g not in groups:
            raise SystemExit(f"unknown group {g!r}; groups: {' '.join(groups)}")
        groups[g]()


if __name__ == "__main__":
    main(sys.argv)
