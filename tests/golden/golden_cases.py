"""Case definitions shared by the golden generator and the tests.

Each case is a small, seeded problem: the generator runs the reference solver on
it and stores the results; the tests rebuild the same inputs (and the same forcing
callables) from these definitions and compare.
"""
from __future__ import annotations

import math

import numpy as np

EDGES = ("west", "east", "south", "north")
MMH = 1.0 / 3.6e6

SWE2D_CASES = {
    # mixed boundaries, batched members with their own roughness, storage, Horton and rain
    "swe2d_bcmix": dict(ny=11, nx=14, dx=25.0, order=2, flux="hllc", batch=2,
                        bc=("discharge", "transmissive", "stage", "closed"), discharge_q=(0.3, 0.5),
                        stage=((0.9, 1.1), 0.15, 1.0 / 60.0), rain_mmh=(30.0, 55.0), horton=True, storage=True,
                        t0=20.0, steps=40, snap_at=(1, 10, 40), seed=1, eta0=1.0),
    # first order, HLL flux, rectangular cells, unbatched
    "swe2d_o1_hll": dict(ny=9, nx=12, dx=30.0, dy=20.0, order=1, flux="hll", batch=None,
                         bc=("closed", "transmissive", "closed", "stage"), stage=((1.2,), 0.0, 0.0),
                         rain_mmh=(80.0,), horton=False, storage=False, t0=0.0, steps=30, snap_at=(1, 30), seed=2,
                         eta0=1.1),
    # one-row strip: mirror ghosts with fewer cells than ghost layers across the strip
    "swe2d_strip": dict(ny=1, nx=40, dx=2.5, order=2, flux="hllc", batch=None,
                        bc=("transmissive", "transmissive", "closed", "closed"), rain_mmh=(0.0,), horton=False,
                        storage=False, t0=0.0, steps=60, snap_at=(1, 60), seed=3, dambreak=True),
    # spatial rain weight, closed box, three members
    "swe2d_rainweight": dict(ny=8, nx=10, dx=15.0, order=2, flux="hllc", batch=3,
                             bc=("closed", "closed", "closed", "closed"), rain_mmh=(120.0, 40.0, 75.0),
                             horton=True, storage=True, t0=0.0, steps=25, snap_at=(1, 25), seed=4, eta0=0.6,
                             rain_weight=True),
    # supercritical outflow through a stage edge over a steep slope, discharge inflow opposite
    "swe2d_steep": dict(ny=10, nx=16, dx=10.0, order=2, flux="hllc", batch=None,
                        bc=("discharge", "stage", "transmissive", "transmissive"), discharge_q=(1.5,),
                        stage=((-2.5,), 0.0, 0.0), rain_mmh=(20.0,), horton=False, storage=False, t0=0.0,
                        steps=50, snap_at=(1, 50), seed=5, slope=0.08, eta0=0.2),
}


def _hills(rng, ny, nx, dx, dy, n_hills=4, amp=(0.5, 2.5)):
    y = (np.arange(ny) + 0.5) * dy
    x = (np.arange(nx) + 0.5) * dx
    X, Y = np.meshgrid(x, y)
    z = 0.002 * Y
    for _ in range(n_hills):
        cx, cy = rng.uniform(0, nx * dx), rng.uniform(0, ny * dy)
        s = rng.uniform(0.15, 0.4) * max(nx * dx, ny * dy)
        z = z + rng.uniform(*amp) * np.exp(-((X - cx) ** 2 + (Y - cy) ** 2) / (2 * s * s))
    return z


def swe2d_inputs(spec) -> dict:
    rng = np.random.default_rng(spec["seed"])
    ny, nx, dx = spec["ny"], spec["nx"], spec["dx"]
    dy = spec.get("dy") or dx
    B = spec.get("batch")
    shp = (ny, nx) if B is None else (B, ny, nx)
    out = {}
    if spec.get("dambreak"):
        z = np.zeros((ny, nx))
        x = (np.arange(nx) + 0.5) * dx
        h0 = np.where(x < nx * dx / 2, 1.0, 0.0)[None, :].repeat(ny, 0)
    else:
        z = _hills(rng, ny, nx, dx, dy)
        if spec.get("slope"):
            z = z + spec["slope"] * ((np.arange(nx) + 0.5) * dx)[None, ::-1] - 2.0
        h0 = np.maximum(spec["eta0"] - z, 0.0)
        h0 = h0 * (rng.uniform(0.7, 1.3, size=h0.shape))
        h0[rng.uniform(size=h0.shape) < 0.15] = 0.0
    wet = h0 > 1e-3
    hu0 = np.where(wet, rng.normal(0, 0.05, size=h0.shape) * h0, 0.0)
    hv0 = np.where(wet, rng.normal(0, 0.05, size=h0.shape) * h0, 0.0)
    if B is not None:
        h0 = np.broadcast_to(h0, shp) * rng.uniform(0.9, 1.1, size=(B, 1, 1))
        hu0 = np.broadcast_to(hu0, shp).copy()
        hv0 = np.broadcast_to(hv0, shp).copy()
    out["z"] = z
    out["h0"] = np.ascontiguousarray(h0)
    out["hu0"] = np.ascontiguousarray(hu0)
    out["hv0"] = np.ascontiguousarray(hv0)
    out["n"] = rng.uniform(0.02, 0.06, size=shp)
    out["S"] = rng.uniform(0.0, 0.005, size=shp) if spec["storage"] else None
    if spec["horton"]:
        out["f0"] = rng.uniform(30, 90, size=shp) * MMH
        out["fc"] = rng.uniform(3, 10, size=shp) * MMH
        out["k"] = rng.uniform(2, 6, size=shp) / 3600.0
    else:
        out["f0"] = out["fc"] = out["k"] = None
    out["rain_weight"] = rng.uniform(0.5, 1.5, size=(ny, nx)) if spec.get("rain_weight") else None
    return out


def bc_value(spec, edge):
    kind = spec["bc"][EDGES.index(edge)]
    B = spec.get("batch")
    if kind == "stage":
        base, amp, w = spec["stage"]
        base = np.asarray(base, dtype=np.float64)

        def stage(t, base=base, amp=amp, w=w):
            v = base + amp * math.sin(w * t)
            return float(v[0]) if B is None else v
        return stage
    if kind == "discharge":
        q = np.asarray(spec["discharge_q"], dtype=np.float64)
        return float(q[0]) if B is None else q
    return None


def rain_value(spec, t):
    """Per-member rain (m/s), piecewise constant in 30 s blocks."""
    r = np.asarray(spec["rain_mmh"], dtype=np.float64) * MMH
    f = 1.0 if int(math.floor(t / 30.0 + 1e-9)) % 2 == 0 else 0.4
    v = r * f
    return float(v[0]) if spec.get("batch") is None else v


# ------------------------------------------------------------------------ 1-D
SWE1D_CASES = {
    # three reaches meeting at a level-pool junction: inflow, closed and stage ends
    "swe1d_net": dict(batch=None, gammas=None, slot_width_frac=1.0, steps=60, snap_at=(1, 20, 60),
                      init_depth=0.9),
    "swe1d_net_b2": dict(batch=2, gammas=((1.0, 1.0, 1.0), (1.3, 0.8, 1.1)), slot_width_frac=0.02, steps=50,
                         snap_at=(1, 50), init_depth=1.6),
}


def network(spec, mod=None):
    """Three reaches + one junction, in the reference's ChannelNetwork vocabulary.
    ``mod`` supplies Reach / Junction / ChannelNetwork (default: the reference's own)."""
    if mod is None:
        from hydrointel.domain import channels as mod
    Reach, Junction, ChannelNetwork = mod.Reach, mod.Junction, mod.ChannelNetwork

    def reach(rid, x, y, bed0, bed1, width, m, up, down, nman=0.03, bank=2.6):
        n = len(x)
        bed = np.linspace(bed0, bed1, n)
        return Reach(rid, np.asarray(x, float), np.asarray(y, float), bed, np.full(n, width), np.full(n, m),
                     np.full(n, nman), bed + bank, up, down)
    j = Junction(500.0, 500.0, 1.0, 12.0, 1.5, 0.03, 3.5, 24.0)
    a = reach("a", np.linspace(0, 440, 8), np.full(8, 500.0), 3.0, 1.2, 10.0, 1.0, ("inflow",), ("junction", 0))
    b = reach("b", np.full(6, 500.0), np.linspace(0, 440, 6), 2.4, 1.3, 6.0, 0.5, ("closed",), ("junction", 0),
              nman=0.035)
    c = reach("c", np.linspace(560, 1100, 10), np.full(10, 500.0), 0.9, -0.2, 14.0, 2.0, ("junction", 0),
              ("stage",), bank=3.0)
    return ChannelNetwork([a, b, c], [j], "a")


def inflow_fn(spec):
    B = spec.get("batch")

    def q(t):
        v = 4.0 + 30.0 * max(0.0, 1.0 - abs(t - 120.0) / 120.0)
        return v if B is None else np.array([v * (1.0 + 0.3 * i) for i in range(B)])
    return q


def stage_fn(spec):
    B = spec.get("batch")

    def s(t):
        v = 1.2 + 0.4 * math.sin(t / 90.0)
        return v if B is None else np.array([v + 0.1 * i for i in range(B)])
    return s


# ------------------------------------------------------------- exchange / coupled
EXCHANGE_CASES = {"exchange_overtop": dict(dx=100.0, seed=11, calls=6, dt=5.0)}

COUPLED_CASES = {"coupled_overtop": dict(dx=100.0, steps=80, t_end=7200.0, snap_at=(1, 40, 80))}


# Two members of the overtopping case batched in one reference CoupledEngine (one
# shared dt, as the reference steps a batch): per-member roughness, channel
# conveyance (apply_gamma), flooded-strip depth, initial channel level, inflow scale
# and rain.
COUPLED_BATCH_CASES = {"coupled_overtop_b2": dict(dx=100.0, steps=80, t_end=7200.0, snap_at=(1, 40, 80),
                                                  gamma=(1.0, 1.44), manning=(0.04, 0.055),
                                                  strip_depth=(0.4, 0.7), level_offset=(0.8, 1.1),
                                                  inflow_scale=(1.0, 0.6), rain_mmh=(90.0, 50.0))}


def rain_fn_batch(spec):
    r = np.asarray(spec["rain_mmh"], dtype=np.float64) * MMH

    def rain(t):
        return r.copy() if 60.0 <= t < 600.0 else np.zeros_like(r)
    return rain


def inflow_batch(spec):
    s = np.asarray(spec["inflow_scale"], dtype=np.float64)

    def q(t):
        return s * overtop_inflow(t)
    return q


def coupled_h0_batch(spec, z):
    return np.stack([coupled_h0(spec, z) * (d / 0.4) for d in spec["strip_depth"]])


def rain_fn_coupled(spec):
    def rain(t):
        return 90.0 * MMH if 60.0 <= t < 600.0 else 0.0
    return rain


def coupled_h0(spec, z):
    """A flooded strip beside the channel, so that water crosses the weirs both ways."""
    ny, nx = z.shape
    h0 = np.zeros_like(z)
    h0[ny // 2 - 2:ny // 2 + 2, : nx // 2] = 0.4
    return h0


def overtop_inflow(t):
    """Upstream hydrograph of the reference's overtopping case (benchmarks/suite.py:420-421)."""
    return 5.0 + (180.0 * max(0.0, 1.0 - abs(t - 1800.0) / 1800.0) if t < 5400.0 else 0.0)
