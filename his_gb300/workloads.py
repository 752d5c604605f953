"""Seeded synthetic storms: terrain, roughness, infiltration, retention, channel
network, weir links and forcing for the five named workloads.

* ``plain_small``   100 x 81 @ 80 m, float64, one reach of 40 rectangular sections
* ``plain_full``    400 x 325 @ 20 m, float64, 3 reaches / 160 trapezoidal sections
                    and a level-pool junction, ~1200 bank-cell links, Horton,
                    retention, 6 h alternating-block storm + 2.5 h recession, M2 tide,
                    inflow hydrograph peaking at 400 m^3/s
* ``batched_uniform`` 64 members on the full terrain, per-member roughness,
                    retention, infiltration, conveyance scale, rain, tide and inflow
* ``batched_uneven`` 48 members: 16 each at 100 x 81 @ 80 m, 200 x 163 @ 40 m and
                    400 x 325 @ 20 m, own terrain, durations U(1, 6) h
* ``served``        a Poisson request stream (2 req/s) of such storms

Terrain: a plane sloping 0.002 toward a sea boundary on the south edge, Gaussian
hills (amplitude U(2, 15) m, sigma U(200, 800) m) and a channel carved 3 m deep,
40 m wide (at least one cell) along a sinusoidal centreline.  Seeds come from a
sha256 of a key string (the reference's derive_seed, config.py:415-417).
"""
from __future__ import annotations

import hashlib
import math
from dataclasses import dataclass, field

import numpy as np

from .channels import ChannelNetwork, Junction, Reach, apply_gamma

MMH = 1.0 / 3.6e6
M2_PERIOD_S = 12.4206012 * 3600.0


def derive_seed(key: str) -> int:
    return int.from_bytes(hashlib.sha256(key.encode()).digest()[:4], "big")


def rng_for(key: str) -> np.random.Generator:
    return np.random.default_rng(derive_seed(key))


# ------------------------------------------------------------------------ forcing
@dataclass
class Forcing:
    """Closed-form forcing of one storm, evaluated identically on the host (drop-in
    path) and on the device (engine): rain blocks (m/s), harmonic tide, inflow table."""
    rain_t0: float = 0.0
    rain_step: float = 600.0
    rain: np.ndarray = field(default_factory=lambda: np.zeros(0))
    tide_base: float = 0.0
    tide_shift: float = 0.0
    tide_on: bool = True
    tide_amp: tuple = ()
    tide_w: tuple = ()
    tide_phase: tuple = ()
    q_t0: float = 0.0
    q_step: float = 60.0
    q: np.ndarray = field(default_factory=lambda: np.zeros(0))

    def rain_rate(self, t: float) -> float:
        if len(self.rain) == 0:
            return 0.0
        k = int(np.floor((t - self.rain_t0) / self.rain_step + 1e-9))
        if k < 0 or k >= len(self.rain):
            return 0.0
        return float(self.rain[k])

    def tide(self, t: float) -> float:
        tt = t + self.tide_shift
        eta = 0.0
        for a, w, p in zip(self.tide_amp, self.tide_w, self.tide_phase):
            eta = eta + a * math.cos(w * tt - p)
        return self.tide_base + (eta if self.tide_on else 0.0)

    def inflow(self, t: float) -> float:
        if len(self.q) == 0:
            return 0.0
        x = (t - self.q_t0) / self.q_step
        if x <= 0:
            return float(self.q[0])
        if x >= len(self.q) - 1:
            return float(self.q[-1])
        k = int(x)
        w = x - k
        return float((1 - w) * self.q[k] + w * self.q[k + 1])


class BatchForcing:
    """The forcing of B storms evaluated for all members at once (arrays over the
    members), with the arithmetic of Forcing per member: the same floor, clamp and
    interpolation steps in float64; the tide's cosines through numpy, which may differ
    from math.cos by an ulp."""

    def __init__(self, forcings: list[Forcing]):
        fs = list(forcings)
        self.B = len(fs)
        self.rain_t0 = np.array([f.rain_t0 for f in fs], np.float64)
        self.rain_step = np.array([f.rain_step for f in fs], np.float64)
        self.rain_n = np.array([len(f.rain) for f in fs], np.int64)
        self.rain = _ragged([f.rain for f in fs])
        self.tide_base = np.array([f.tide_base for f in fs], np.float64)
        self.tide_shift = np.array([f.tide_shift for f in fs], np.float64)
        self.tide_on = np.array([bool(f.tide_on) for f in fs])
        nh = max((len(f.tide_amp) for f in fs), default=0)
        pad = lambda xs: np.array([list(x) + [0.0] * (nh - len(x)) for x in xs], np.float64).reshape(self.B, nh)
        self.tide_amp = pad([f.tide_amp for f in fs])
        self.tide_w = pad([f.tide_w for f in fs])
        self.tide_phase = pad([f.tide_phase for f in fs])
        self.q_t0 = np.array([f.q_t0 for f in fs], np.float64)
        self.q_step = np.array([f.q_step for f in fs], np.float64)
        self.q_n = np.array([len(f.q) for f in fs], np.int64)
        self.q = _ragged([f.q for f in fs])
        self._rows = np.arange(self.B)

    def rain_rate(self, t: float) -> np.ndarray:
        k = np.floor((t - self.rain_t0) / self.rain_step + 1e-9).astype(np.int64)
        ok = (k >= 0) & (k < self.rain_n)
        return np.where(ok, self.rain[self._rows, np.clip(k, 0, max(self.rain.shape[1] - 1, 0))], 0.0) \
            if self.rain.shape[1] else np.zeros(self.B)

    def tide(self, t: float) -> np.ndarray:
        tt = t + self.tide_shift
        eta = np.zeros(self.B)
        for j in range(self.tide_amp.shape[1]):      # harmonics in order, as Forcing.tide sums them
            eta = eta + self.tide_amp[:, j] * np.cos(self.tide_w[:, j] * tt - self.tide_phase[:, j])
        return self.tide_base + np.where(self.tide_on, eta, 0.0)

    def inflow(self, t: float) -> np.ndarray:
        if not self.q.shape[1]:
            return np.zeros(self.B)
        x = (t - self.q_t0) / self.q_step
        last = np.maximum(self.q_n - 1, 0)
        k = np.clip(x.astype(np.int64), 0, np.maximum(last - 1, 0))
        w = x - k
        mid = (1 - w) * self.q[self._rows, k] + w * self.q[self._rows, np.minimum(k + 1, last)]
        out = np.where(x <= 0, self.q[:, 0], np.where(x >= last, self.q[self._rows, last], mid))
        return np.where(self.q_n > 0, out, 0.0)


def _ragged(rows) -> np.ndarray:
    """Rows of different lengths as one zero-padded (B, max length) array."""
    n = max((len(r) for r in rows), default=0)
    out = np.zeros((len(rows), n))
    for i, r in enumerate(rows):
        out[i, :len(r)] = r
    return out


def alternating_block(duration_s: float, step_s: float, peak_mmh: float, position: float = 0.5) -> np.ndarray:
    """Alternating-block hyetograph from a generic IDF depth curve D(d) = i(d) d,
    i(d) = 1 / (d + 10 min)^0.75, blocks placed alternately about the peak position
    and rescaled so the peak block is ``peak_mmh`` (the block arrangement of the
    reference's hyetograph.alternating_block, hyetograph.py:58-81)."""
    n = max(1, int(round(duration_s / step_s)))          # a storm shorter than a block is one block
    d = step_s / 60.0 * np.arange(1, n + 1)
    cum = d / (d + 10.0) ** 0.75
    blocks = np.diff(np.concatenate([[0.0], cum]))
    order = np.argsort(-blocks)
    out = np.zeros(n)
    centre = int(np.clip(round(position * (n - 1)), 0, n - 1))
    pos = [centre]
    left, right = centre - 1, centre + 1
    for k in range(1, n):
        if (k % 2 == 1 and right < n) or left < 0:
            pos.append(right)
            right += 1
        else:
            pos.append(left)
            left -= 1
    for rank, p in zip(order, pos):
        out[p] = blocks[rank]
    return out / out.max() * peak_mmh * MMH


def triangular_rain(rise_s: float, step_s: float, peak_mmh: float) -> np.ndarray:
    n = int(round(rise_s / step_s))
    mid = (np.arange(n) + 0.5) * step_s
    return peak_mmh * MMH * np.maximum(0.0, 1.0 - np.abs(mid - rise_s / 2) / (rise_s / 2))


def triangular_inflow(t_end: float, peak: float, base: float, t_peak: float, half_width: float,
                      step_s: float = 60.0) -> np.ndarray:
    t = np.arange(int(np.ceil(t_end / step_s)) + 1) * step_s
    return base + (peak - base) * np.maximum(0.0, 1.0 - np.abs(t - t_peak) / half_width)


def m2_tide(amp: float, t_high: float) -> dict:
    w = 2 * math.pi / M2_PERIOD_S
    return dict(tide_amp=(amp,), tide_w=(w,), tide_phase=(0.0,), tide_shift=-t_high)


# ------------------------------------------------------------------------ terrain
@dataclass
class Terrain:
    nx: int
    ny: int
    dx: float
    z: np.ndarray              # carved bed used by the 2-D model
    z_plain: np.ndarray        # bed before carving (bank level of the channel)
    carved: np.ndarray         # bool mask of carved channel cells
    paths: dict                # reach id -> (x, y) polyline of the channel centreline
    junction: tuple | None


def _centreline_x(y, lx, ly):
    return 0.5 * lx + 0.15 * lx * np.sin(2 * np.pi * y / ly)


def make_terrain(nx: int, ny: int, dx: float, n_hills: int, key: str, network: str = "single") -> Terrain:
    rng = rng_for(f"terrain/{key}")
    lx, ly = nx * dx, ny * dx
    x = (np.arange(nx) + 0.5) * dx
    y = (np.arange(ny) + 0.5) * dx
    X, Y = np.meshgrid(x, y)
    z = 0.002 * Y
    for _ in range(n_hills):
        a, s = rng.uniform(2.0, 15.0), rng.uniform(200.0, 800.0)
        cx, cy = rng.uniform(0, lx), rng.uniform(0, ly)
        z = z + a * np.exp(-((X - cx) ** 2 + (Y - cy) ** 2) / (2 * s * s))
    half = max(20.0, 0.5 * dx)
    ys = np.linspace(ly - 0.5 * dx, 0.5 * dx, 400)
    main = np.stack([_centreline_x(ys, lx, ly), ys], axis=1)
    paths, junction = {}, None
    polylines = [main]
    if network == "single":
        paths["main"] = main
    else:
        yj = 0.4 * ly
        xj = float(_centreline_x(np.array([yj]), lx, ly)[0])
        junction = (xj, yj)
        paths["upper"] = main[main[:, 1] > yj + dx]
        paths["lower"] = main[main[:, 1] < yj - dx]
        t = np.linspace(0.0, 1.0, 200)[:, None]
        start = np.array([0.95 * lx, 0.65 * ly])
        trib = start + t * (np.array([xj, yj]) - start)
        paths["trib"] = trib[np.hypot(trib[:, 0] - xj, trib[:, 1] - yj) > dx]
        polylines.append(trib)
    carved = np.zeros((ny, nx), dtype=bool)
    r = int(np.ceil(half / dx)) + 1            # the disc of each point lies in this window
    for pl in polylines:
        for px, py in pl[:: max(1, len(pl) // 400)]:
            i0, j0 = int(px / dx), int(py / dx)
            ia, ib = max(i0 - r, 0), min(i0 + r + 1, nx)
            ja, jb = max(j0 - r, 0), min(j0 + r + 1, ny)
            if ia < ib and ja < jb:
                carved[ja:jb, ia:ib] |= np.hypot(X[ja:jb, ia:ib] - px, Y[ja:jb, ia:ib] - py) < half
    # the main channel is also carved row by row, so no row is skipped on coarse grids
    carved |= np.abs(X - _centreline_x(Y, lx, ly)) < half
    z_plain = z.copy()
    zc = np.where(carved, z - 3.0, z)
    return Terrain(nx, ny, dx, zc, z_plain, carved, paths, junction)


def _sample(ter: Terrain, xs, ys):
    i = np.clip((np.asarray(xs) / ter.dx).astype(int), 0, ter.nx - 1)
    j = np.clip((np.asarray(ys) / ter.dx).astype(int), 0, ter.ny - 1)
    return ter.z_plain[j, i]


def _resample(pl: np.ndarray, n: int) -> np.ndarray:
    seg = np.hypot(np.diff(pl[:, 0]), np.diff(pl[:, 1]))
    s = np.concatenate([[0.0], np.cumsum(seg)])
    t = np.linspace(0.0, s[-1], n)
    return np.stack([np.interp(t, s, pl[:, 0]), np.interp(t, s, pl[:, 1])], axis=1)


def make_network(ter: Terrain, kind: str, gamma=None) -> ChannelNetwork:
    """One reach of 40 rectangular sections (kind 'single') or three trapezoidal
    reaches of 60 + 40 + 60 sections meeting at a level-pool junction."""
    def reach(rid, pl, n, b, m, up, down):
        p = _resample(pl, n)
        bank = _sample(ter, p[:, 0], p[:, 1])
        bed = bank - 3.0
        return Reach(rid, p[:, 0].copy(), p[:, 1].copy(), bed, np.full(n, b), np.full(n, m), np.full(n, 0.03),
                     bank, up, down)
    if kind == "single":
        net = ChannelNetwork([reach("main", ter.paths["main"], 40, 30.0, 0.0, ("inflow",), ("stage",))], [], "main")
    else:
        xj, yj = ter.junction
        bank_j = float(_sample(ter, [xj], [yj])[0])
        j = Junction(xj, yj, bank_j - 3.0, 20.0, 2.0, 0.03, bank_j, 40.0)
        net = ChannelNetwork([reach("upper", ter.paths["upper"], 60, 20.0, 2.0, ("inflow",), ("junction", 0)),
                              reach("trib", ter.paths["trib"], 40, 12.0, 2.0, ("closed",), ("junction", 0)),
                              reach("lower", ter.paths["lower"], 60, 20.0, 2.0, ("junction", 0), ("stage",))],
                             [j], "upper")
    net.validate()
    if gamma is not None:
        net = apply_gamma(net, np.full(net.n_reaches, float(gamma)))
    return net


def bank_links(ter: Terrain, topo) -> tuple[np.ndarray, np.ndarray, float]:
    """Every uncarved cell 8-adjacent to the carved channel, linked to the nearest 1-D
    interior cell; weir length = the cell edge length."""
    c = ter.carved
    nb = np.zeros_like(c)
    for dj in (-1, 0, 1):
        for di in (-1, 0, 1):
            if dj or di:
                nb[max(dj, 0):c.shape[0] + min(dj, 0), max(di, 0):c.shape[1] + min(di, 0)] |= \
                    c[max(-dj, 0):c.shape[0] + min(-dj, 0), max(-di, 0):c.shape[1] + min(-di, 0)]
    bank = nb & ~c
    jj, ii = np.nonzero(bank)
    cx, cy = (ii + 0.5) * ter.dx, (jj + 0.5) * ter.dx
    interior = np.nonzero(topo.kind <= 1)[0]
    px, py = topo.x[interior], topo.y[interior]
    d2 = (cx[:, None] - px[None, :]) ** 2 + (cy[:, None] - py[None, :]) ** 2
    near = interior[np.argmin(d2, axis=1)]
    order = np.argsort(jj * ter.nx + ii, kind="stable")
    return near[order], (jj * ter.nx + ii)[order], ter.dx


def normal_depth(topo, sec: dict, Q: float, slope_min: float = 1e-4) -> np.ndarray:
    """Manning normal depth for discharge Q in every cell by 60 bisections
    (engine.py:78-101)."""
    z = np.asarray(sec["z"] if "z" in sec else topo.z, dtype=float)
    s = np.full(z.shape, slope_min)
    for ri in np.unique(topo.reach_of[topo.reach_of >= 0]):
        idx = np.nonzero((topo.reach_of == ri) & (topo.kind == 0))[0]
        if len(idx) > 1:
            dz = -np.gradient(z[idx], topo.chain[idx])
            s[idx] = np.maximum(dz, slope_min)
    b, m, yb, ts = sec["b"], sec["m"], sec["yb"], sec["ts"]
    lo, hi = np.zeros_like(z), np.broadcast_to(yb, z.shape).copy()
    for _ in range(60):
        mid = 0.5 * (lo + hi)
        yt = np.minimum(mid, yb)
        A = yt * (b + m * yt) + ts * np.maximum(mid - yb, 0.0)
        P = b + 2.0 * yt * np.sqrt(1.0 + m * m)
        q = A * (A / P) ** (2 / 3) * np.sqrt(s) / topo.n
        lo, hi = np.where(q < Q, mid, lo), np.where(q < Q, hi, mid)
    return 0.5 * (lo + hi)


# ------------------------------------------------------------------------ storms
@dataclass
class Storm:
    """One storm: everything a member of the engine needs (host arrays)."""
    key: str
    terrain: Terrain
    manning: float | np.ndarray
    storage: np.ndarray | None
    horton: tuple | None               # (f0, fc, k, t0) in m/s, m/s, 1/s, s
    forcing: Forcing
    t_end: float
    network: ChannelNetwork | None
    slot_width_frac: float = 1.0
    bc: tuple = ("transmissive", "transmissive", "stage", "transmissive")
    sea_frac: float = 0.04

    @property
    def cells(self) -> int:
        return self.terrain.nx * self.terrain.ny

    def h0(self) -> np.ndarray:
        """Sea cells (the southern strip below the initial tide) at the tide level."""
        ter = self.terrain
        eta0 = self.forcing.tide(0.0)
        y = (np.arange(ter.ny) + 0.5) * ter.dx
        sea = (y < self.sea_frac * ter.ny * ter.dx)[:, None] & (ter.z < eta0)
        return np.where(sea, np.maximum(eta0 - ter.z, 0.0), 0.0)


def plain_small(key: str = "plain_small") -> Storm:
    ter = make_terrain(100, 81, 80.0, 12, key, "single")
    rain = triangular_rain(1800.0, 60.0, 60.0)
    f = Forcing(rain_t0=0.0, rain_step=60.0, rain=rain, tide_base=0.5, tide_on=False,
                q_t0=0.0, q_step=60.0, q=np.array([2.0, 2.0]))
    net = make_network(ter, "single")
    return Storm(key, ter, 0.035, None, None, f, 3600.0, net, slot_width_frac=0.01 / 30.0)


def _full_forcing(rng, rain_peak=120.0, tide_amp=1.2, q_peak=400.0, duration_s=6 * 3600.0,
                  recession_s=2.5 * 3600.0) -> tuple[Forcing, float]:
    t_end = duration_s + recession_s
    rain = alternating_block(duration_s, 600.0, rain_peak)
    t_peak = 0.5 * duration_s
    f = Forcing(rain_t0=0.0, rain_step=600.0, rain=rain, tide_base=0.0, tide_on=True,
                q_t0=0.0, q_step=60.0, q=triangular_inflow(t_end, q_peak, 0.05 * q_peak, t_peak + 1800.0,
                                                             0.5 * duration_s),
                **m2_tide(tide_amp, t_peak))
    return f, t_end


def plain_full(key: str = "plain_full") -> Storm:
    ter = make_terrain(400, 325, 20.0, 24, key, "triple")
    f, t_end = _full_forcing(rng_for(f"forcing/{key}"))
    shp = (ter.ny, ter.nx)
    horton = (np.full(shp, 60.0 * MMH), np.full(shp, 8.0 * MMH), np.full(shp, 4.0 / 3600.0), 0.0)
    return Storm(key, ter, 0.035, np.full(shp, 0.005), horton, f, t_end, make_network(ter, "triple"))


def batched_uniform(n: int = 64, key: str = "plain_full") -> list[Storm]:
    """Members on the shared full-resolution terrain with per-member draws."""
    ter = make_terrain(400, 325, 20.0, 24, key, "triple")
    shp = (ter.ny, ter.nx)
    out = []
    for b in range(n):
        r = rng_for(f"member/{key}/{b}")
        nm, S, f0 = r.uniform(0.02, 0.06), r.uniform(0.0, 0.010), r.uniform(30.0, 90.0)
        gamma, rain_pk, tide_a, q_pk = r.uniform(0.7, 1.3), r.uniform(40, 150), r.uniform(0.5, 1.5), \
            r.uniform(100, 600)
        f, t_end = _full_forcing(r, rain_pk, tide_a, q_pk)
        horton = (np.full(shp, f0 * MMH), np.full(shp, 8.0 * MMH), np.full(shp, 4.0 / 3600.0), 0.0)
        out.append(Storm(f"{key}/{b}", ter, nm, np.full(shp, S), horton, f, t_end,
                         make_network(ter, "triple", gamma)))
    return out


SIZES = ((100, 81, 80.0, 12), (200, 163, 40.0, 18), (400, 325, 20.0, 24))


def uneven_member(key: str, size_index: int, duration_s: float) -> Storm:
    nx, ny, dx, hills = SIZES[size_index]
    ter = make_terrain(nx, ny, dx, hills, key, "triple")
    r = rng_for(f"forcing/{key}")
    storm_s = 0.7 * duration_s
    f, _ = _full_forcing(r, r.uniform(40, 150), r.uniform(0.5, 1.5), r.uniform(100, 600), storm_s,
                         duration_s - storm_s)
    shp = (ny, nx)
    horton = (np.full(shp, r.uniform(30, 90) * MMH), np.full(shp, 8.0 * MMH), np.full(shp, 4.0 / 3600.0), 0.0)
    return Storm(key, ter, r.uniform(0.02, 0.06), np.full(shp, r.uniform(0.0, 0.010)), horton, f, duration_s,
                 make_network(ter, "triple", r.uniform(0.7, 1.3)))


def batched_uneven(per_size: int = 16, key: str = "uneven") -> list[Storm]:
    out = []
    for s in range(3):
        for k in range(per_size):
            d = rng_for(f"duration/{key}/{s}/{k}").uniform(1.0, 6.0) * 3600.0
            out.append(uneven_member(f"{key}/{s}/{k}", s, d))
    return out


def served_requests(rate_per_s: float = 2.0, horizon_s: float = 600.0, key: str = "served"):
    """Poisson arrivals: (arrival time, size index, duration) per request."""
    r = rng_for(f"arrivals/{key}")
    t, out = 0.0, []
    while True:
        t += r.exponential(1.0 / rate_per_s)
        if t > horizon_s:
            return out
        out.append((t, int(r.integers(0, 3)), r.uniform(0.5, 6.0) * 3600.0))
