"""Drop-in 1-D <-> 2-D coupling and time loop: the reference's ``Links``,
``build_links``, ``exchange`` and ``CoupledEngine`` (hydrointel/solver/coupling.py)
over the CUDA 2-D and 1-D solvers.

Exchange per link (positive = 2-D -> 1-D): free weir Q = Cw L h^1.5, Villemonte
submergence (1 - (d_down/d_up)^1.5)^0.385, relaxation to half the level-equalising
volume and donor limits of half the volume above the bank, applied in place by the
exchange kernel before the 2-D step.
"""
from __future__ import annotations

import ctypes as C
import logging
import math
import time
from dataclasses import dataclass, field

import numpy as np
import torch

from . import _lib
from ._lib import NumericalInstabilityError
from .boundaries import edge_values
from .config import SolverConfig
from .massbalance import MassBalance
from .swe1d import SWE1D, Step1DVolumes
from .swe2d import SWE2D, StepVolumes

log = logging.getLogger("his_gb300.solver")

MAX_PLAUSIBLE_DEPTH_2D_M = 10.0
MAX_PLAUSIBLE_RISE_1D_M = 10.0


class Links:
    """Link arrays (per link: 1-D cell, bank crest, weir length, 2-D bed; unique linked 2-D
    cells), shared by every member, plus the device handle binding a grid set and a network."""

    def __init__(self, cell1d, zbank, length, z2, inv, uniq, one: SWE1D, two: SWE2D):
        own = lambda a, dt=None: torch.from_numpy(np.array(a, dtype=dt))     # a private copy
        self.cell1d = own(cell1d, np.int64)
        self.zbank = own(zbank, np.float64)
        self.length = own(length, np.float64)
        self.z2 = own(z2, np.float64)
        self.inv = own(inv, np.int64)
        self.uniq_dev = own(uniq, np.int64)
        self.n_unique = int(len(self.uniq_dev))
        if one.B != two.B:
            raise ValueError(f"the 2-D model is batched {two.batch} and the 1-D model {one.batch}; they must match")
        self._host = {"cell1d": _lib.host_array(cell1d, np.int32), "inv": _lib.host_array(inv, np.int32),
                      "uniq": _lib.host_array(uniq, np.int64), "zbank": _lib.host_array(zbank, np.float64),
                      "length": _lib.host_array(length, np.float64), "z2": _lib.host_array(z2, np.float64)}
        n = len(self._host["cell1d"])
        for k in ("inv", "zbank", "length", "z2"):
            if len(self._host[k]) != n:
                raise ValueError(f"link array '{k}' has {len(self._host[k])} entries, expected {n}")
        descs = (_lib.LinksDesc * one.B)()
        for b in range(one.B):
            d = descs[b]
            d.n_links, d.n_unique = n, self.n_unique
            for k, v in self._host.items():
                setattr(d, k, _lib.as_p(v))
        self._lib = _lib.load()
        self._handle = C.c_void_p()
        self.B = one.B
        self.n_links = n
        with _lib.on_device(two.device):
            _lib.check(self._lib.his_links_create(two._handle, one._handle, one.B, descs, C.byref(self._handle)),
                       "his_links_create")
        self._owners = (one, two)

    def __del__(self):
        h = getattr(self, "_handle", None)
        if h is not None and h.value and _lib._LIB is not None:
            _lib._LIB.his_links_destroy(h)
            self._handle = C.c_void_p()

    def cfg_struct(self, cfg: SolverConfig):
        """his_solver_cfg for his_exchange, rebuilt only when one of the three values
        the exchange reads (weir_cw, exchange_limit, exchange_relax) changes."""
        key = (cfg.weir_cw, cfg.exchange_limit, cfg.exchange_relax)
        if getattr(self, "_cfg_key", None) != key:
            self._cfg_c, self._cfg_key = _lib.solver_cfg(cfg), key
        return self._cfg_c

    def exchanged(self, reset: bool = False) -> np.ndarray:
        out = np.zeros((self.B, 2))
        _lib.check(self._lib.his_links_exchanged(self._handle, _lib.as_p(out), int(reset), _lib.stream_handle()),
                   "his_links_exchanged")
        return out


def build_links(one: SWE1D, two: SWE2D) -> Links:
    """One link per interior 1-D cell, to the 2-D cell containing it; weir length twice the
    1-D cell length (both banks) (coupling.py:60-70)."""
    tp = one.topo
    idx = np.nonzero(tp.kind <= 1)[0]
    i = np.clip((tp.x[idx] / two.dx).astype(int), 0, two.nx - 1)
    j = np.clip((tp.y[idx] / two.dy).astype(int), 0, two.ny - 1)
    flat = j * two.nx + i
    uniq, inv = np.unique(flat, return_inverse=True)
    z2 = two.z.reshape(-1)[torch.as_tensor(flat, device=two.device)].double().cpu().numpy()
    return Links(idx, tp.zbank[idx], 2.0 * tp.dx[idx], z2, inv, uniq, one, two)


def links_from_cells(one: SWE1D, two: SWE2D, cell1d, cells2d, length) -> Links:
    """Links for an explicit list of (1-D cell, flat 2-D cell, weir length) triples, e.g.
    every bank cell of a channel mapped to its nearest 1-D cell."""
    cell1d = np.asarray(cell1d, dtype=np.int64)
    cells2d = np.asarray(cells2d, dtype=np.int64)
    uniq, inv = np.unique(cells2d, return_inverse=True)
    z2 = two.z.reshape(-1)[torch.as_tensor(cells2d, device=two.device)].double().cpu().numpy()
    return Links(cell1d, one.topo.zbank[cell1d], np.broadcast_to(np.asarray(length, float), cell1d.shape), z2, inv,
                 uniq, one, two)


def exchange(one: SWE1D, two: SWE2D, links: Links, dt: float, cfg: SolverConfig, volumes: bool = True,
             stream: int | None = None):
    """Move water between the models in place; per-link volumes (m^3, + = 2-D -> 1-D)
    as a float64 device tensor, enqueued on ``stream`` (default: the current stream)
    without waiting for it (coupling.py:73-124).  ``volumes=False`` skips them (the
    coupled step discards them)."""
    V = torch.empty((links.B, links.n_links), dtype=torch.float64, device=two.device) if volumes else None
    cfgc = links.cfg_struct(cfg)
    one._kernel_writes += 1
    two._kernel_writes += 1
    with _lib.on_device(two.device):
        _lib.check(links._lib.his_exchange_async(links._handle, C.byref(cfgc), float(dt),
                                                 V.data_ptr() if V is not None and V.numel() else None,
                                                 _lib.stream_handle() if stream is None else stream),
                   "his_exchange_async")
    if V is None:
        return None
    return V if one.batch is not None else V[0]


@dataclass
class Snapshot:
    t: float
    h: np.ndarray
    u: np.ndarray
    v: np.ndarray
    eta1: np.ndarray
    q1: np.ndarray
    ledger: dict = field(default_factory=dict)


@dataclass
class RunLog:
    steps: int = 0
    wall_s: float = 0.0
    dt_min: float = math.inf
    dt_max: float = 0.0
    n_sub_max: int = 0
    n_dt_clamped: int = 0
    exchanged_in_m3: float = 0.0
    exchanged_out_m3: float = 0.0
    series: list = field(default_factory=list)


class CoupledEngine:
    """Coupled 1-D/2-D time loop with mass accounting and snapshot output (coupling.py:151-286)."""

    def __init__(self, two: SWE2D, one: SWE1D | None, cfg: SolverConfig, rain=None, links: Links | None = None):
        self.two, self.one, self.cfg = two, one, cfg
        self.rain = rain or (lambda t: 0.0)
        if one is not None and one.batch != two.batch:
            raise ValueError(f"the 2-D model is batched {two.batch} and the 1-D model {one.batch}; they must match")
        self.links = (links or build_links(one, two)) if one is not None else None
        if self.links is not None:
            self.links.exchanged(reset=True)
        self.batch = two.batch
        self.bshape = two.bshape
        self.mb = MassBalance(two.device, self.total_volume())
        self.log = RunLog()
        self._last_dt = 0.0
        # CFL rates of both models land in one pinned buffer: one wait per step
        self._rates = torch.zeros(3 * two.B, dtype=torch.float64, pin_memory=True)
        # the 1-D substeps overlap the 2-D step (disjoint state once the exchange is done)
        self._side = torch.cuda.Stream(two.device) if one is not None else None
        self._exchanged = torch.cuda.Event() if one is not None else None
        # the step kernels add their volume terms straight into the mass balance's device
        # ledger: no copy and no extra kernel per step
        self._ledger = self.mb.device_ledger(two.device)
        # state version of the 1-D model when its rates were last reduced ahead, and of
        # the 2-D model when a step of this engine last left its rates (None: not)
        self._rates1_at = None
        self._rates2_at = None

    def plausibility(self) -> np.ndarray:
        """Per member (rows): the largest 2-D depth and the highest 1-D water level above
        its bank crest over interior cells (NaN where a model is absent), reduced on the
        device and copied to the host in one transfer."""
        two, one = self.two, self.one
        cols = [two.h.reshape(two.B, -1).amax(dim=1).double()]
        if one is not None:
            above = one.z + one.sec.depth(one.A) - torch.as_tensor(one.topo.zbank, dtype=one.A.dtype,
                                                                  device=one.A.device)
            above = torch.where(one.interior, above, torch.full_like(above, -math.inf)).reshape(one.B, -1)
            cols.append(above.amax(dim=1).double().to(two.device))
        stats = torch.stack(cols, dim=1).cpu().numpy()
        if one is None:
            stats = np.concatenate([stats, np.full((two.B, 1), np.nan)], axis=1)
        return stats

    def check_plausible(self, t: float, label: str = "") -> None:
        """Raise NumericalInstabilityError naming every member whose state left the
        physically possible range: a non-finite or deeper than 10 m 2-D cell, or a 1-D
        level non-finite or more than 10 m above the bank (coupling.py:169-192)."""
        stats = self.plausibility()
        limits = np.array([MAX_PLAUSIBLE_DEPTH_2D_M, MAX_PLAUSIBLE_RISE_1D_M])
        broken = np.isnan(stats[:, 0]) | np.isinf(stats[:, 0]) | (stats[:, 0] > limits[0])
        if self.one is not None:
            broken |= ~np.isfinite(stats[:, 1]) | (stats[:, 1] > limits[1])
        if not broken.any():
            return
        fmt = lambda m: (f"{'member %d: ' % m if self.batch is not None else ''}max 2-D depth {stats[m, 0]:.2f} m, "
                         f"max 1-D rise above bank {stats[m, 1]:.2f} m")
        where = f" in {label}" if label else ""
        raise NumericalInstabilityError(
            f"physically impossible state{where} at t = {t / 3600:.3f} h "
            f"({', '.join(fmt(int(m)) for m in np.flatnonzero(broken))}; bounds {limits[0]:g} m and "
            f"{limits[1]:g} m). The run is invalid.")

    def total_volume(self):
        v = self.two.volume() + self.two.storage_volume()
        if self.one is not None:
            v = v + self.one.volume().to(v.device)
        v = v.cpu()
        return v if self.batch is not None else float(v)

    def _enqueue_rates(self, need2: bool, need1: bool, stream: int) -> None:
        """Both CFL rates of the current state, into one pinned buffer, on ``stream``.
        The 2-D rates are those the last step's own last stage formed, and the 1-D
        rates those reduced ahead on the side stream at the end of the last step,
        unless the state has been written since (state versions); then they are
        reduced afresh."""
        B = self.two.B
        with _lib.on_device(self.two.device):
            if need2:
                if self._rates2_at is not None and self._rates2_at == self.two.state_version():
                    self.two.step_rate_async(self._rates[:B], stream)
                else:
                    self.two.rates_async(self._rates[:B], stream)
            if need1 and self._rates1_at != self.one.state_version():
                self.one.rates_async(self._rates[B:], stream)
        self._rates1_at = None

    def _wait_rates(self, main):
        """Largest 2-D rate and (largest 1-D rate, any wet), after one wait for ``main``."""
        B = self.two.B
        main.synchronize()
        r = self._rates.numpy()
        rw = r[B:].reshape(B, 2)
        return float(r[:B].max()), float(rw[:, 0].max()), bool((rw[:, 1] > 0).any())

    def step(self, t: float, t_limit: float, dt: float | None = None, n_sub: int | None = None) -> float:
        """One coupled step (coupling.py:205-230): CFL dt and 1-D substep count, the
        exchange, the 2-D step and the 1-D substeps, mass terms added on the device by
        the step kernels themselves.
        The step waits on the GPU once, for the CFL rates; the 1-D substeps run on a
        side stream beside the 2-D step and join before the step returns."""
        two, one = self.two, self.one
        need1 = one is not None and n_sub is None
        wait = dt is None or need1
        main = torch.cuda.current_stream(two.device)       # looked up once per step
        ms = main.cuda_stream
        if wait:
            self._enqueue_rates(dt is None, need1, ms)
        # forcing at t does not depend on dt: evaluated while the GPU reduces
        rain_t = self.rain(t)
        edges_t = edge_values(two.bcs, t)
        if wait:
            r2, r1, wet1 = self._wait_rates(main)
        dt = min(two.dt_from_rate(r2) if dt is None else dt, t_limit - t)
        if one is not None:
            if n_sub is None:
                n_sub = max(1, math.ceil(dt / one.dt_from_rate(r1, wet1) - 1e-9))
            exchange(one, two, self.links, dt, self.cfg, volumes=False, stream=ms)
            self._exchanged.record(main)
        two.step_ledger(dt, t, rain_t, edges_t, self._ledger.data_ptr(), ms)
        self._rates2_at = two.state_version()        # its last stage formed the new state's rates
        if one is not None:
            # after the 2-D launch, so the host prepares the substeps while it runs;
            # the next step's 1-D rates are reduced right behind them, beside the 2-D
            side = self._side
            side.wait_event(self._exchanged)
            one.substeps_ledger(dt, t, n_sub, self._ledger.data_ptr(), side.cuda_stream)
            one.rates_async(self._rates[two.B:], side.cuda_stream)
            self._rates1_at = one.state_version()
        if one is not None:
            main.wait_stream(self._side)
            self.log.n_sub_max = max(self.log.n_sub_max, n_sub)
            self._last_n_sub = n_sub
        self.log.steps += 1
        self._last_dt = dt
        self.log.dt_min = min(self.log.dt_min, dt)
        self.log.dt_max = max(self.log.dt_max, dt)
        return t + dt

    def snapshot(self, t: float) -> Snapshot:
        """The state at ``t`` as host float32 arrays (depth, KP velocities, 1-D level and
        discharge) and the volume ledger (2-D surface, 1-D channel and retained water
        plus the accumulated terms), gathered with non-blocking copies into pinned
        memory and one wait (coupling.py:229-242)."""
        two, one = self.two, self.one
        u, v = two.velocities(two.h, two.hu, two.hv)
        parts = {"h": two.h, "u": u, "v": v}
        if one is not None:
            parts.update(eta1=one.level(), q1=one.Q)
        vols = {"v2d": two.volume(), "storage": two.storage_volume()}
        if one is not None:
            vols["v1d"] = one.volume()
        host = {}
        for name, x in list(parts.items()) + list(vols.items()):
            dt = torch.float64 if name in vols else torch.float32
            dst = torch.empty(x.shape, dtype=dt, pin_memory=True)
            dst.copy_(x.detach().to(dt), non_blocking=True)
            host[name] = dst
        torch.cuda.current_stream(two.device).synchronize()
        as_num = (lambda a: a.numpy()) if self.batch is not None else (lambda a: float(a))
        ledger = {"v2d": as_num(host["v2d"]), "v1d": as_num(host["v1d"]) if one is not None else 0.0,
                  "storage": as_num(host["storage"])}
        ledger.update(self.mb.sources())
        empty = np.zeros(0, np.float32)
        return Snapshot(t, host["h"].numpy(), host["u"].numpy(), host["v"].numpy(),
                        host["eta1"].numpy() if one is not None else empty,
                        host["q1"].numpy() if one is not None else empty, ledger)

    def run(self, t_end: float, out_times=(), t0: float = 0.0, on_snapshot=None, check_every: int = 500,
            label: str = "", progress_s: float = 120.0):
        """Advance from t0 to t_end; each requested output time cuts a step and, with
        ``on_snapshot``, hands it the snapshot there.  The state is checked for
        plausibility at every output and every ``check_every`` steps (when the mass
        series also gets an entry), and at the end, where the mass balance must hold
        to cfg.mass_tol; returns the final relative mass errors (coupling.py:244-286).
        Every ``progress_s`` s of wall time a progress line is logged."""
        clock0 = time.perf_counter()
        schedule = _OutputSchedule(out_times, t0, t_end)
        report = _Progress(label, t0, t_end, progress_s)
        t = t0
        if schedule.due(t0) and on_snapshot is not None:
            on_snapshot(self.snapshot(t0))
        if schedule.due(t0):
            schedule.advance()
        n = 0
        while t < t_end - 1e-9:
            t = self.step(t, schedule.limit(t_end))
            n += 1
            at_output = schedule.due(t)
            periodic = n % check_every == 0
            if at_output or periodic:
                self.check_plausible(t, label)
            if at_output:
                if on_snapshot is not None:
                    on_snapshot(self.snapshot(t))
                schedule.advance()
            if periodic:
                self.mb.check(self.total_volume(), t)
            report.maybe(t, self.log)
        self.log.wall_s += time.perf_counter() - clock0
        if self.links is not None:
            totals = self.links.exchanged()
            pick = (lambda col: totals[:, col]) if self.batch is not None else (lambda col: float(totals[0, col]))
            self.log.exchanged_in_m3, self.log.exchanged_out_m3 = pick(0), pick(1)
        self.log.n_dt_clamped = self.two.n_dt_clamped
        self.check_plausible(t, label)
        return self.mb.assert_ok(self.total_volume(), t, self.cfg.mass_tol, label)


class _OutputSchedule:
    """Requested output times within [t0, t_end], in order; the next one limits a step."""

    def __init__(self, times, t0: float, t_end: float):
        self._times = sorted(float(x) for x in times if t0 <= x <= t_end + 1e-9)
        self._k = 0

    def due(self, t: float) -> bool:
        return self._k < len(self._times) and t >= self._times[self._k] - 1e-9

    def advance(self) -> None:
        self._k += 1

    def limit(self, t_end: float) -> float:
        return self._times[self._k] if self._k < len(self._times) else t_end


class _Progress:
    """Logs how far a long run has got, at most every ``period`` s of wall time."""

    def __init__(self, label: str, t0: float, t_end: float, period: float):
        self.prefix = f"{label}: " if label else ""
        self.t0, self.span, self.period = t0, t_end - t0, period
        self.start = self.last = time.perf_counter()

    def maybe(self, t: float, runlog) -> None:
        if not self.period:
            return
        now = time.perf_counter()
        if now - self.last < self.period:
            return
        self.last = now
        frac = (t - self.t0) / self.span if self.span > 0 else 1.0
        spent = now - self.start
        left = spent * (1.0 - frac) / frac if frac > 0 else float("nan")
        log.info("%s%.1f%% of %.2f h simulated (t = %.2f h) after %d steps and %.0f s; about %.0f s to go",
                 self.prefix, 100.0 * frac, self.span / 3600.0, t / 3600.0, runlog.steps, spent, left)


__all__ = ["Links", "build_links", "links_from_cells", "exchange", "CoupledEngine", "Snapshot", "RunLog",
           "NumericalInstabilityError"]
