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
        self.cell1d = torch.as_tensor(np.asarray(cell1d), dtype=torch.long)
        self.zbank = torch.as_tensor(np.asarray(zbank, dtype=np.float64))
        self.length = torch.as_tensor(np.asarray(length, dtype=np.float64))
        self.z2 = torch.as_tensor(np.asarray(z2, dtype=np.float64))
        self.inv = torch.as_tensor(np.asarray(inv), dtype=torch.long)
        self.uniq_dev = torch.as_tensor(np.asarray(uniq), dtype=torch.long)
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


def exchange(one: SWE1D, two: SWE2D, links: Links, dt: float, cfg: SolverConfig, volumes: bool = True):
    """Move water between the models in place; per-link volumes (m^3, + = 2-D -> 1-D)
    as a float64 device tensor, enqueued on the current stream without waiting for it
    (coupling.py:73-124).  ``volumes=False`` skips them (the coupled step discards them)."""
    V = torch.empty((links.B, links.n_links), dtype=torch.float64, device=two.device) if volumes else None
    cfgc = links.cfg_struct(cfg)
    one._kernel_writes += 1
    with _lib.on_device(two.device):
        _lib.check(links._lib.his_exchange_async(links._handle, C.byref(cfgc), float(dt),
                                                 V.data_ptr() if V is not None and V.numel() else None,
                                                 _lib.stream_handle()), "his_exchange_async")
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
        # volumes of the step in flight, added to the mass terms on the device
        self._vol2d = torch.zeros((two.B, 5), dtype=torch.float64, device=two.device)
        self._vol1d = torch.zeros((two.B, 3), dtype=torch.float64, device=two.device) if one is not None else None
        # state version of the 1-D model when its rates were last reduced ahead (None: not)
        self._rates1_at = None

    def check_plausible(self, t: float, label: str = "") -> None:
        h = self.two.h
        dmax = h.flatten(-2).amax(-1) if h.dim() == 3 else h.max()
        bad2 = ~torch.isfinite(dmax) | (dmax > MAX_PLAUSIBLE_DEPTH_2D_M)
        bad1 = torch.zeros_like(bad2)
        rise = None
        if self.one is not None:
            one = self.one
            level = one.z + one.sec.depth(one.A)
            zb = torch.as_tensor(one.topo.zbank, dtype=level.dtype, device=level.device)
            rise = torch.where(one.interior, level - zb, torch.full_like(level, -1e9)).amax(-1)
            bad1 = (~torch.isfinite(rise) | (rise > MAX_PLAUSIBLE_RISE_1D_M)).to(bad2.device)
        bad = (bad2 | bad1).reshape(-1)
        if bool(bad.any()):
            members = torch.nonzero(bad).reshape(-1).tolist()
            d2 = dmax.reshape(-1).tolist()
            d1 = rise.reshape(-1).tolist() if rise is not None else [float("nan")] * len(d2)
            who = ", ".join(f"member {m}: max 2-D depth {d2[m]:.2f} m, max 1-D rise above bank {d1[m]:.2f} m"
                            for m in members) if self.batch is not None else \
                f"max 2-D depth {d2[0]:.2f} m, max 1-D rise above bank {d1[0]:.2f} m"
            raise NumericalInstabilityError(
                f"physically impossible state{(' in ' + label) if label else ''} at t = {t / 3600:.3f} h ({who}; "
                f"bounds {MAX_PLAUSIBLE_DEPTH_2D_M:g} m and {MAX_PLAUSIBLE_RISE_1D_M:g} m). The run is invalid.")

    def total_volume(self):
        v = self.two.volume() + self.two.storage_volume()
        if self.one is not None:
            v = v + self.one.volume().to(v.device)
        v = v.cpu()
        return v if self.batch is not None else float(v)

    def _enqueue_rates(self, need2: bool, need1: bool) -> None:
        """Both CFL reductions of the current state, into one pinned buffer.  The 1-D
        rates reduced ahead on the side stream at the end of the last step are the
        current state's unless A or Q has been written since (state version)."""
        B = self.two.B
        with _lib.on_device(self.two.device):
            if need2:
                self.two.rates_async(self._rates[:B])
            if need1 and self._rates1_at != self.one.state_version():
                self.one.rates_async(self._rates[B:])
        self._rates1_at = None

    def _wait_rates(self):
        """Largest 2-D rate and (largest 1-D rate, any wet), after one wait for the GPU."""
        B = self.two.B
        with _lib.on_device(self.two.device):
            torch.cuda.current_stream().synchronize()
        r = self._rates.numpy()
        rw = r[B:].reshape(B, 2)
        return float(r[:B].max()), float(rw[:, 0].max()), bool((rw[:, 1] > 0).any())

    def step(self, t: float, t_limit: float, dt: float | None = None, n_sub: int | None = None) -> float:
        """One coupled step (coupling.py:205-230): CFL dt and 1-D substep count, the
        exchange, the 2-D step and the 1-D substeps, mass terms added on the device.
        The step waits on the GPU once, for the CFL rates; the 1-D substeps run on a
        side stream beside the 2-D step and join before the step returns."""
        two, one = self.two, self.one
        need1 = one is not None and n_sub is None
        wait = dt is None or need1
        if wait:
            self._enqueue_rates(dt is None, need1)
        # forcing at t does not depend on dt: evaluated while the GPU reduces
        rain_t = self.rain(t)
        edges_t = edge_values(two.bcs, t)
        if wait:
            r2, r1, wet1 = self._wait_rates()
        dt = min(two.dt_from_rate(r2) if dt is None else dt, t_limit - t)
        main = torch.cuda.current_stream(two.device)
        if one is not None:
            if n_sub is None:
                n_sub = max(1, math.ceil(dt / one.dt_from_rate(r1, wet1) - 1e-9))
            exchange(one, two, self.links, dt, self.cfg, volumes=False)
            self._exchanged.record(main)
        two.step_into(dt, t, rain_t, edges_t, self._vol2d.data_ptr(), main.cuda_stream)
        if one is not None:
            # after the 2-D launch, so the host prepares the substeps while it runs;
            # the next step's 1-D rates are reduced right behind them, beside the 2-D
            side = self._side
            side.wait_event(self._exchanged)
            one.substeps_into(dt, t, n_sub, self._vol1d.data_ptr(), side.cuda_stream)
            one.rates_async(self._rates[two.B:], side.cuda_stream)
            self._rates1_at = one.state_version()
        mb = self.mb
        mb.add_columns(StepVolumes.TERMS, self._vol2d)
        if one is not None:
            main.wait_stream(self._side)
            mb.add_columns(Step1DVolumes.TERMS, self._vol1d)
            self.log.n_sub_max = max(self.log.n_sub_max, n_sub)
            self._last_n_sub = n_sub
        self.log.steps += 1
        self._last_dt = dt
        self.log.dt_min = min(self.log.dt_min, dt)
        self.log.dt_max = max(self.log.dt_max, dt)
        return t + dt

    def snapshot(self, t: float) -> Snapshot:
        two = self.two
        u, v = two.velocities(two.h, two.hu, two.hv)
        cast = lambda a: a.to(torch.float32).cpu().numpy()
        if self.one is not None:
            eta1, q1 = cast(self.one.level()), cast(self.one.Q)
        else:
            eta1 = q1 = np.zeros(0, np.float32)
        src = self.mb.sources()
        num = (lambda x: x.detach().cpu().numpy()) if self.batch is not None else float
        ledger = {"v2d": num(two.volume()), "v1d": num(self.one.volume()) if self.one is not None else 0.0,
                  "storage": num(two.storage_volume()), **src}
        return Snapshot(t, cast(two.h), cast(u), cast(v), eta1, q1, ledger)

    def run(self, t_end: float, out_times=(), t0: float = 0.0, on_snapshot=None, check_every: int = 500,
            label: str = "", progress_s: float = 120.0):
        wall = time.perf_counter()
        last_report = wall
        t = t0
        outs = sorted(float(x) for x in out_times if t0 <= x <= t_end + 1e-9)
        k = 0
        if outs and abs(outs[0] - t0) < 1e-9:
            on_snapshot and on_snapshot(self.snapshot(t0))
            outs.pop(0)
        while t < t_end - 1e-9:
            limit = outs[0] if outs else t_end
            t = self.step(t, limit)
            if outs and t >= outs[0] - 1e-9:
                self.check_plausible(t, label)
                on_snapshot and on_snapshot(self.snapshot(t))
                outs.pop(0)
            k += 1
            if k % check_every == 0:
                self.mb.check(self.total_volume(), t)
                self.check_plausible(t, label)
            if progress_s and time.perf_counter() - last_report >= progress_s:
                last_report = time.perf_counter()
                done = (t - t0) / (t_end - t0) if t_end > t0 else 1.0
                log.info("%s%.1f%% of %.2f h: t = %.2f h, %d steps", f"{label}: " if label else "", 100 * done,
                         (t_end - t0) / 3600, t / 3600, self.log.steps)
        self.log.wall_s += time.perf_counter() - wall
        if self.links is not None:
            ex = self.links.exchanged()
            num = (lambda x: x) if self.batch is not None else (lambda x: float(x[0]))
            self.log.exchanged_in_m3 = num(ex[:, 0])
            self.log.exchanged_out_m3 = num(ex[:, 1])
        self.log.n_dt_clamped = self.two.n_dt_clamped
        self.check_plausible(t, label)
        return self.mb.assert_ok(self.total_volume(), t, self.cfg.mass_tol, label)


__all__ = ["Links", "build_links", "links_from_cells", "exchange", "CoupledEngine", "Snapshot", "RunLog",
           "NumericalInstabilityError"]
