"""Device-resident batch engine: many storms, each with its own grid, channel network,
forcing, duration and time step, advanced together by the CUDA kernels with no host
round trip per step (CUDA graphs of several steps).

This is the production form of the reference's engine assembly and time loop
(hydrointel/engine.py:169-238 build_engine / build_engine_batch, solver/coupling.py:
201-286 CoupledEngine.step / run) with two deliberate changes: every member keeps
its own CFL time step (the reference shares the smallest one across a batch,
swe2d.py:177-184), and members of different grid sizes share one launch.  A member
run alone and the same member in a batch execute identical arithmetic in the same
order, so their results are bit-identical.
"""
from __future__ import annotations

import ctypes as C
import math
import time
from dataclasses import dataclass

import numpy as np
import torch

from . import _lib
from .boundaries import KIND_CODE
from .config import SolverConfig
from .massbalance import TERMS
from .swe2d import cuda_device
from .topology import build_topology, sections
from .workloads import Storm, bank_links, normal_depth


@dataclass
class MemberResult:
    key: str
    status: str
    t: float
    steps: int
    dt_min: float
    dt_max: float
    n_sub_max: int
    n_dt_clamped: int
    sources: dict
    volume0: float
    volume: float
    mass_error: float


class FloodEngine:
    def __init__(self, storms: list[Storm], cfg: SolverConfig | None = None, precision: str = "fp32",
                 device=None, tile=None, graph_steps: int = 16, max_sub: int = 64, couple: bool = True,
                 track_peaks: bool = False):
        if not storms:
            raise ValueError("FloodEngine needs at least one storm")
        self.cfg = cfg or SolverConfig()
        self.cfg.precision = precision
        self.cfg.validate()
        self.storms = list(storms)
        self.B = len(storms)
        self.device = cuda_device(device)
        self.dtype = torch.float64 if precision == "fp64" else torch.float32
        self.prec = _lib.PREC_F64 if precision == "fp64" else _lib.PREC_F32
        self._lib = _lib.load()
        dev, dt_ = self.device, self.dtype
        T = lambda a: torch.as_tensor(np.ascontiguousarray(a), dtype=dt_, device=dev)
        self.h, self.hu, self.hv, self.s_filled, self.infil_cum = [], [], [], [], []
        self.peak_h, self.peak_speed = [], []
        self._keep = []
        zcache = {}
        gdesc = (_lib.GridDesc * self.B)()
        for b, s in enumerate(storms):
            ter = s.terrain
            ny, nx = ter.ny, ter.nx
            if id(ter) not in zcache:
                zcache[id(ter)] = T(ter.z)
            z = zcache[id(ter)]
            n = T(np.broadcast_to(np.asarray(s.manning, dtype=float), (ny, nx)))
            S = T(s.storage) if s.storage is not None else None
            f0 = fc = kk = None
            if s.horton is not None:
                f0, fc, kk = T(np.broadcast_to(s.horton[0], (ny, nx))), T(np.broadcast_to(s.horton[1], (ny, nx))), \
                    T(np.broadcast_to(s.horton[2], (ny, nx)))
            h = T(s.h0())
            st = [h, torch.zeros_like(h), torch.zeros_like(h), torch.zeros_like(h), torch.zeros_like(h)]
            for lst, x in zip((self.h, self.hu, self.hv, self.s_filled, self.infil_cum), st):
                lst.append(x)
            self._keep += [z, n, S, f0, fc, kk]
            d = gdesc[b]
            d.ny, d.nx = ny, nx
            for e, kind in enumerate(s.bc):
                d.bc[e] = KIND_CODE[kind]
            d.dx = d.dy = ter.dx
            d.horton_t0 = float(s.horton[3]) if s.horton is not None else 0.0
            d.h, d.hu, d.hv, d.s_filled, d.infil_cum = (x.data_ptr() for x in st)
            d.z, d.manning = z.data_ptr(), n.data_ptr()
            d.storage = S.data_ptr() if S is not None else None
            d.f0 = f0.data_ptr() if f0 is not None else None
            d.fc = fc.data_ptr() if fc is not None else None
            d.k = kk.data_ptr() if kk is not None else None
            d.rain_weight = None
            if track_peaks:
                pk, ps = h.clone(), torch.zeros_like(h)
                self.peak_h.append(pk)
                self.peak_speed.append(ps)
                d.peak_h, d.peak_speed = pk.data_ptr(), ps.data_ptr()
            else:
                d.peak_h = d.peak_speed = None
        self._grid = C.c_void_p()
        cfgc = _lib.solver_cfg(self.cfg)
        tx, ty = tile if tile is not None else (0, 0)
        with torch.cuda.device(dev):
            _lib.check(self._lib.his_grid_create(self.prec, C.byref(cfgc), self.B, gdesc, int(tx), int(ty),
                                                 C.byref(self._grid)), "his_grid_create")
        self._net = C.c_void_p()
        self._links = C.c_void_p()
        self.coupled = couple and all(s.network is not None for s in storms)
        self.A, self.Q, self.topos = [], [], []
        if self.coupled:
            self._build_network(cfgc)
        self._build_engine(graph_steps, max_sub)
        self.volume0 = self.volumes()

    # ------------------------------------------------------------------ set-up
    def _build_network(self, cfgc):
        ndesc = (_lib.NetDesc * self.B)()
        ldesc = (_lib.LinksDesc * self.B)()
        for b, s in enumerate(self.storms):
            tp = build_topology(s.network)
            sec = sections(tp, s.slot_width_frac)
            f = s.forcing
            yn = normal_depth(tp, sec, f.inflow(0.0))
            level = np.maximum(tp.z + yn, f.tide(0.0))
            y = np.maximum(level - tp.z, 0.0)
            yt = np.minimum(y, sec["yb"])
            A0 = yt * (sec["b"] + sec["m"] * yt) + sec["ts"] * np.maximum(y - sec["yb"], 0.0)
            A = torch.as_tensor(A0, dtype=torch.float64, device=self.device)
            Q = torch.zeros_like(A)
            self.A.append(A)
            self.Q.append(Q)
            self.topos.append(tp)
            arrs = {k: _lib.host_array(getattr(tp, k), np.int32) for k in ("kind", "ghost_src", "face_l", "face_r")}
            arrs.update({"ghost_sign": _lib.host_array(tp.ghost_sign, np.float64),
                         "z": _lib.host_array(tp.z, np.float64), "manning": _lib.host_array(tp.n, np.float64),
                         "dx": _lib.host_array(tp.dx, np.float64)})
            arrs.update({k: _lib.host_array(v, np.float64) for k, v in sec.items()})
            self._keep.append(arrs)
            d = ndesc[b]
            d.n_cells, d.n_faces = tp.n_cells, tp.n_faces
            for k, v in arrs.items():
                setattr(d, k, _lib.as_p(v))
            d.A, d.Q = A.data_ptr(), Q.data_ptr()
            cell1d, cells2d, length = bank_links(s.terrain, tp)
            uniq, inv = np.unique(cells2d, return_inverse=True)
            la = {"cell1d": _lib.host_array(cell1d, np.int32), "inv": _lib.host_array(inv, np.int32),
                  "uniq": _lib.host_array(uniq, np.int64), "zbank": _lib.host_array(tp.zbank[cell1d], np.float64),
                  "length": _lib.host_array(np.full(len(cell1d), length), np.float64),
                  "z2": _lib.host_array(s.terrain.z.reshape(-1)[cells2d], np.float64)}
            self._keep.append(la)
            ld = ldesc[b]
            ld.n_links, ld.n_unique = len(cell1d), len(uniq)
            for k, v in la.items():
                setattr(ld, k, _lib.as_p(v))
        with torch.cuda.device(self.device):
            _lib.check(self._lib.his_net_create(C.byref(cfgc), self.B, ndesc, C.byref(self._net)), "his_net_create")
            _lib.check(self._lib.his_links_create(self._grid, self._net, self.B, ldesc, C.byref(self._links)),
                       "his_links_create")
        self.n_links = [int(ldesc[b].n_links) for b in range(self.B)]

    def _build_engine(self, graph_steps, max_sub):
        fdesc = (_lib.ForcingDesc * self.B)()
        for b, s in enumerate(self.storms):
            f = s.forcing
            d = fdesc[b]
            d.t0, d.t_end = 0.0, float(s.t_end)
            rain = _lib.host_array(f.rain, np.float64)
            q = _lib.host_array(f.q, np.float64)
            self._keep += [rain, q]
            d.rain_t0, d.rain_step, d.rain_n = f.rain_t0, f.rain_step, len(rain)
            d.rain = _lib.as_p(rain) if len(rain) else None
            d.tide_on, d.tide_n = int(bool(f.tide_on)), len(f.tide_amp)
            d.tide_base, d.tide_shift = f.tide_base, f.tide_shift
            for j in range(len(f.tide_amp)):
                d.tide_amp[j], d.tide_w[j], d.tide_phase[j] = f.tide_amp[j], f.tide_w[j], f.tide_phase[j]
            d.q_t0, d.q_step, d.q_n = f.q_t0, f.q_step, len(q)
            d.q = _lib.as_p(q) if len(q) else None
            for e, kind in enumerate(s.bc):
                d.edge_src[e] = 1 if kind == "stage" else 0
                d.edge_val[e] = 0.0
        self._engine = C.c_void_p()
        with torch.cuda.device(self.device):
            _lib.check(self._lib.his_engine_create(self._grid, self._net if self.coupled else None,
                                                   self._links if self.coupled else None, self.B, fdesc,
                                                   int(max_sub), int(graph_steps), C.byref(self._engine)),
                       "his_engine_create")

    def __del__(self):
        L = _lib._LIB
        if L is None:
            return
        for attr, fn in (("_engine", "his_engine_destroy"), ("_links", "his_links_destroy"),
                         ("_net", "his_net_destroy"), ("_grid", "his_grid_destroy")):
            h = getattr(self, attr, None)
            if h is not None and h.value:
                getattr(L, fn)(h)
                setattr(self, attr, C.c_void_p())

    # ------------------------------------------------------------------ running
    @property
    def cells(self) -> list[int]:
        return [s.cells for s in self.storms]

    def advance(self, n_steps: int) -> None:
        with torch.cuda.device(self.device):
            _lib.check(self._lib.his_engine_advance(self._engine, int(n_steps), _lib.stream_handle()),
                       "his_engine_advance")

    def reports(self):
        reps = (_lib.MemberReport * self.B)()
        with torch.cuda.device(self.device):
            _lib.check(self._lib.his_engine_report(self._engine, reps, _lib.stream_handle()), "his_engine_report")
        return reps

    def run(self, chunk: int = 256, max_steps: int | None = None, timeout_s: float | None = None):
        """Advance until every member is done (or failed); returns the reports."""
        t0 = time.perf_counter()
        total = 0
        while True:
            reps = self.reports()
            if all(r.status != 0 for r in reps):
                return reps
            if max_steps is not None and total >= max_steps:
                return reps
            if timeout_s is not None and time.perf_counter() - t0 > timeout_s:
                return reps
            n = chunk if max_steps is None else min(chunk, max_steps - total)
            self.advance(n)
            total += n

    def volumes(self) -> np.ndarray:
        """Total water per member: 2-D surface + retained + 1-D channel (float64)."""
        v2 = np.zeros((self.B, 2))
        with torch.cuda.device(self.device):
            _lib.check(self._lib.his_grid_volumes(self._grid, _lib.as_p(v2), _lib.stream_handle()),
                       "his_grid_volumes")
            v = v2.sum(axis=1)
            if self.coupled:
                v1 = np.zeros(self.B)
                _lib.check(self._lib.his_net_volume(self._net, _lib.as_p(v1), _lib.stream_handle()),
                           "his_net_volume")
                v = v + v1
        return v

    def results(self) -> list[MemberResult]:
        reps = self.reports()
        vol = self.volumes()
        out = []
        for b, (s, r) in enumerate(zip(self.storms, reps)):
            src = {k: float(r.acc[j]) for j, k in enumerate(TERMS)}
            net = src["rain"] - src["infiltration"] + src["bnd2d_in"] - src["bnd2d_out"] + src["bnd1d_in"] - \
                src["bnd1d_out"]
            gross = src["rain"] + src["infiltration"] + src["bnd2d_in"] + src["bnd2d_out"] + src["bnd1d_in"] + \
                src["bnd1d_out"]
            v0 = float(self.volume0[b])
            err = abs((float(vol[b]) - v0) - net) / max(gross, 1e-9 * abs(v0) + 1.0)
            out.append(MemberResult(s.key, _lib.STATUS.get(r.status, str(r.status)), r.t, int(r.steps), r.dt_min,
                                    r.dt_max, r.n_sub_max, r.n_dt_clamped, src, v0, float(vol[b]), err))
        return out

    def assert_mass_ok(self, tol: float | None = None) -> np.ndarray:
        tol = self.cfg.mass_tol if tol is None else tol
        res = self.results()
        errs = np.array([r.mass_error for r in res])
        bad = np.nonzero(~(errs < tol))[0]
        if len(bad):
            detail = ", ".join(f"member {int(i)}: {errs[int(i)]:.3e}" for i in bad[:8])
            raise AssertionError(f"mass balance violated for {len(bad)}/{self.B} batch members "
                                 f"(tolerance {tol:.1e}) -- {detail}")
        return errs


__all__ = ["FloodEngine", "MemberResult"]
