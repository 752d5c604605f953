"""Device-resident batch engine: many storms, each with its own grid, channel network,
forcing, duration and time step, advanced together by the CUDA kernels with no host
round trip per step (CUDA graphs of several steps).

This is the production form of the reference's engine assembly and time loop
(hydrointel/engine.py:169-238 build_engine / build_engine_batch, solver/coupling.py:
201-286 CoupledEngine.step / run) with two deliberate changes: every member keeps
its own CFL time step (the reference shares the smallest one across a batch,
swe2d.py:177-184), and members of different grid sizes share one launch.  A member
run alone and the same member in a batch execute identical arithmetic in the same
order, so their states are bit-identical.

A storm's device resources (state, fields, channel network, peaks) belong to a
``Member``; an engine is built over a list of members and can be rebuilt over
another list (members joining or leaving a batch), each continuing member resuming
its clock and accumulators exactly (``his_engine_resume``).
"""
from __future__ import annotations

import ctypes as C
import math
import time
from dataclasses import dataclass, field

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


@dataclass(frozen=True)
class FloodResult:
    """One storm's outputs, with the fields of the reference's FloodResult
    (hydrointel/api.py:62-82): series at the output times (float32), maxima over them,
    infiltrated and stored volume and the mass-balance error.  extras adds the running
    maxima over every step, the accumulated sources and the run statistics."""
    depth_max: torch.Tensor            # (ny, nx) [m], over the output times
    depth_series: torch.Tensor         # (nt, ny, nx) [m]
    u: torch.Tensor                    # (nt, ny, nx) [m/s]
    v: torch.Tensor                    # (nt, ny, nx) [m/s]
    channel_eta: torch.Tensor          # (nt, n_nodes) [m], interior 1-D cells
    channel_q: torch.Tensor            # (nt, n_nodes) [m^3/s]
    times: torch.Tensor                # (nt,) [s]
    infiltrated_volume_m3: float
    stored_volume_m3: float
    mass_balance_error: float
    provenance: object = None
    in_distribution: bool = True
    distribution_warnings: list = field(default_factory=list)
    extras: dict = field(default_factory=dict)
    speed_max: torch.Tensor | None = None


LEDGER_KEYS = ("v2d", "v1d", "storage", "rain", "infiltration", "bnd2d_in", "bnd2d_out", "bnd1d_in", "bnd1d_out",
               "clip")


def output_count(t_end: float, interval: float) -> int:
    """Number of output times k * interval <= t_end, k >= 0 (hydrointel/engine.py:48-50)."""
    return int(math.floor(t_end / interval + 1e-9)) + 1


def _level_1d(topo_z, sec, A):
    """Channel level z + depth(A) of the trapezoid-plus-slot sections (swe1d.py:51-84)."""
    A = np.maximum(A, 0.0)
    b, m, yb, ts = sec["b"], sec["m"], sec["yb"], sec["ts"]
    ab = yb * (b + m * yb)
    y = np.where(A <= ab, 2.0 * A / (b + np.sqrt(b * b + 4.0 * m * A)), yb + (A - ab) / ts)
    return topo_z + y


def _report_copy(r) -> _lib.MemberReport:
    out = _lib.MemberReport()
    C.memmove(C.byref(out), C.byref(r), C.sizeof(_lib.MemberReport))
    return out


class Member:
    """One storm's device-resident state and tables, in the engine's precision."""

    def __init__(self, storm: Storm, dtype: torch.dtype, device: torch.device, couple: bool = True,
                 track_peaks: bool = False, zcache: dict | None = None, output_interval: float | None = None):
        self.storm = storm
        self.key = storm.key
        self.dtype = dtype
        self.device = device
        ter = storm.terrain
        ny, nx = ter.ny, ter.nx
        self.shape = (ny, nx)
        T = lambda a: torch.as_tensor(np.array(a, order="C"), dtype=dtype, device=device)
        if zcache is not None and id(ter) in zcache:
            self.z = zcache[id(ter)]
        else:
            self.z = T(ter.z)
            if zcache is not None:
                zcache[id(ter)] = self.z
        s = storm
        self.n = T(np.broadcast_to(np.asarray(s.manning, dtype=float), (ny, nx)))
        self.S = T(s.storage) if s.storage is not None else None
        self.f0 = self.fc = self.k = None
        if s.horton is not None:
            self.f0, self.fc, self.k = (T(np.broadcast_to(s.horton[j], (ny, nx))) for j in range(3))
        self.h = T(s.h0())
        self.hu, self.hv, self.s_filled, self.infil_cum = (torch.zeros_like(self.h) for _ in range(4))
        self.peak_h = self.h.clone() if track_peaks else None
        self.peak_speed = torch.zeros_like(self.h) if track_peaks else None
        self.coupled = couple and s.network is not None
        self.A = self.Q = self.topo = None
        self.n_links = 0
        if self.coupled:
            self._build_network()
        self._forcing_arrays = (_lib.host_array(s.forcing.rain, np.float64), _lib.host_array(s.forcing.q, np.float64))
        self.record: _lib.MemberReport | None = None     # clock and accumulators to resume from
        self.volume0: float | None = None
        self.output_interval = output_interval
        self.n_out = 0
        if output_interval is not None:
            self._alloc_outputs(float(output_interval))

    def _alloc_outputs(self, interval: float) -> None:
        """Device slots for the outputs at k * interval; slot 0 is the initial state."""
        if not interval > 0:
            raise ValueError(f"output_interval must be positive (got {interval})")
        n = output_count(float(self.storm.t_end), interval)
        self.n_out = n
        f32 = dict(dtype=torch.float32, device=self.device)
        self.snap_h = torch.zeros((n,) + self.shape, **f32)
        self.snap_u = torch.zeros((n,) + self.shape, **f32)
        self.snap_v = torch.zeros((n,) + self.shape, **f32)
        self.snap_t = torch.zeros(n, dtype=torch.float64, device=self.device)
        # volume ledger per output time (LEDGER_KEYS); slot 0 is set when the first
        # engine measures the initial volumes
        self.snap_ledger = torch.zeros((n, len(LEDGER_KEYS)), dtype=torch.float64, device=self.device)
        self.snap_h[0] = self.h.float()                  # momentum starts at rest: u = v = 0
        if self.coupled:
            n1d = self.topo.n_cells
            self.snap_eta = torch.zeros((n, n1d), **f32)
            self.snap_q = torch.zeros((n, n1d), **f32)
            sec = {k: self._net_arrays[k] for k in ("b", "m", "yb", "ts")}
            eta0 = _level_1d(self._net_arrays["z"], sec, self.A.cpu().numpy())
            self.snap_eta[0] = torch.as_tensor(eta0, dtype=torch.float32)
            self.snap_q[0] = self.Q.float()
        else:
            self.snap_eta = self.snap_q = None

    @property
    def cells(self) -> int:
        return self.shape[0] * self.shape[1]

    def state(self) -> list[torch.Tensor]:
        return [self.h, self.hu, self.hv, self.s_filled, self.infil_cum]

    def nbytes(self) -> int:
        """Device bytes held by this member (state, fields, peaks, network), plus the
        stage scratch and tables a grid set allocates for it."""
        ts = [self.z, self.n, self.S, self.f0, self.fc, self.k, self.h, self.hu, self.hv, self.s_filled,
              self.infil_cum, self.peak_h, self.peak_speed, self.A, self.Q]
        if self.n_out:
            ts += [self.snap_h, self.snap_u, self.snap_v, self.snap_t, self.snap_eta, self.snap_q, self.snap_ledger]
        held = sum(t.numel() * t.element_size() for t in ts if t is not None)
        return held + 3 * self.h.numel() * self.h.element_size() + 64 * 1024

    # ---------------------------------------------------------------- descriptors
    def _build_network(self):
        s = self.storm
        tp = build_topology(s.network)
        sec = sections(tp, s.slot_width_frac)
        f = s.forcing
        yn = normal_depth(tp, sec, f.inflow(0.0))
        level = np.maximum(tp.z + yn, f.tide(0.0))
        y = np.maximum(level - tp.z, 0.0)
        yt = np.minimum(y, sec["yb"])
        A0 = yt * (sec["b"] + sec["m"] * yt) + sec["ts"] * np.maximum(y - sec["yb"], 0.0)
        self.A = torch.as_tensor(A0, dtype=torch.float64, device=self.device)
        self.Q = torch.zeros_like(self.A)
        self.topo = tp
        arrs = {k: _lib.host_array(getattr(tp, k), np.int32) for k in ("kind", "ghost_src", "face_l", "face_r")}
        arrs.update({"ghost_sign": _lib.host_array(tp.ghost_sign, np.float64),
                     "z": _lib.host_array(tp.z, np.float64), "manning": _lib.host_array(tp.n, np.float64),
                     "dx": _lib.host_array(tp.dx, np.float64)})
        arrs.update({k: _lib.host_array(v, np.float64) for k, v in sec.items()})
        self._net_arrays = arrs
        cell1d, cells2d, length = bank_links(s.terrain, tp)
        uniq, inv = np.unique(cells2d, return_inverse=True)
        self._link_arrays = {
            "cell1d": _lib.host_array(cell1d, np.int32), "inv": _lib.host_array(inv, np.int32),
            "uniq": _lib.host_array(uniq, np.int64), "zbank": _lib.host_array(tp.zbank[cell1d], np.float64),
            "length": _lib.host_array(np.full(len(cell1d), length), np.float64),
            "z2": _lib.host_array(s.terrain.z.reshape(-1)[cells2d], np.float64)}
        self.n_links = len(cell1d)

    def fill_grid(self, d) -> None:
        s = self.storm
        d.ny, d.nx = self.shape
        for e, kind in enumerate(s.bc):
            d.bc[e] = KIND_CODE[kind]
        d.dx = d.dy = s.terrain.dx
        d.horton_t0 = float(s.horton[3]) if s.horton is not None else 0.0
        d.h, d.hu, d.hv, d.s_filled, d.infil_cum = (x.data_ptr() for x in self.state())
        d.z, d.manning = self.z.data_ptr(), self.n.data_ptr()
        d.storage = self.S.data_ptr() if self.S is not None else None
        d.f0 = self.f0.data_ptr() if self.f0 is not None else None
        d.fc = self.fc.data_ptr() if self.fc is not None else None
        d.k = self.k.data_ptr() if self.k is not None else None
        d.rain_weight = None
        d.peak_h = self.peak_h.data_ptr() if self.peak_h is not None else None
        d.peak_speed = self.peak_speed.data_ptr() if self.peak_speed is not None else None

    def fill_net(self, d) -> None:
        tp = self.topo
        d.n_cells, d.n_faces = tp.n_cells, tp.n_faces
        for k, v in self._net_arrays.items():
            setattr(d, k, _lib.as_p(v))
        d.A, d.Q = self.A.data_ptr(), self.Q.data_ptr()

    def fill_links(self, d) -> None:
        la = self._link_arrays
        d.n_links, d.n_unique = len(la["cell1d"]), len(la["uniq"])
        for k, v in la.items():
            setattr(d, k, _lib.as_p(v))

    def fill_forcing(self, d) -> None:
        s = self.storm
        f = s.forcing
        rain, q = self._forcing_arrays
        d.t0, d.t_end = 0.0, float(s.t_end)
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
        d.n_out = self.n_out
        if self.n_out:
            d.out_dt = float(self.output_interval)
            d.snap_h, d.snap_u, d.snap_v = (x.data_ptr() for x in (self.snap_h, self.snap_u, self.snap_v))
            d.snap_t = self.snap_t.data_ptr()
            d.snap_ledger = self.snap_ledger.data_ptr()
            if self.coupled:
                d.snap_eta, d.snap_q = self.snap_eta.data_ptr(), self.snap_q.data_ptr()


class FloodEngine:
    def __init__(self, storms: list, cfg: SolverConfig | None = None, precision: str = "fp32",
                 device=None, tile="auto", graph_steps: int = 16, max_sub: int = 64, couple: bool = True,
                 track_peaks: bool = False, output_interval: float | None = None, chains: int | None = None):
        """storms: Storm objects (new members) or Member objects (members moved from
        another engine, resumed from their records).  tile: (tile_x, tile_y) strip width
        and chunk height of the 2-D kernels, (0, 0) or None for the defaults, "auto"
        (default) to let the autotuner measure the candidates for this batch (cached per
        device, precision and batch shape).  output_interval: seconds between the
        outputs of new members (None: no series; running peaks with track_peaks).
        chains: independent member chains the device advances side by side (1..8;
        None: the library's default, one per 256 strip-chunk tiles)."""
        if not storms:
            raise ValueError("FloodEngine needs at least one storm")
        self.cfg = cfg or SolverConfig()
        self.cfg.precision = precision
        self.cfg.validate()
        self.device = cuda_device(device)
        self.dtype = torch.float64 if precision == "fp64" else torch.float32
        self.prec = _lib.PREC_F64 if precision == "fp64" else _lib.PREC_F32
        self._lib = _lib.load()
        self._grid = C.c_void_p()
        self._net = C.c_void_p()
        self._links = C.c_void_p()
        self._engine = C.c_void_p()
        zcache = {}
        members = []
        for s in storms:
            if isinstance(s, Member):
                if s.dtype != self.dtype or s.device != self.device:
                    raise ValueError(f"member {s.key} was built for {s.dtype} on {s.device}")
                members.append(s)
            else:
                members.append(Member(s, self.dtype, self.device, couple, track_peaks, zcache, output_interval))
        self.members = members
        self.storms = [m.storm for m in members]
        self.B = len(members)
        self.coupled = all(m.coupled for m in members)
        if any(m.coupled for m in members) and not self.coupled:
            raise ValueError("a batch is either fully coupled (every storm has a network) or not coupled")
        gdesc = (_lib.GridDesc * self.B)()
        for b, m in enumerate(members):
            m.fill_grid(gdesc[b])
        cfgc = _lib.solver_cfg(self.cfg)
        if isinstance(tile, str):
            if tile != "auto":
                raise ValueError(f"tile must be (tile_x, tile_y), None or 'auto' (got {tile!r})")
            from .autotune import choose_tile, choose_tile_engine
            if all(not isinstance(s, Member) for s in storms):
                # new storms: time the candidates as this engine will run them
                tile = choose_tile_engine(self.storms, self.cfg, precision, self.device, couple)
            else:
                tile = choose_tile(self.device, self.prec, self.cfg, gdesc, [m.state() for m in members])
        self.tile = tuple(tile) if tile is not None else (0, 0)
        tx, ty = self.tile
        with torch.cuda.device(self.device):
            _lib.check(self._lib.his_grid_create(self.prec, C.byref(cfgc), self.B, gdesc, int(tx), int(ty),
                                                 C.byref(self._grid)), "his_grid_create")
            if self.coupled:
                ndesc = (_lib.NetDesc * self.B)()
                ldesc = (_lib.LinksDesc * self.B)()
                for b, m in enumerate(members):
                    m.fill_net(ndesc[b])
                    m.fill_links(ldesc[b])
                _lib.check(self._lib.his_net_create(C.byref(cfgc), self.B, ndesc, C.byref(self._net)),
                           "his_net_create")
                _lib.check(self._lib.his_links_create(self._grid, self._net, self.B, ldesc, C.byref(self._links)),
                           "his_links_create")
            fdesc = (_lib.ForcingDesc * self.B)()
            for b, m in enumerate(members):
                m.fill_forcing(fdesc[b])
            _lib.check(self._lib.his_engine_create(self._grid, self._net if self.coupled else None,
                                                   self._links if self.coupled else None, self.B, fdesc,
                                                   int(max_sub), int(graph_steps), C.byref(self._engine)),
                       "his_engine_create")
            if chains is not None:
                _lib.check(self._lib.his_engine_set_chains(self._engine, int(chains)), "his_engine_set_chains")
            if any(m.record is not None for m in members):
                reps = (_lib.MemberReport * self.B)()
                mask = np.zeros(self.B, dtype=np.int32)
                for b, m in enumerate(members):
                    if m.record is not None:
                        reps[b] = m.record
                        mask[b] = 1
                _lib.check(self._lib.his_engine_resume(self._engine, reps, _lib.as_p(mask), _lib.stream_handle()),
                           "his_engine_resume")
        if any(m.volume0 is None for m in members):
            v2 = np.zeros((self.B, 2))
            v1 = np.zeros(self.B)
            with torch.cuda.device(self.device):
                _lib.check(self._lib.his_grid_volumes(self._grid, _lib.as_p(v2), _lib.stream_handle()),
                           "his_grid_volumes")
                if self.coupled:
                    _lib.check(self._lib.his_net_volume(self._net, _lib.as_p(v1), _lib.stream_handle()),
                               "his_net_volume")
            for b, m in enumerate(members):
                if m.volume0 is None:
                    m.volume0 = float(v2[b].sum() + v1[b])
                    if m.n_out:
                        m.snap_ledger[0, :3] = torch.tensor([v2[b, 0], v1[b], v2[b, 1]], dtype=torch.float64)
        self.n_links = [m.n_links for m in members] if self.coupled else []

    # ------------------------------------------------------- per-member views
    h = property(lambda s: [m.h for m in s.members])
    hu = property(lambda s: [m.hu for m in s.members])
    hv = property(lambda s: [m.hv for m in s.members])
    s_filled = property(lambda s: [m.s_filled for m in s.members])
    infil_cum = property(lambda s: [m.infil_cum for m in s.members])
    peak_h = property(lambda s: [m.peak_h for m in s.members])
    peak_speed = property(lambda s: [m.peak_speed for m in s.members])
    A = property(lambda s: [m.A for m in s.members])
    Q = property(lambda s: [m.Q for m in s.members])
    topos = property(lambda s: [m.topo for m in s.members])

    @property
    def volume0(self) -> np.ndarray:
        return np.array([m.volume0 for m in self.members])

    def __del__(self):
        self.close()

    @property
    def chains(self) -> int:
        """Independent member chains the device advances side by side."""
        return int(self._lib.his_engine_chains(self._engine))

    def close(self) -> None:
        """Free the engine's device tables (the members keep their state)."""
        L = _lib._LIB
        if L is None:
            return
        for attr, fn in (("_engine", "his_engine_destroy"), ("_links", "his_links_destroy"),
                         ("_net", "his_net_destroy"), ("_grid", "his_grid_destroy")):
            h = getattr(self, attr, None)
            if h is not None and h.value:
                getattr(L, fn)(h)
                setattr(self, attr, C.c_void_p())

    def detach(self) -> list[Member]:
        """Save every member's record for a later resume, free the engine and return the
        members (to be placed in another engine)."""
        reps = self.reports()
        for m, r in zip(self.members, reps):
            m.record = _report_copy(r)
        self.close()
        return self.members

    # ------------------------------------------------------------------ running
    @property
    def cells(self) -> list[int]:
        return [m.cells for m in self.members]

    def advance(self, n_steps: int) -> None:
        with torch.cuda.device(self.device):
            _lib.check(self._lib.his_engine_advance(self._engine, int(n_steps), _lib.stream_handle()),
                       "his_engine_advance")

    def prepare(self, n_steps: int) -> None:
        """Capture the CUDA graphs that ``advance(n_steps)`` launches, without running
        any step (the capture is then outside the advance)."""
        with torch.cuda.device(self.device):
            _lib.check(self._lib.his_engine_prepare(self._engine, int(n_steps)), "his_engine_prepare")

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

    def results(self, reps=None) -> list[MemberResult]:
        reps = self.reports() if reps is None else reps
        vol = self.volumes()
        out = []
        for b, (m, r) in enumerate(zip(self.members, reps)):
            src = {k: float(r.acc[j]) for j, k in enumerate(TERMS)}
            net = src["rain"] - src["infiltration"] + src["bnd2d_in"] - src["bnd2d_out"] + src["bnd1d_in"] - \
                src["bnd1d_out"]
            gross = src["rain"] + src["infiltration"] + src["bnd2d_in"] + src["bnd2d_out"] + src["bnd1d_in"] + \
                src["bnd1d_out"]
            v0 = float(m.volume0)
            err = abs((float(vol[b]) - v0) - net) / max(gross, 1e-9 * abs(v0) + 1.0)
            out.append(MemberResult(m.key, _lib.STATUS.get(r.status, str(r.status)), r.t, int(r.steps), r.dt_min,
                                    r.dt_max, r.n_sub_max, r.n_dt_clamped, src, v0, float(vol[b]), err))
        return out

    def flood_results(self, reps=None, only: list[int] | None = None) -> list[FloodResult]:
        """FloodResult of every member (or of the members listed in ``only``) from the
        outputs written so far (the series ends at the last output time reached).  The
        device data are copied to pinned host memory with non-blocking copies and one
        synchronisation."""
        reps = self.reports() if reps is None else reps
        runs = self.results(reps)
        pick = list(range(self.B)) if only is None else list(only)
        v2 = np.zeros((self.B, 2))
        with torch.cuda.device(self.device):
            _lib.check(self._lib.his_grid_volumes(self._grid, _lib.as_p(v2), _lib.stream_handle()),
                       "his_grid_volumes")
        pending = []
        with torch.cuda.device(self.device):
            for b in pick:
                m = self.members[b]
                k = int(reps[b].outputs) if m.n_out else 0
                host = {}
                for name in ("snap_h", "snap_u", "snap_v", "snap_t", "snap_eta", "snap_q", "snap_ledger", "peak_h",
                             "peak_speed"):
                    src = getattr(m, name, None)
                    if src is None or (name.startswith("snap") and k == 0):
                        continue
                    src = src[:k] if name.startswith("snap") else src
                    dst = torch.empty(src.shape, dtype=src.dtype, pin_memory=True)
                    dst.copy_(src, non_blocking=True)
                    host[name] = dst
                pending.append((k, host))
            torch.cuda.current_stream(self.device).synchronize()
        out = []
        for b, (k, host) in zip(pick, pending):
            m, run = self.members[b], runs[b]
            h = host.get("snap_h", torch.zeros((0,) + m.shape))
            u = host.get("snap_u", torch.zeros((0,) + m.shape))
            v = host.get("snap_v", torch.zeros((0,) + m.shape))
            interior = torch.as_tensor(m.topo.kind <= 1) if m.coupled else None
            eta = host["snap_eta"][:, interior] if "snap_eta" in host else torch.zeros((len(h), 0))
            q = host["snap_q"][:, interior] if "snap_q" in host else torch.zeros((len(h), 0))
            extras = {"sources": run.sources, "run": run, "volume0": run.volume0, "volume": run.volume,
                      "outputs": k}
            if "snap_ledger" in host:
                extras["ledger"] = [dict(zip(LEDGER_KEYS, row.tolist())) for row in host["snap_ledger"]]
            if "peak_h" in host:
                extras["depth_max_every_step"] = host["peak_h"]
                extras["speed_max_every_step"] = host["peak_speed"]
            out.append(FloodResult(
                depth_max=h.amax(0) if len(h) else torch.zeros(m.shape),
                depth_series=h, u=u, v=v, channel_eta=eta, channel_q=q,
                times=host.get("snap_t", torch.zeros(0, dtype=torch.float64)),
                infiltrated_volume_m3=run.sources["infiltration"], stored_volume_m3=float(v2[b, 1]),
                mass_balance_error=run.mass_error, extras=extras,
                speed_max=torch.sqrt(u.double() ** 2 + v.double() ** 2).amax(0).float() if len(h) else None))
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


__all__ = ["FloodEngine", "FloodResult", "Member", "MemberResult", "output_count"]
