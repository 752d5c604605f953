"""Drop-in 1-D channel-network solver: the reference's ``SWE1D`` interface
(hydrointel/solver/swe1d.py:169-318) with each step computed by the network kernel
of ``libhis_gb300.so`` (one CTA per member, the whole network in shared memory).

State ``A`` (wetted area) and ``Q`` (discharge), (n_cells,) or (B, n_cells), are
float64 CUDA buffers, and this drop-in solver steps them in float64 whatever the
2-D model's precision.  The device-resident engine's float32 form runs its networks'
arithmetic in float32 with the same float64 state and junction depths.
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass, field

import numpy as np
import torch

from . import _lib
from .channels import ChannelNetwork
from .config import SolverConfig
from .swe2d import cuda_device, per_member
from .topology import Topology, build_topology, sections


@dataclass
class Step1DVolumes:
    bnd_in: torch.Tensor
    bnd_out: torch.Tensor
    clip: torch.Tensor
    # the three columns above as one (B, 3) device table, for one-operation accounting
    table: torch.Tensor | None = field(default=None, repr=False, compare=False)

    TERMS = ("bnd1d_in", "bnd1d_out", "clip")


@dataclass
class Sections:
    """Cross-section geometry of every 1-D cell (or face), torch form for host-side
    queries (levels, depths, plausibility); the step evaluates the same closed forms
    in the network kernel.

    A section is a trapezoid of bottom width b and side slope m (horizontal per
    vertical) up to the bankfull depth yb, continued above the bank by vertical walls
    ts apart.  Its width at height s above the bed is w(s) = b + 2 m s for s <= yb and
    ts above, and every quantity below is an integral of w over the wetted height y:
    the area A = int_0^y w, the first moment of area about the surface
    I1 = int_0^y (y - s) w(s) ds (the hydrostatic force per unit weight), the top
    width T = w(y), and the wetted perimeter, which the vertical walls do not add to
    (the channel above the bank is the floodplain's).  (hydrointel/solver/swe1d.py:51-84)"""
    b: torch.Tensor
    m: torch.Tensor
    yb: torch.Tensor
    ts: torch.Tensor

    def _split(self, y):
        """Depth in the trapezoid and height of water above the bank."""
        return torch.minimum(y, self.yb), torch.clamp(y - self.yb, min=0.0)

    def _trapezoid_area(self, yt):
        # int_0^yt (b + 2 m s) ds
        return yt * (self.b + self.m * yt)

    def bank_area(self):
        return self._trapezoid_area(self.yb)

    def area(self, y):
        yt, above = self._split(y)
        return self._trapezoid_area(yt) + self.ts * above

    def top_width(self, y):
        return torch.where(y <= self.yb, self.b + 2.0 * self.m * y, self.ts)

    def i1(self, y):
        yt, above = self._split(y)
        # the trapezoid's own moment about its top, int_0^yt (yt - s)(b + 2 m s) ds
        # = b yt^2 / 2 + m yt^3 / 3, then its whole area shifted down by the water
        # standing above the bank, then the wall part's moment ts above^2 / 2
        own = self.b * yt * yt / 2.0 + self.m * yt ** 3 / 3.0
        return own + self._trapezoid_area(yt) * above + self.ts * above * above / 2.0

    def perimeter(self, y):
        yt, _ = self._split(y)
        # bed plus two sloping sides of length yt sqrt(1 + m^2)
        return self.b + 2.0 * yt * torch.sqrt(1.0 + self.m * self.m)

    def depth(self, A):
        """Depth holding area A: below the bank the positive root of m y^2 + b y - A = 0,
        written as 2 A / (b + sqrt(b^2 + 4 m A)) so that it stays exact as m -> 0 (a
        rectangle, y = A / b) and has no cancellation; above the bank the extra area
        spreads over the wall width ts."""
        A = torch.clamp(A, min=0.0)
        full = self.bank_area()
        in_trapezoid = 2.0 * A / (self.b + torch.sqrt(self.b * self.b + 4.0 * self.m * A))
        return torch.where(A <= full, in_trapezoid, self.yb + (A - full) / self.ts)


class SWE1D:
    SHARED = ("kind", "reach_of", "ghost_src", "ghost_sign", "face_l", "face_r", "n", "m", "zbank", "dx", "x", "y",
              "chain")

    def __init__(self, net: ChannelNetwork | list, cfg: SolverConfig, device=None, dtype=torch.float64, inflow=None,
                 stage=None):
        batched = isinstance(net, (list, tuple))
        nets = list(net) if batched else [net]
        if not nets:
            raise ValueError("SWE1D needs at least one channel network")
        for n in nets:
            n.validate()
        self.net, self.cfg = nets[0], cfg
        self.batch = len(nets) if batched else None
        self.bshape = () if self.batch is None else (self.batch,)
        self.B = len(nets)
        self.device = cuda_device(device)
        self.dtype = torch.float64
        topos = [build_topology(n) for n in nets]
        self.topo: Topology = topos[0]
        tp = self.topo
        for k, other in enumerate(topos[1:], start=1):
            for name in self.SHARED:
                if not np.array_equal(getattr(other, name), getattr(tp, name)):
                    raise ValueError(f"batched channel network {k} differs from member 0 in '{name}'; only the bed "
                                     "and the bottom width may vary between members (that is what gamma changes)")
        z_np = np.stack([o.z for o in topos]).reshape(self.bshape + (tp.n_cells,))
        b_np = np.stack([o.b for o in topos]).reshape(self.bshape + (tp.n_cells,))
        sec = sections(tp, cfg.slot_width_frac, z_np, b_np)
        self._sec_np = sec
        T = lambda a, dt=torch.float64: torch.as_tensor(np.array(a), dtype=dt, device=self.device)
        self.z, self.nman, self.dx = T(z_np), T(tp.n), T(tp.dx)
        self.sec = Sections(T(sec["b"]), T(sec["m"]), T(sec["yb"]), T(sec["ts"]))
        self.fsec = Sections(T(sec["fb"]), T(sec["fm"]), T(sec["fyb"]), T(sec["fts"]))
        self.is_ghost = T(tp.kind >= 2, torch.bool)
        self.is_junc = T(tp.kind == 1, torch.bool)
        self.interior = ~self.is_ghost
        self.a_dry = self.sec.area(torch.full_like(self.z, cfg.h_dry))
        self.inflow, self.stage = inflow, stage
        self._kernel_writes = 0
        self._A = torch.zeros(self.bshape + (tp.n_cells,), dtype=torch.float64, device=self.device)
        self._Q = torch.zeros_like(self._A)
        self._lib = _lib.load()
        self._handle = C.c_void_p()
        self._host = {k: _lib.host_array(getattr(tp, k), np.int32) for k in ("kind", "ghost_src", "face_l", "face_r")}
        self._host["ghost_sign"] = _lib.host_array(tp.ghost_sign, np.float64)
        self._host["manning"] = _lib.host_array(tp.n, np.float64)
        self._host["dx"] = _lib.host_array(tp.dx, np.float64)
        descs = (_lib.NetDesc * self.B)()
        keep = []
        for b in range(self.B):
            d = descs[b]
            d.n_cells, d.n_faces = tp.n_cells, tp.n_faces
            for k in ("kind", "ghost_src", "face_l", "face_r", "ghost_sign", "manning", "dx"):
                setattr(d, k, _lib.as_p(self._host[k]))
            per = {"z": z_np.reshape(self.B, -1)[b]}
            for k in ("b", "m", "yb", "ts"):
                per[k] = sec[k].reshape(self.B, -1)[b]
            for k in ("fb", "fm", "fyb", "fts"):
                per[k] = np.broadcast_to(sec[k], self.bshape + (tp.n_faces,)).reshape(self.B, -1)[b]
            for k, v in per.items():
                a = _lib.host_array(v, np.float64)
                keep.append(a)
                setattr(d, k, _lib.as_p(a))
            stride = tp.n_cells * 8
            d.A = self._A.data_ptr() + b * stride
            d.Q = self._Q.data_ptr() + b * stride
        cfgc = _lib.solver_cfg(cfg)
        with _lib.on_device(self.device):
            _lib.check(self._lib.his_net_create(C.byref(cfgc), self.B, descs, C.byref(self._handle)),
                       "his_net_create")

    def __del__(self):
        h = getattr(self, "_handle", None)
        if h is not None and h.value and _lib._LIB is not None:
            _lib._LIB.his_net_destroy(h)
            self._handle = C.c_void_p()

    def _assign(self, buf, value):
        v = torch.as_tensor(value, dtype=torch.float64, device=self.device)
        buf.copy_(v.expand_as(buf) if v.shape != buf.shape else v)

    A = property(lambda s: s._A, lambda s, v: s._assign(s._A, v))
    Q = property(lambda s: s._Q, lambda s, v: s._assign(s._Q, v))

    # ---------------------------------------------------------------- state
    def depth(self, A=None):
        return self.sec.depth(self._A if A is None else A)

    def level(self):
        return self.z + self.depth()

    def set_level(self, eta):
        y = torch.clamp(torch.as_tensor(eta, dtype=torch.float64, device=self.device) - self.z, min=0.0)
        self._assign(self._A, self.sec.area(y).expand(self._A.shape))
        self._Q.zero_()

    def volume(self) -> torch.Tensor:
        return (self._A * self.dx * self.interior).to(torch.float64).sum(-1)

    def velocity(self, A, Q, sec: Sections | None = None):
        y = (sec or self.sec).depth(A)
        return torch.where(y >= self.cfg.h_dry, Q / torch.clamp(A, min=1e-12), torch.zeros_like(Q))

    def member_rates(self):
        rate = np.zeros(self.B)
        wet = np.zeros(self.B, dtype=np.int32)
        with _lib.on_device(self.device):
            _lib.check(self._lib.his_net_max_rate(self._handle, _lib.as_p(rate), _lib.as_p(wet),
                                                  _lib.stream_handle()), "his_net_max_rate")
        return rate, wet

    def rates_async(self, out: torch.Tensor, stream: int | None = None) -> None:
        """Enqueue per-member (rate, wet) into ``out`` (B x 2 float64, device or pinned
        host memory), valid once ``stream`` (default: the current one) reaches this point."""
        with _lib.on_device(self.device):
            _lib.check(self._lib.his_net_max_rate_async(self._handle, out.data_ptr(),
                                                        _lib.stream_handle() if stream is None else stream),
                       "his_net_max_rate_async")

    def max_dt(self) -> float:
        rate, wet = self.member_rates()
        return self.dt_from_rate(float(rate.max()), bool(wet.any()))

    def dt_from_rate(self, rate: float, any_wet: bool) -> float:
        """The 1-D CFL choice of swe1d.py:253-262 from the batch's largest rate."""
        if not any_wet:
            return self.cfg.dt_max
        return min(self.cfg.cfl_1d / rate, self.cfg.dt_max)

    # ----------------------------------------------------------------- step
    def forcing(self, t: float) -> np.ndarray:
        q_in = self.inflow(t) if self.inflow is not None else 0.0
        eta = self.stage(t) if self.stage is not None else 0.0
        return per_member([q_in, eta], self.B).T        # (B, 2)

    def substeps(self, dt: float, t: float, n_sub: int) -> Step1DVolumes:
        """n_sub substeps of dt/n_sub, forcing evaluated at each substep start
        (coupling.py:216-221), in one launch."""
        vols = torch.empty((self.B, 3), dtype=torch.float64, device=self.device)
        self.substeps_into(dt, t, n_sub, vols.data_ptr())
        cols = vols.t().unbind(0) if self.bshape else vols[0].unbind(0)
        return Step1DVolumes(*cols, table=vols)

    def substeps_into(self, dt: float, t: float, n_sub: int, vols_ptr: int, stream: int | None = None) -> None:
        """The substeps with their (B, 3) float64 volumes written to ``vols_ptr`` (device
        or page-locked memory) on ``stream`` (default: the current stream)."""
        sub = dt / n_sub
        f = self.forcing(t) if n_sub == 1 else np.stack([self.forcing(t + k * sub) for k in range(n_sub)], axis=1)
        f = np.ascontiguousarray(f, dtype=np.float64)
        self._kernel_writes += 1
        with _lib.on_device(self.device):
            _lib.check(self._lib.his_net_step_async(self._handle, float(dt), int(n_sub), _lib.as_p(f), vols_ptr,
                                                    _lib.stream_handle() if stream is None else stream),
                       "his_net_step_async")

    def substeps_ledger(self, dt: float, t: float, n_sub: int, ledger_ptr: int, stream: int | None = None) -> None:
        """The substeps with their boundary volumes and clip added into an 8 x B float64
        device ledger (``MassBalance.device_ledger``) on ``stream``."""
        sub = dt / n_sub
        f = self.forcing(t) if n_sub == 1 else np.stack([self.forcing(t + k * sub) for k in range(n_sub)], axis=1)
        f = np.ascontiguousarray(f, dtype=np.float64)
        self._kernel_writes += 1
        with _lib.on_device(self.device):
            _lib.check(self._lib.his_net_step_ledger_async(self._handle, float(dt), int(n_sub), _lib.as_p(f),
                                                           ledger_ptr,
                                                           _lib.stream_handle() if stream is None else stream),
                       "his_net_step_ledger_async")

    def state_version(self) -> tuple:
        """Changes whenever A or Q is written: through torch (assignment, in-place ops)
        or by this library's substeps and exchange."""
        return (self._A._version, self._Q._version, self._kernel_writes)

    def step(self, dt: float, t: float) -> Step1DVolumes:
        return self.substeps(dt, t, 1)


__all__ = ["SWE1D", "Step1DVolumes", "Sections"]
