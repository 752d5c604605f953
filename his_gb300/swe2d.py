"""Drop-in 2-D shallow-water solver: the reference's ``SWE2D`` interface
(hydrointel/solver/swe2d.py:104-303) with every time step computed by the
hand-written sm_103a kernels of ``libhis_gb300.so``.

State ``h, hu, hv, s_filled, infil_cum`` is (ny, nx), or (B, ny, nx) when batched,
and lives in fixed CUDA buffers that the kernels update in place; assigning to
one of the attributes copies into its buffer.  ``dtype=torch.float64`` selects the
plain method, ``torch.float32`` the production form.  The model always computes
on a CUDA device: ``device`` selects which one (a CPU device request means the
current CUDA device).
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass, field

import numpy as np
import torch

from . import _lib
from .boundaries import EDGES, EdgeBC, bc_codes, edge_values
from .config import SolverConfig
from .infiltration import Horton

SQRT2 = 1.4142135623730951


@dataclass
class StepVolumes:
    bnd_in: torch.Tensor
    bnd_out: torch.Tensor
    rain: torch.Tensor
    infil: torch.Tensor
    clip: torch.Tensor
    # the five columns above as one (B, 5) device table, for one-operation accounting
    table: torch.Tensor | None = field(default=None, repr=False, compare=False)

    TERMS = ("bnd2d_in", "bnd2d_out", "rain", "infiltration", "clip")


def cuda_device(device=None) -> torch.device:
    if not torch.cuda.is_available():
        raise RuntimeError("his_gb300 runs its time step on a CUDA GPU and none is available")
    if device is not None:
        d = torch.device(device)
        if d.type == "cuda":
            return torch.device("cuda", d.index if d.index is not None else torch.cuda.current_device())
    return torch.device("cuda", torch.cuda.current_device())


_STEP_DTYPE = np.dtype(_lib.StepParams)


def per_member(values, B: int, dtype=np.float64) -> np.ndarray:
    """1 value (broadcast) or one per member, else ValueError (swe2d.py:282-296)."""
    if all(isinstance(v, (float, int)) or (isinstance(v, np.ndarray) and v.size in (1, B)) for v in values):
        out = np.empty((len(values), B), dtype=dtype)
        for k, v in enumerate(values):
            out[k] = v.reshape(-1) if isinstance(v, np.ndarray) else v
        return out
    out = []
    for v in values:
        if torch.is_tensor(v):
            v = v.detach().cpu().numpy()
        x = np.asarray(v, dtype=dtype).reshape(-1)
        if x.size == 1:
            out.append(np.full(B, x[0], dtype=dtype))
        elif x.size == B:
            out.append(x)
        else:
            raise ValueError(f"expected 1 or {B} values per step quantity, got {x.size}")
    return np.stack(out, axis=0)


class SWE2D:
    def __init__(self, z, manning, dx: float, cfg: SolverConfig, bcs: dict, device=None, dtype=torch.float64,
                 storage=None, horton: Horton | None = None, rain_weight=None, dy: float | None = None,
                 batch: int | None = None, tile=None):
        self.cfg = cfg
        self.device = cuda_device(device)
        if dtype not in (torch.float64, torch.float32):
            raise ValueError(f"dtype must be torch.float64 or torch.float32 (got {dtype})")
        self.dtype = dtype
        self.prec = _lib.PREC_F64 if dtype == torch.float64 else _lib.PREC_F32

        def t(a):
            x = a if torch.is_tensor(a) else torch.as_tensor(np.asarray(a))
            return x.to(device=self.device, dtype=dtype).contiguous().clone()

        self.z = t(z)
        if self.z.dim() != 2:
            raise ValueError(f"bed must be (ny, nx), got shape {tuple(self.z.shape)}")
        self.batch = None if batch is None else int(batch)
        self.bshape = () if batch is None else (int(batch),)
        self.B = 1 if batch is None else int(batch)
        self.ny, self.nx = self.z.shape
        self.n = t(manning) if (torch.is_tensor(manning) or hasattr(manning, "shape")) \
            else torch.full_like(self.z, float(manning))
        self.dx, self.dy = float(dx), float(dy if dy is not None else dx)
        self.area = self.dx * self.dy
        self.bcs = bcs
        self._bc = bc_codes(bcs)
        self.g = cfg.g
        self.order = cfg.spatial_order
        self.ng = 1 if self.order == 1 else 2
        self.storage = t(storage) if storage is not None else None
        self.horton = horton
        self.rain_weight = t(rain_weight) if rain_weight is not None else None
        if self.rain_weight is not None and tuple(self.rain_weight.shape) != (self.ny, self.nx):
            raise ValueError("rain_weight must be (ny, nx)")
        if horton is not None:
            self._f0, self._fc, self._k = t(horton.f0), t(horton.fc), t(horton.k)
        else:
            self._f0 = self._fc = self._k = None
        full = self.bshape + (self.ny, self.nx)
        zeros = torch.zeros(full, dtype=dtype, device=self.device)
        self._h, self._hu, self._hv = zeros.clone(), zeros.clone(), zeros.clone()
        self._kernel_writes = 0          # the library's writes of h, hu, hv outside a step
        self._sf, self._ic = zeros.clone(), zeros.clone()
        self.n_dt_clamped = 0
        self._lib = _lib.load()
        self._handle = C.c_void_p()
        descs = (_lib.GridDesc * self.B)()
        for b in range(self.B):
            d = descs[b]
            d.ny, d.nx = self.ny, self.nx
            for e in range(4):
                d.bc[e] = int(self._bc[e])
            d.dx, d.dy = self.dx, self.dy
            d.horton_t0 = float(horton.t0) if horton is not None else 0.0
            d.h, d.hu, d.hv = self._plane(self._h, b), self._plane(self._hu, b), self._plane(self._hv, b)
            d.s_filled, d.infil_cum = self._plane(self._sf, b), self._plane(self._ic, b)
            d.z = self._plane(self.z, b)
            d.manning = self._plane(self.n, b)
            d.storage = self._plane(self.storage, b)
            d.f0, d.fc, d.k = self._plane(self._f0, b), self._plane(self._fc, b), self._plane(self._k, b)
            d.rain_weight = self._plane(self.rain_weight, b)
        tx, ty = tile if tile is not None else (0, 0)
        self._params_rec = np.zeros(self.B, dtype=_STEP_DTYPE)
        self._params_ptr = self._params_rec.ctypes.data_as(C.POINTER(_lib.StepParams))
        cfgc = _lib.solver_cfg(cfg)
        with _lib.on_device(self.device):
            _lib.check(self._lib.his_grid_create(self.prec, C.byref(cfgc), self.B, descs, int(tx), int(ty),
                                                 C.byref(self._handle)), "his_grid_create")
        self._descs = descs

    def _plane(self, a, b):
        """Device address of member b's (ny, nx) plane of a; shared fields alias one plane."""
        if a is None:
            return None
        if a.dim() == 2:
            return a.data_ptr()
        if a.dim() == 3 and a.shape[0] == self.B and tuple(a.shape[1:]) == (self.ny, self.nx):
            return a.data_ptr() + b * self.ny * self.nx * a.element_size()
        if a.dim() == 3 and a.shape[0] == 1:
            return a.data_ptr()
        raise ValueError(f"field of shape {tuple(a.shape)} does not fit batch {self.batch} on a "
                         f"{self.ny}x{self.nx} grid")

    def __del__(self):
        h = getattr(self, "_handle", None)
        if h is not None and h.value and _lib._LIB is not None:
            _lib._LIB.his_grid_destroy(h)
            self._handle = C.c_void_p()

    # ------------------------------------------------------------ state access
    def _assign(self, buf, value):
        v = torch.as_tensor(value, dtype=self.dtype, device=self.device)
        buf.copy_(v.expand_as(buf) if v.shape != buf.shape else v)

    h = property(lambda s: s._h, lambda s, v: s._assign(s._h, v))
    hu = property(lambda s: s._hu, lambda s, v: s._assign(s._hu, v))
    hv = property(lambda s: s._hv, lambda s, v: s._assign(s._hv, v))
    s_filled = property(lambda s: s._sf, lambda s, v: s._assign(s._sf, v))
    infil_cum = property(lambda s: s._ic, lambda s, v: s._assign(s._ic, v))

    def set_state(self, h, hu=None, hv=None):
        self._assign(self._h, h)
        self._assign(self._hu, 0.0 if hu is None else hu)
        self._assign(self._hv, 0.0 if hv is None else hv)

    def set_level(self, eta, mask=None):
        if torch.is_tensor(eta) or hasattr(eta, "shape"):
            eta = torch.as_tensor(eta, dtype=self.dtype, device=self.device).reshape(self.bshape + (1, 1))
        h = torch.clamp(eta - self.z, min=0.0).expand(self.bshape + (self.ny, self.nx))
        if mask is not None:
            h = torch.where(torch.as_tensor(mask, device=self.device), h, torch.zeros_like(h))
        self.set_state(h)

    def velocities(self, h, hu, hv):
        """Kurganov-Petrova velocities of a state (for output; the step computes its own)."""
        h4 = h ** 4
        den = torch.sqrt(h4 + torch.clamp(h4, min=self.cfg.kp_eps))
        wet = h >= self.cfg.h_dry
        u = torch.where(wet, SQRT2 * h * hu / den, torch.zeros_like(h))
        v = torch.where(wet, SQRT2 * h * hv / den, torch.zeros_like(h))
        return u, v

    def volume(self) -> torch.Tensor:
        return self._h.to(torch.float64).sum(dim=(-2, -1)) * self.area

    def storage_volume(self) -> torch.Tensor:
        return self._sf.to(torch.float64).sum(dim=(-2, -1)) * self.area

    # -------------------------------------------------------------- time step
    def member_rates(self) -> np.ndarray:
        out = np.zeros(self.B)
        with _lib.on_device(self.device):
            _lib.check(self._lib.his_grid_max_rate(self._handle, _lib.as_p(out), _lib.stream_handle()),
                       "his_grid_max_rate")
        return out

    def rates_async(self, out: torch.Tensor, stream: int | None = None) -> None:
        """Enqueue the per-member CFL rates into ``out`` (B float64, device or pinned
        host memory), valid once ``stream`` (default: the current one) reaches this point."""
        with _lib.on_device(self.device):
            _lib.check(self._lib.his_grid_max_rate_async(self._handle, out.data_ptr(),
                                                         _lib.stream_handle() if stream is None else stream),
                       "his_grid_max_rate_async")

    def step_rate_async(self, out: torch.Tensor, stream: int | None = None) -> None:
        """Enqueue the per-member CFL rates of the state the last step left into
        ``out``, from that step's own last stage (no reduction); valid only while
        ``state_version()`` is what it was after the step."""
        with _lib.on_device(self.device):
            _lib.check(self._lib.his_grid_step_rate_async(self._handle, out.data_ptr(),
                                                          _lib.stream_handle() if stream is None else stream),
                       "his_grid_step_rate_async")

    def state_version(self) -> tuple:
        """Changes whenever h, hu or hv is written: through torch (assignment, in-place
        ops, set_state) or by this library outside a step (the weir exchange)."""
        return (self._h._version, self._hu._version, self._hv._version, self._kernel_writes)

    def max_dt(self) -> float:
        """CFL step over the whole batch (the reference shares one dt across members)."""
        return self.dt_from_rate(float(self.member_rates().max()))

    def dt_from_rate(self, m: float) -> float:
        """The CFL choice of swe2d.py:186-193 from the batch's largest rate."""
        cfg = self.cfg
        dt = cfg.cfl / m if m > 0 else cfg.dt_max
        if dt < cfg.dt_min or dt > cfg.dt_max:
            if dt < cfg.dt_min:
                self.n_dt_clamped += 1
            dt = min(max(dt, cfg.dt_min), cfg.dt_max)
        return dt

    def step_params(self, dt: float, t: float, rain_rate=0.0, edges_t=None):
        """his_step_params of every member, as a numpy record array with the C layout
        (filled column-wise: a Python loop over members costs more than a GPU step).
        ``edges_t``: the edge values at t, when the caller has them already.
        The records live in one buffer per solver, refilled by every call: the pointer
        returned is valid until the next call (the C entry points copy the records
        before returning)."""
        at_t = edge_values(self.bcs, t) if edges_t is None else edges_t
        pm = per_member([rain_rate] + at_t + edge_values(self.bcs, t + dt), self.B)
        a = self._params_rec
        a["dt"], a["t"], a["rain"] = float(dt), float(t), pm[0]
        a["bc_t"], a["bc_t_dt"] = pm[1:5].T, pm[5:9].T
        return self._params_ptr

    def step(self, dt: float, t: float, rain_rate=0.0, edges_t=None) -> StepVolumes:
        """One SSP-RK2 step, enqueued on the current stream without waiting for it; the
        volumes are float64 device tensors, as the reference's are."""
        vols = torch.empty((self.B, 5), dtype=torch.float64, device=self.device)
        self.step_into(dt, t, rain_rate, edges_t, vols.data_ptr())
        cols = vols.t().unbind(0) if self.bshape else vols[0].unbind(0)
        return StepVolumes(*cols, table=vols)

    def step_into(self, dt: float, t: float, rain_rate, edges_t, vols_ptr: int, stream: int | None = None) -> None:
        """The step with its (B, 5) float64 volumes written to ``vols_ptr`` (device or
        page-locked memory) on ``stream`` (default: the current stream)."""
        params = self.step_params(dt, t, rain_rate, edges_t)
        with _lib.on_device(self.device):
            _lib.check(self._lib.his_grid_step_async(self._handle, params, vols_ptr,
                                                     _lib.stream_handle() if stream is None else stream),
                       "his_grid_step_async")

    def step_ledger(self, dt: float, t: float, rain_rate, edges_t, ledger_ptr: int, stream: int | None = None) -> None:
        """The step with its volume terms added into an 8 x B float64 device ledger
        (``MassBalance.device_ledger``) by the step's own finalize kernel, on ``stream``."""
        params = self.step_params(dt, t, rain_rate, edges_t)
        with _lib.on_device(self.device):
            _lib.check(self._lib.his_grid_step_ledger_async(self._handle, params, ledger_ptr,
                                                            _lib.stream_handle() if stream is None else stream),
                       "his_grid_step_ledger_async")

    def scratch_bytes(self) -> int:
        return int(self._lib.his_grid_scratch_bytes(self._handle))


__all__ = ["SWE2D", "StepVolumes", "EdgeBC", "EDGES"]
