"""ORACLE -- test infrastructure only.

Python front end of the C restatement in ``swe_oracle.c``: float64 numpy state,
one C call per member.  Only tests/, ``__graft_entry__.smoke()`` and bench.py's
CPU-baseline leg may import this module, and only as the checker; the product
path (``his_gb300``) never imports it.

Parity of this oracle with the reference is pinned by tests/test_oracle_golden.py
against vectors the reference itself produced (tests/golden/make_golden.py).

Reference map (file:line in the reference project):
  OracleSWE2D.step / max_dt    hydrointel/solver/swe2d.py:186-193, :298-371
  sections_1d                  hydrointel/solver/swe1d.py:204-215
  OracleSWE1D.step / max_dt    hydrointel/solver/swe1d.py:253-262, :312-368
  OracleCoupled.step           hydrointel/solver/coupling.py:201-227
  OracleCoupled.exchange       hydrointel/solver/coupling.py:73-124
"""
from __future__ import annotations

import ctypes as C
import math

import numpy as np

from . import build as _build

_F64P = C.POINTER(C.c_double)
_I32P = C.POINTER(C.c_int32)
_I64P = C.POINTER(C.c_int64)

EDGES = ("west", "east", "south", "north")
BC_CODES = {"closed": 0, "transmissive": 1, "stage": 2, "discharge": 3}


class OrcCfg(C.Structure):
    _fields_ = [(n, C.c_double) for n in ("g", "h_dry", "kp_eps", "cfl", "dt_min", "dt_max", "cfl_1d",
                                           "slot_width_frac", "weir_cw", "exchange_limit", "exchange_relax")] + \
               [("order", C.c_int32), ("hllc", C.c_int32)]


_LIB = None


def lib():
    global _LIB
    if _LIB is None:
        path = _build.build()
        L = C.CDLL(str(path))
        L.orc_max_rate.restype = C.c_double
        L.orc_swe1d_max_rate.restype = C.c_double
        L.orc_max_threads.restype = C.c_int
        _LIB = L
    return _LIB


def set_threads(n: int) -> None:
    lib().orc_set_threads(int(n))


def max_threads() -> int:
    return int(lib().orc_max_threads())


def make_cfg(cfg) -> OrcCfg:
    """``cfg`` is any object with the reference SolverConfig's field names."""
    return OrcCfg(cfg.g, cfg.h_dry, cfg.kp_eps, cfg.cfl, cfg.dt_min, cfg.dt_max, cfg.cfl_1d,
                  cfg.slot_width_frac, cfg.weir_cw, cfg.exchange_limit, cfg.exchange_relax,
                  int(cfg.spatial_order), 1 if cfg.flux == "hllc" else 0)


def _p(a: np.ndarray):
    if a is None:
        return None
    assert a.flags.c_contiguous, "oracle arrays must be C-contiguous"
    if a.dtype == np.float64:
        return a.ctypes.data_as(_F64P)
    if a.dtype == np.int32:
        return a.ctypes.data_as(_I32P)
    if a.dtype == np.int64:
        return a.ctypes.data_as(_I64P)
    raise TypeError(a.dtype)


def _f64(a, shape=None):
    x = np.ascontiguousarray(np.asarray(a, dtype=np.float64))
    if shape is not None:
        x = np.ascontiguousarray(np.broadcast_to(x, shape))
    return x


def _per_member(v, B):
    x = np.asarray(v, dtype=np.float64).reshape(-1)
    if x.size == 1:
        return np.full(B, float(x[0]))
    if x.size != B:
        raise ValueError(f"expected 1 or {B} values per step quantity, got {x.size}")
    return x


class OracleSWE2D:
    """The 2-D solver: state (B, ny, nx) float64; B = 1 when unbatched."""

    def __init__(self, z, manning, dx, cfg, bcs, storage=None, horton=None, rain_weight=None, dy=None,
                 batch=None):
        self.cfg = cfg
        self.c = make_cfg(cfg)
        self.z = _f64(z)
        self.ny, self.nx = self.z.shape[-2:]
        self.batch = batch
        self.B = 1 if batch is None else int(batch)
        shp = (self.B, self.ny, self.nx)
        self.n = _f64(manning, shp)
        self.dx = float(dx)
        self.dy = float(dy if dy is not None else dx)
        self.area = self.dx * self.dy
        self.bcs = bcs
        self.bc = np.array([BC_CODES[bcs[e].kind] for e in EDGES], dtype=np.int32)
        self.storage = None if storage is None else _f64(storage, shp)
        if horton is not None:
            f0, fc, k, t0 = horton
            self.f0, self.fc, self.k, self.t0 = _f64(f0, shp), _f64(fc, shp), _f64(k, shp), float(t0)
        else:
            self.f0 = self.fc = self.k = None
            self.t0 = 0.0
        self.rain_weight = None if rain_weight is None else _f64(rain_weight, (self.ny, self.nx))
        self.h = np.zeros(shp)
        self.hu = np.zeros(shp)
        self.hv = np.zeros(shp)
        self.s_filled = np.zeros(shp)
        self.infil_cum = np.zeros(shp)
        self.n_dt_clamped = 0

    def set_state(self, h, hu=None, hv=None):
        shp = (self.B, self.ny, self.nx)
        self.h = _f64(h, shp).copy()
        self.hu = np.zeros(shp) if hu is None else _f64(hu, shp).copy()
        self.hv = np.zeros(shp) if hv is None else _f64(hv, shp).copy()

    def edge_values(self, t):
        out = []
        for e in EDGES:
            bc = self.bcs[e]
            if bc.kind in ("stage", "discharge"):
                v = bc.value(t) if callable(bc.value) else bc.value
                out.append(_per_member(v, self.B))
            else:
                out.append(np.zeros(self.B))
        return np.stack(out, axis=1)      # (B, 4)

    def max_rate(self) -> float:
        L = lib()
        return max(L.orc_max_rate(C.byref(self.c), self.ny, self.nx, C.c_double(self.dx), C.c_double(self.dy),
                                  _p(self.h[b]), _p(self.hu[b]), _p(self.hv[b])) for b in range(self.B))

    def max_dt(self) -> float:
        m = self.max_rate()
        cfg = self.cfg
        dt = cfg.cfl / m if m > 0 else cfg.dt_max
        if dt < cfg.dt_min or dt > cfg.dt_max:
            if dt < cfg.dt_min:
                self.n_dt_clamped += 1
            dt = min(max(dt, cfg.dt_min), cfg.dt_max)
        return dt

    def _zb(self, b):
        return self.z if self.z.ndim == 2 else self.z[b]

    def rhs(self, b, vals, dt, h=None, hu=None, hv=None):
        """One right-hand side evaluation (used by the unit tests of the kernels' stages)."""
        h = self.h[b] if h is None else np.ascontiguousarray(h)
        hu = self.hu[b] if hu is None else np.ascontiguousarray(hu)
        hv = self.hv[b] if hv is None else np.ascontiguousarray(hv)
        d = [np.zeros((self.ny, self.nx)) for _ in range(3)]
        q = np.zeros(2)
        lib().orc_rhs(C.byref(self.c), self.ny, self.nx, C.c_double(self.dx), C.c_double(self.dy), _p(self.bc),
                      _p(np.ascontiguousarray(vals, dtype=np.float64)), _p(self._zb(b)), _p(h), _p(hu), _p(hv),
                      C.c_double(dt), _p(d[0]), _p(d[1]), _p(d[2]), _p(q))
        return d[0], d[1], d[2], q

    def step(self, dt, t, rain_rate=0.0):
        """Returns per-member volumes dict of (B,) arrays (bnd_in, bnd_out, rain, infil, clip)."""
        L = lib()
        rain = _per_member(rain_rate, self.B)
        v0, v1 = self.edge_values(t), self.edge_values(t + dt)
        vols = np.zeros((self.B, 5))
        for b in range(self.B):
            vol = np.zeros(5)
            L.orc_swe2d_step(C.byref(self.c), self.ny, self.nx, C.c_double(self.dx), C.c_double(self.dy),
                             _p(self.bc), _p(np.ascontiguousarray(v0[b])), _p(np.ascontiguousarray(v1[b])),
                             _p(self._zb(b)), _p(self.n[b]),
                             _p(self.storage[b]) if self.storage is not None else None,
                             _p(self.f0[b]) if self.f0 is not None else None,
                             _p(self.fc[b]) if self.fc is not None else None,
                             _p(self.k[b]) if self.k is not None else None, C.c_double(self.t0),
                             _p(self.rain_weight), C.c_double(dt), C.c_double(t), C.c_double(rain[b]),
                             _p(self.h[b]), _p(self.hu[b]), _p(self.hv[b]), _p(self.s_filled[b]),
                             _p(self.infil_cum[b]), _p(vol))
            vols[b] = vol
        keys = ("bnd_in", "bnd_out", "rain", "infil", "clip")
        return {k: vols[:, i] for i, k in enumerate(keys)}

    def volume(self):
        return self.h.sum(axis=(-2, -1)) * self.area

    def storage_volume(self):
        return self.s_filled.sum(axis=(-2, -1)) * self.area


def sections_1d(topo, cfg, z=None, b=None):
    """Cell and face sections from a flattened topology (swe1d.py:204-215).
    ``z`` / ``b`` may carry a leading member axis (bed and bottom width differ per member)."""
    z = np.asarray(topo.z if z is None else z, dtype=np.float64)
    b = np.asarray(topo.b if b is None else b, dtype=np.float64)
    m, zbank = np.asarray(topo.m, float), np.asarray(topo.zbank, float)
    yb = np.maximum(zbank - z, 0.2)
    ts = cfg.slot_width_frac * (b + 2 * m * yb)
    fl, fr = np.asarray(topo.face_l), np.asarray(topo.face_r)
    zf = np.maximum(z[..., fl], z[..., fr])
    bank_f = 0.5 * (zbank[fl] + zbank[fr])
    ybf = np.maximum(bank_f - zf, 0.1)
    bf, mf = 0.5 * (b[..., fl] + b[..., fr]), 0.5 * (m[fl] + m[fr])
    tsf = cfg.slot_width_frac * (bf + 2 * mf * ybf)
    shp = z.shape
    return {"b": _f64(b, shp), "m": _f64(m, shp), "yb": _f64(yb, shp), "ts": _f64(ts, shp),
            "fb": _f64(bf), "fm": _f64(np.broadcast_to(mf, bf.shape)), "fyb": _f64(ybf), "fts": _f64(tsf)}


class OracleSWE1D:
    """The 1-D network solver on a flattened topology; state (B, n_cells)."""

    def __init__(self, topo, cfg, batch=None, z=None, b=None, inflow=None, stage=None):
        self.topo, self.cfg, self.c = topo, cfg, make_cfg(cfg)
        self.batch = batch
        self.B = 1 if batch is None else int(batch)
        n = int(topo.n_cells)
        self.n_cells, self.n_faces = n, len(topo.face_l)
        zz = np.asarray(topo.z if z is None else z, dtype=np.float64)
        bb = np.asarray(topo.b if b is None else b, dtype=np.float64)
        self.z = _f64(zz, (self.B, n))
        sec = sections_1d(topo, cfg, self.z, _f64(bb, (self.B, n)))
        self.sec = sec
        self.kind = np.ascontiguousarray(topo.kind, dtype=np.int32)
        self.gsrc = np.ascontiguousarray(topo.ghost_src, dtype=np.int32)
        self.gsign = np.ascontiguousarray(topo.ghost_sign, dtype=np.float64)
        self.fl = np.ascontiguousarray(topo.face_l, dtype=np.int32)
        self.fr = np.ascontiguousarray(topo.face_r, dtype=np.int32)
        self.nman = _f64(topo.n)
        self.dx = _f64(topo.dx)
        self.inflow, self.stage = inflow, stage
        self.A = np.zeros((self.B, n))
        self.Q = np.zeros((self.B, n))

    def _sec(self, k, b):
        return _p(np.ascontiguousarray(self.sec[k][b]))

    def max_dt(self) -> float:
        L = lib()
        best, wet = 0.0, False
        for b in range(self.B):
            any_wet = C.c_int32(0)
            r = L.orc_swe1d_max_rate(C.byref(self.c), self.n_cells, _p(self.kind), self._sec("b", b),
                                     self._sec("m", b), self._sec("yb", b), self._sec("ts", b), _p(self.dx),
                                     _p(self.A[b]), _p(self.Q[b]), C.byref(any_wet))
            wet |= bool(any_wet.value)
            best = max(best, r)
        if not wet:
            return self.cfg.dt_max
        return min(self.cfg.cfl_1d / best, self.cfg.dt_max)

    def step(self, dt, t):
        L = lib()
        q_in = _per_member(self.inflow(t) if self.inflow is not None else 0.0, self.B)
        eta = _per_member(self.stage(t) if self.stage is not None else 0.0, self.B)
        out = np.zeros((self.B, 3))
        for b in range(self.B):
            o = np.zeros(3)
            L.orc_swe1d_step(C.byref(self.c), self.n_cells, self.n_faces, _p(self.kind), _p(self.gsrc),
                             _p(self.gsign), _p(self.fl), _p(self.fr), _p(self.z[b]), _p(self.nman), _p(self.dx),
                             self._sec("b", b), self._sec("m", b), self._sec("yb", b), self._sec("ts", b),
                             self._sec("fb", b), self._sec("fm", b), self._sec("fyb", b), self._sec("fts", b),
                             C.c_double(q_in[b]), C.c_double(eta[b]), C.c_double(dt),
                             _p(self.A[b]), _p(self.Q[b]), _p(o))
            out[b] = o
        return {"bnd_in": out[:, 0], "bnd_out": out[:, 1], "clip": out[:, 2]}

    def volume(self):
        interior = (self.kind <= 1).astype(np.float64)
        return (self.A * self.dx * interior).sum(axis=-1)


class OracleLinks:
    """Link arrays: cell1d, zbank, length, z2 per link; inv -> unique 2-D cell; uniq flat 2-D index."""

    def __init__(self, cell1d, zbank, length, z2, inv, uniq):
        self.cell1d = np.ascontiguousarray(cell1d, dtype=np.int32)
        self.zbank = _f64(zbank)
        self.length = _f64(length)
        self.z2 = _f64(z2)
        self.inv = np.ascontiguousarray(inv, dtype=np.int32)
        self.uniq = np.ascontiguousarray(uniq, dtype=np.int64)
        self.n_links, self.n_unique = len(self.cell1d), len(self.uniq)


def exchange(one: OracleSWE1D, two: OracleSWE2D, links: OracleLinks, dt: float):
    """Move water between the models in place; returns per-link volumes (B, n_links)."""
    L = lib()
    V = np.zeros((one.B, links.n_links))
    for b in range(one.B):
        h = two.h[b].reshape(-1)
        hu = two.hu[b].reshape(-1)
        hv = two.hv[b].reshape(-1)
        v = np.zeros(links.n_links)
        L.orc_exchange(C.byref(one.c), links.n_links, links.n_unique, one.n_cells, _p(links.cell1d),
                       _p(links.zbank), _p(links.length), _p(links.z2), _p(links.inv), _p(links.uniq),
                       _p(one.z[b]), _p(one.dx), one._sec("b", b), one._sec("m", b), one._sec("yb", b),
                       one._sec("ts", b), C.c_double(two.area), C.c_double(dt), _p(h), _p(hu), _p(hv),
                       _p(one.A[b]), _p(v))
        V[b] = v
    return V


TERMS = ("rain", "infiltration", "bnd2d_in", "bnd2d_out", "bnd1d_in", "bnd1d_out", "clip")


class OracleCoupled:
    """The coupled step of coupling.py:201-227 over the oracle's 2-D and 1-D solvers."""

    def __init__(self, two: OracleSWE2D, one: OracleSWE1D | None, links: OracleLinks | None, cfg, rain=None):
        self.two, self.one, self.links, self.cfg = two, one, links, cfg
        self.rain = rain or (lambda t: 0.0)
        self.acc = {k: np.zeros(two.B) for k in TERMS}
        # exchanged volume per member, 2-D -> 1-D and 1-D -> 2-D, and the links that moved
        # water at least once (diagnostics: which parts of the coupling a run exercised)
        self.exch = np.zeros((two.B, 2))
        self.links_active = np.zeros((two.B, links.n_links if links is not None else 0), dtype=bool)
        self.v0 = self.total_volume()
        self.steps = 0

    def total_volume(self):
        v = self.two.volume() + self.two.storage_volume()
        if self.one is not None:
            v = v + self.one.volume()
        return v

    def step(self, t, t_limit, dt=None, n_sub=None):
        two, one = self.two, self.one
        dt = min(two.max_dt() if dt is None else dt, t_limit - t)
        if one is not None:
            if n_sub is None:
                n_sub = max(1, math.ceil(dt / one.max_dt() - 1e-9))
            V = exchange(one, two, self.links, dt)
            self.exch[:, 0] += np.where(V > 0, V, 0.0).sum(axis=1)
            self.exch[:, 1] += np.where(V < 0, -V, 0.0).sum(axis=1)
            self.links_active |= V != 0
        vol = two.step(dt, t, self.rain(t))
        a = self.acc
        a["rain"] += vol["rain"]; a["infiltration"] += vol["infil"]; a["clip"] += vol["clip"]
        a["bnd2d_in"] += vol["bnd_in"]; a["bnd2d_out"] += vol["bnd_out"]
        if one is not None:
            sub = dt / n_sub
            for k in range(n_sub):
                v1 = one.step(sub, t + k * sub)
                a["bnd1d_in"] += v1["bnd_in"]; a["bnd1d_out"] += v1["bnd_out"]; a["clip"] += v1["clip"]
        self.steps += 1
        return t + dt

    def mass_error(self):
        a = self.acc
        net = a["rain"] - a["infiltration"] + a["bnd2d_in"] - a["bnd2d_out"] + a["bnd1d_in"] - a["bnd1d_out"]
        gross = a["rain"] + a["infiltration"] + a["bnd2d_in"] + a["bnd2d_out"] + a["bnd1d_in"] + a["bnd1d_out"]
        dv = self.total_volume() - self.v0
        return np.abs(dv - net) / np.maximum(gross, 1e-9 * np.abs(self.v0) + 1.0)


__all__ = ["OracleSWE2D", "OracleSWE1D", "OracleLinks", "OracleCoupled", "exchange", "sections_1d",
           "make_cfg", "set_threads", "max_threads", "lib"]
