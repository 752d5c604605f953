"""ctypes binding of ``libhis_gb300.so`` (the C ABI in include/his_gb300.h).

There is no fallback: if the library cannot be built or loaded, importing a
solver raises.  Status codes map to the reference's exceptions: bad arguments to
``ValueError``, implausible or non-finite states to ``NumericalInstabilityError``,
CUDA failures to ``RuntimeError``.
"""
from __future__ import annotations

import ctypes as C
import threading

import numpy as np

from . import build as _build

HIS_OK, HIS_ERR_BAD_ARG, HIS_ERR_NONFINITE, HIS_ERR_IMPLAUSIBLE = 0, 1, 2, 3
HIS_ERR_WAIT_TIMEOUT, HIS_ERR_OOM_ADMISSION, HIS_ERR_CUDA, HIS_ERR_UNSUPPORTED = 4, 5, 6, 7
PREC_F64, PREC_F32 = 0, 1
NOALLOC_SCRATCH_BYTES = 16 * 1024 * 1024     # HIS_NOALLOC_SCRATCH_BYTES

_I32P = C.POINTER(C.c_int32)
_I64P = C.POINTER(C.c_int64)
_F64P = C.POINTER(C.c_double)


class NumericalInstabilityError(RuntimeError):
    """The engine produced a physically impossible state. The run is invalid."""


class SolverCfg(C.Structure):
    _fields_ = [(n, C.c_double) for n in ("g", "h_dry", "kp_eps", "cfl", "dt_min", "dt_max", "cfl_1d",
                                           "slot_width_frac", "weir_cw", "exchange_limit", "exchange_relax")] + \
               [("order", C.c_int32), ("hllc", C.c_int32)]


class GridDesc(C.Structure):
    _fields_ = [("ny", C.c_int32), ("nx", C.c_int32), ("bc", C.c_int32 * 4), ("dx", C.c_double),
                ("dy", C.c_double), ("horton_t0", C.c_double)] + \
               [(n, C.c_void_p) for n in ("h", "hu", "hv", "s_filled", "infil_cum", "z", "manning", "storage",
                                         "f0", "fc", "k", "rain_weight", "peak_h", "peak_speed")]


class StepParams(C.Structure):
    _fields_ = [("dt", C.c_double), ("t", C.c_double), ("rain", C.c_double), ("bc_t", C.c_double * 4),
                ("bc_t_dt", C.c_double * 4)]


class NetDesc(C.Structure):
    _fields_ = [("n_cells", C.c_int32), ("n_faces", C.c_int32), ("kind", _I32P), ("ghost_src", _I32P),
                ("face_l", _I32P), ("face_r", _I32P), ("ghost_sign", _F64P)] + \
               [(n, _F64P) for n in ("z", "manning", "dx", "b", "m", "yb", "ts", "fb", "fm", "fyb", "fts")] + \
               [("A", C.c_void_p), ("Q", C.c_void_p)]


class LinksDesc(C.Structure):
    _fields_ = [("n_links", C.c_int32), ("n_unique", C.c_int32), ("cell1d", _I32P), ("inv", _I32P),
                ("uniq", _I64P), ("zbank", _F64P), ("length", _F64P), ("z2", _F64P)]


class ForcingDesc(C.Structure):
    _fields_ = [("t0", C.c_double), ("t_end", C.c_double), ("rain_t0", C.c_double), ("rain_step", C.c_double),
                ("rain_n", C.c_int32), ("tide_on", C.c_int32), ("rain", _F64P), ("tide_n", C.c_int32),
                ("q_n", C.c_int32), ("tide_base", C.c_double), ("tide_shift", C.c_double),
                ("tide_amp", C.c_double * 4), ("tide_w", C.c_double * 4), ("tide_phase", C.c_double * 4),
                ("q_t0", C.c_double), ("q_step", C.c_double), ("q", _F64P), ("edge_src", C.c_int32 * 4),
                ("edge_val", C.c_double * 4), ("out_dt", C.c_double), ("n_out", C.c_int32), ("pad", C.c_int32)] + \
               [(n, C.c_void_p) for n in ("snap_h", "snap_u", "snap_v", "snap_eta", "snap_q", "snap_t", "snap_ledger")]


class MemberReport(C.Structure):
    _fields_ = [("t", C.c_double), ("dt_last", C.c_double), ("dt_min", C.c_double), ("dt_max", C.c_double),
                ("rate", C.c_double), ("steps", C.c_int64), ("status", C.c_int32), ("n_sub_max", C.c_int32),
                ("n_dt_clamped", C.c_int32), ("outputs", C.c_int32), ("acc", C.c_double * 7)]


STATUS = {0: "running", 1: "done", 2: "non-finite state", 3: "implausible state", 4: "too many 1-D substeps"}

# entry point -> (restype, argtypes); the exact set declared in include/his_gb300.h
_H = C.c_void_p
SIGNATURES = {
    "his_version": (C.c_int32, []),
    "his_last_error": (C.c_char_p, []),
    "his_grid_create": (C.c_int32, [C.c_int32, C.POINTER(SolverCfg), C.c_int32, C.POINTER(GridDesc), C.c_int32,
                                    C.c_int32, C.POINTER(_H)]),
    "his_grid_destroy": (C.c_int32, [_H]),
    "his_grid_scratch_bytes": (C.c_int64, [_H]),
    "his_grid_step": (C.c_int32, [_H, C.POINTER(StepParams), _F64P, C.c_void_p]),
    "his_grid_max_rate": (C.c_int32, [_H, _F64P, C.c_void_p]),
    "his_grid_step_async": (C.c_int32, [_H, C.POINTER(StepParams), C.c_void_p, C.c_void_p]),
    "his_grid_step_ledger_async": (C.c_int32, [_H, C.POINTER(StepParams), C.c_void_p, C.c_void_p]),
    "his_grid_max_rate_async": (C.c_int32, [_H, C.c_void_p, C.c_void_p]),
    "his_grid_step_rate_async": (C.c_int32, [_H, C.c_void_p, C.c_void_p]),
    "his_grid_volumes": (C.c_int32, [_H, _F64P, C.c_void_p]),
    "his_grid_step_noalloc": (C.c_int32, [C.c_int32, C.POINTER(SolverCfg), C.POINTER(GridDesc),
                                          C.POINTER(StepParams), _F64P, C.c_void_p]),
    "his_net_create": (C.c_int32, [C.POINTER(SolverCfg), C.c_int32, C.POINTER(NetDesc), C.POINTER(_H)]),
    "his_net_destroy": (C.c_int32, [_H]),
    "his_net_step": (C.c_int32, [_H, C.c_double, C.c_int32, _F64P, _F64P, C.c_void_p]),
    "his_net_max_rate": (C.c_int32, [_H, _F64P, _I32P, C.c_void_p]),
    "his_net_step_async": (C.c_int32, [_H, C.c_double, C.c_int32, _F64P, C.c_void_p, C.c_void_p]),
    "his_net_step_ledger_async": (C.c_int32, [_H, C.c_double, C.c_int32, _F64P, C.c_void_p, C.c_void_p]),
    "his_net_max_rate_async": (C.c_int32, [_H, C.c_void_p, C.c_void_p]),
    "his_net_volume": (C.c_int32, [_H, _F64P, C.c_void_p]),
    "his_links_create": (C.c_int32, [_H, _H, C.c_int32, C.POINTER(LinksDesc), C.POINTER(_H)]),
    "his_links_destroy": (C.c_int32, [_H]),
    "his_exchange": (C.c_int32, [_H, C.POINTER(SolverCfg), C.c_double, _F64P, C.c_void_p]),
    "his_exchange_async": (C.c_int32, [_H, C.POINTER(SolverCfg), C.c_double, C.c_void_p, C.c_void_p]),
    "his_links_exchanged": (C.c_int32, [_H, _F64P, C.c_int32, C.c_void_p]),
    "his_engine_create": (C.c_int32, [_H, _H, _H, C.c_int32, C.POINTER(ForcingDesc), C.c_int32, C.c_int32,
                                      C.POINTER(_H)]),
    "his_engine_destroy": (C.c_int32, [_H]),
    "his_engine_advance": (C.c_int32, [_H, C.c_int32, C.c_void_p]),
    "his_engine_prepare": (C.c_int32, [_H, C.c_int32]),
    "his_engine_set_chains": (C.c_int32, [_H, C.c_int32]),
    "his_engine_chains": (C.c_int32, [_H]),
    "his_engine_default_chains": (C.c_int32, [C.c_int32, C.c_int32]),
    "his_engine_report": (C.c_int32, [_H, C.POINTER(MemberReport), C.c_void_p]),
    "his_engine_resume": (C.c_int32, [_H, C.POINTER(MemberReport), _I32P, C.c_void_p]),
    "his_engine_profile": (C.c_int32, [_H, C.c_int32, _F64P, C.c_void_p]),
}

_LIB = None
_LOCK = threading.Lock()


def load():
    """Build (if stale) and load the library; raises if that is impossible."""
    global _LIB
    with _LOCK:
        if _LIB is None:
            path = _build.build()
            L = C.CDLL(str(path))
            for name, (res, args) in SIGNATURES.items():
                fn = getattr(L, name)
                fn.restype = res
                fn.argtypes = args
            _LIB = L
    return _LIB


def last_error() -> str:
    """The library's message for the last failed call on this thread."""
    return (load().his_last_error() or b"").decode(errors="replace")


def check(rc: int, what: str) -> None:
    if rc == HIS_OK:
        return
    msg = (_LIB.his_last_error() or b"").decode(errors="replace")
    text = f"{what}: {msg}" if msg else what
    if rc == HIS_ERR_BAD_ARG:
        raise ValueError(text)
    if rc in (HIS_ERR_NONFINITE, HIS_ERR_IMPLAUSIBLE):
        raise NumericalInstabilityError(text)
    raise RuntimeError(f"{text} (status {rc})")


def solver_cfg(cfg) -> SolverCfg:
    return SolverCfg(cfg.g, cfg.h_dry, cfg.kp_eps, cfg.cfl, cfg.dt_min, cfg.dt_max, cfg.cfl_1d, cfg.slot_width_frac,
                     cfg.weir_cw, cfg.exchange_limit, cfg.exchange_relax, int(cfg.spatial_order),
                     1 if cfg.flux == "hllc" else 0)


def ptr(t) -> int | None:
    """Device address of a torch tensor (None for None)."""
    if t is None:
        return None
    assert t.is_cuda and t.is_contiguous(), "device tensors must be contiguous CUDA tensors"
    return t.data_ptr()


def host_array(a, dtype):
    return np.ascontiguousarray(np.asarray(a, dtype=dtype))


def as_p(a: np.ndarray):
    if a.dtype == np.float64:
        return a.ctypes.data_as(_F64P)
    if a.dtype == np.int32:
        return a.ctypes.data_as(_I32P)
    if a.dtype == np.int64:
        return a.ctypes.data_as(_I64P)
    raise TypeError(a.dtype)


def on_device(device):
    """Make ``device`` (a torch.device with an index) current for a block; no switch
    when it already is, which is the common case on the step's hot path."""
    import contextlib
    import torch
    if device.index == torch.cuda.current_device():
        return contextlib.nullcontext()
    return torch.cuda.device(device)


def stream_handle(device=None) -> int:
    import torch
    return torch.cuda.current_stream(device).cuda_stream
