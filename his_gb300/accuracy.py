"""Error of a production-form result against the float64 method on the same storm:
peak depth, flood arrival time and volume, the figures a float32 run reports beside
its speed.

Arrival time is the first output time at which a cell's depth reaches a threshold
(0.1 m by default), read from the output series, so it resolves to the output
interval. The reference has no arrival field; its FloodResult holds the same series
(hydrointel/api.py:62-82), from which this is computed the same way on both runs.
"""
from __future__ import annotations

import numpy as np


def _np(a) -> np.ndarray:
    if hasattr(a, "detach"):
        return a.detach().to("cpu").double().numpy()
    return np.asarray(a, dtype=np.float64)


def arrival_times(depth_series, times, threshold: float = 0.1) -> np.ndarray:
    """First time at which each cell's depth reaches ``threshold`` (NaN: never), from
    an (nt, ny, nx) series at ``times`` (nt,)."""
    h = _np(depth_series)
    t = _np(times)
    if h.shape[0] != t.shape[0]:
        raise ValueError(f"{h.shape[0]} snapshots but {t.shape[0]} times")
    out = np.full(h.shape[1:], np.nan)
    if h.shape[0] == 0:
        return out
    reached = h >= threshold
    first = reached.argmax(axis=0)
    ever = reached.any(axis=0)
    out[ever] = t[first[ever]]
    return out


def compare(test, ref, threshold: float = 0.1, wet: float = 1e-3) -> dict:
    """Errors of FloodResult ``test`` against FloodResult ``ref`` of the same storm.

    Peak depth: max and RMSE over cells wet (peak > ``wet``) in either run. Arrival:
    max and RMSE over cells that reach ``threshold`` in both runs, plus the number of
    cells that reach it in only one. Volume: relative difference of the final surface
    volume (sum of the last depth snapshot) and of the infiltrated and stored volumes."""
    p_t, p_r = _np(test.depth_max), _np(ref.depth_max)
    if p_t.shape != p_r.shape:
        raise ValueError(f"grids differ: {p_t.shape} and {p_r.shape}")
    sel = (p_t > wet) | (p_r > wet)
    d = (p_t - p_r)[sel]
    a_t = arrival_times(test.depth_series, test.times, threshold)
    a_r = arrival_times(ref.depth_series, ref.times, threshold)
    both = ~np.isnan(a_t) & ~np.isnan(a_r)
    only = int((np.isnan(a_t) != np.isnan(a_r)).sum())
    da = (a_t - a_r)[both]
    h_t, h_r = _np(test.depth_series), _np(ref.depth_series)
    v_t = float(h_t[-1].sum()) if len(h_t) else 0.0
    v_r = float(h_r[-1].sum()) if len(h_r) else 0.0
    rel = lambda x, y: abs(x - y) / max(abs(y), 1e-12)
    return {
        "peak_depth_max_m": float(np.abs(d).max()) if d.size else 0.0,
        "peak_depth_rmse_m": float(np.sqrt(np.mean(d ** 2))) if d.size else 0.0,
        "wet_cells": int(sel.sum()),
        "arrival_threshold_m": float(threshold),
        "arrival_max_s": float(np.abs(da).max()) if da.size else 0.0,
        "arrival_rmse_s": float(np.sqrt(np.mean(da ** 2))) if da.size else 0.0,
        "arrival_cells": int(both.sum()),
        "arrival_cells_in_one_run_only": only,
        "output_interval_s": float(np.diff(_np(ref.times)).min()) if len(ref.times) > 1 else 0.0,
        "final_surface_volume_rel": rel(v_t, v_r),
        "infiltrated_volume_rel": rel(float(test.infiltrated_volume_m3), float(ref.infiltrated_volume_m3)),
        "stored_volume_rel": rel(float(test.stored_volume_m3), float(ref.stored_volume_m3)),
    }


__all__ = ["arrival_times", "compare"]
