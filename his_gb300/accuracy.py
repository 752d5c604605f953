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


# The reference's own acceptance criteria for a float32 run against float64
# (hydrointel/benchmarks/precision.py:37-44 and criteria.py:40-46); reported beside
# the comparison; the production form's own bar is peak-depth RMSE <= 1 cm.
REFERENCE_FP32_CRITERIA = {
    "mass_balance_error": 1e-4,
    "depth_max_abs_m": 5e-3,
    "depth_rmse_wet_m": 1e-3,
    "peak_depth_max_m": 5e-3,
    "flooded_area_rel": 0.005,
    "reach_peak_discharge_rel": 0.02,
}
AREA_THRESHOLDS_M = (0.15, 0.30, 0.50)


def series_metrics(test, ref, reach_of=None, h_dry: float = 1e-3) -> dict:
    """Output-series agreement in the reference's terms (criteria.py:25-33): depth RMSE
    and 99th-percentile |dh| over every (output time, cell) wet in either run, the
    largest |dh| anywhere, the flooded area (peak depth at 0.15 / 0.30 / 0.50 m, cells
    dry at the start) relative to ``ref``, and per reach the peak of |Q| over time and
    its nodes relative to ``ref`` (``reach_of``: reach index of each output node)."""
    h_t, h_r = _np(test.depth_series), _np(ref.depth_series)
    n = min(len(h_t), len(h_r))
    h_t, h_r = h_t[:n], h_r[:n]
    d = h_t - h_r
    wet = np.maximum(h_t, h_r) > h_dry
    out = {"depth_rmse_wet_m": float(np.sqrt(np.mean(d[wet] ** 2))) if wet.any() else 0.0,
           "depth_p99_abs_m": float(np.percentile(np.abs(d[wet]), 99)) if wet.any() else 0.0,
           "depth_max_abs_m": float(np.abs(d).max()) if d.size else 0.0}
    land = (h_r[0] <= 0.0) & (h_t[0] <= 0.0) if n else None
    rel_area = 0.0
    if n:
        pk_t, pk_r = h_t.max(axis=0), h_r.max(axis=0)
        for thr in AREA_THRESHOLDS_M:
            a_r = float(((pk_r >= thr) & land).sum())
            a_t = float(((pk_t >= thr) & land).sum())
            if a_r > 0:
                rel_area = max(rel_area, abs(a_t - a_r) / a_r)
    out["flooded_area_rel"] = rel_area
    q_t, q_r = _np(test.channel_q)[:n], _np(ref.channel_q)[:n]
    if reach_of is not None and q_r.size:
        reach_of = np.asarray(reach_of)
        worst = 0.0
        for rch in np.unique(reach_of):
            sel = reach_of == rch
            p_r = float(np.abs(q_r[:, sel]).max())
            p_t = float(np.abs(q_t[:, sel]).max())
            if p_r > 0:
                worst = max(worst, abs(p_t - p_r) / p_r)
        out["reach_peak_discharge_rel"] = worst
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


def against_fp64(storms, interval_s: float, cfg=None, chunk: int = 1024, timeout_s: float | None = None):
    """Run ``storms`` to their end twice through the device engine, in the float32
    production form and in the float64 method, with outputs every ``interval_s``, and
    compare each member (``compare``).  Each member keeps its own dt, so a member's
    arithmetic does not depend on the batch it runs in.  Returns one dict per member
    with the comparison, both runs' mass-balance errors, statuses and step counts."""
    from .config import SolverConfig
    from .engine import FloodEngine
    runs = {}
    for prec in ("fp64", "fp32"):
        c = cfg or SolverConfig(slot_width_frac=storms[0].slot_width_frac)
        fe = FloodEngine(list(storms), c, precision=prec, track_peaks=True, output_interval=interval_s)
        reps = fe.run(chunk=chunk, timeout_s=timeout_s)
        res = fe.results(reps)
        runs[prec] = (fe.flood_results(reps), res)
        fe.close()
    out = []
    for b, s in enumerate(storms):
        (f64, r64), (f32, r32) = (runs["fp64"][0][b], runs["fp64"][1][b]), (runs["fp32"][0][b], runs["fp32"][1][b])
        m = compare(f32, f64)
        reach_of = None
        if s.network is not None:
            from .topology import build_topology
            tp = build_topology(s.network)
            reach_of = tp.reach_of[tp.kind <= 1]
        m.update(series_metrics(f32, f64, reach_of))
        # the running maxima over every step, beside the maxima over the output times
        e32, e64 = f32.extras.get("depth_max_every_step"), f64.extras.get("depth_max_every_step")
        if e32 is not None and e64 is not None:
            a, b_ = _np(e32), _np(e64)
            wet = (a > 1e-3) | (b_ > 1e-3)
            d = (a - b_)[wet]
            m["peak_every_step_rmse_m"] = float(np.sqrt(np.mean(d ** 2))) if d.size else 0.0
            m["peak_every_step_max_m"] = float(np.abs(d).max()) if d.size else 0.0
        m.update({"member": s.key, "grid": f"{s.terrain.nx}x{s.terrain.ny}", "t_end_s": float(s.t_end),
                  "status_fp32": r32.status, "status_fp64": r64.status, "steps_fp32": r32.steps,
                  "steps_fp64": r64.steps, "mass_error_fp32": float(r32.mass_error),
                  "mass_error_fp64": float(r64.mass_error),
                  "final_volume_rel": abs(r32.volume - r64.volume) / max(abs(r64.volume), 1.0)})
        out.append(m)
    return out


def reference_criteria(m: dict) -> dict:
    """Each of the reference's float32 acceptance criteria with its value in ``m`` and
    whether it holds (mass balance taken from the float32 run)."""
    vals = dict(m)
    vals.setdefault("mass_balance_error", m.get("mass_error_fp32"))
    return {k: {"value": vals.get(k), "limit": lim, "pass": vals.get(k) is not None and vals[k] <= lim}
            for k, lim in REFERENCE_FP32_CRITERIA.items()}


__all__ = ["arrival_times", "compare", "against_fp64", "series_metrics", "reference_criteria",
           "REFERENCE_FP32_CRITERIA"]
