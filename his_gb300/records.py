"""Dataset records of finished storms, in the layout of the reference's dataset
writer (hydrointel/data/generate.py:37-63 record paths and gzip save/load, :104-110
storage-grid coarsening, :355-397 the per-simulation record and its index entry,
:409-425 the volume ledger and tensor conversion), so that served or batched storms
feed the surrogate's training data directly.

A record holds the output series block-averaged to the storage grid (a store factor
f: depths by area mean, velocities weighted by depth), the full-resolution peak
depth, the channel level and discharge, the storm's fields on the storage grid, its
forcing sampled at the model's forcing steps, the volumes and ledger, and the run
statistics.  Records are written as ``sim_#####.pt`` or ``.pt.gz`` with an
``index.json`` beside them.
"""
from __future__ import annotations

import gzip
import json
from pathlib import Path

import numpy as np
import torch

COMPRESSED_SUFFIX = ".pt.gz"
FORCING_STEPS = 64


def record_path(root: Path, sim_id: int, compress: bool | None = None) -> Path:
    """Path of record ``sim_id`` under ``root`` (hydrointel/data/generate.py:37).
    compress True / False picks the gzip or the plain file; None (default) picks the
    gzip file only when it exists and the plain one does not, so a directory of plain
    records resolves to its own files."""
    root = Path(root)
    plain, packed = root / f"sim_{sim_id:05d}.pt", root / f"sim_{sim_id:05d}{COMPRESSED_SUFFIX}"
    if compress is None:
        return packed if packed.exists() and not plain.exists() else plain
    return packed if compress else plain


def save_record(rec: dict, path: Path) -> None:
    path = Path(path)
    if path.name.endswith(COMPRESSED_SUFFIX):
        with gzip.open(path, "wb", compresslevel=1) as fh:
            torch.save(rec, fh)
    else:
        torch.save(rec, path)


def load_record(path: Path) -> dict:
    path = Path(path)
    if path.name.endswith(COMPRESSED_SUFFIX):
        with gzip.open(path, "rb") as fh:
            return torch.load(fh, weights_only=False)
    return torch.load(path, weights_only=False)


def coarsen_mean(a: np.ndarray, f: int) -> np.ndarray:
    """Mean over f x f blocks of the trailing two axes (rows and columns past the last
    whole block are dropped)."""
    if f == 1:
        return a
    *lead, ny, nx = a.shape
    cy, cx = ny // f, nx // f
    return a[..., :cy * f, :cx * f].reshape(*lead, cy, f, cx, f).mean(axis=(-1, -3))


def _tensors(obj):
    if isinstance(obj, dict):
        return {k: _tensors(v) for k, v in obj.items()}
    if isinstance(obj, np.ndarray) and obj.dtype != object and obj.dtype.kind in "fiub":
        return torch.from_numpy(np.ascontiguousarray(obj))
    return obj


def flood_record(storm, res, store_factor: int = 1, forcing_steps: int = FORCING_STEPS) -> dict:
    """The training record of one finished storm from its FloodResult."""
    f = int(store_factor)
    h, u, v = res.depth_series.numpy(), res.u.numpy(), res.v.numpy()
    hc = coarsen_mean(h, f)
    safe = np.where(hc > 0, hc, 1.0)
    uc = np.where(hc > 0, coarsen_mean(h * u, f) / safe, 0.0)
    vc = np.where(hc > 0, coarsen_mean(h * v, f) / safe, 0.0)
    ter = storm.terrain
    shape = (ter.ny, ter.nx)
    full = lambda a: np.broadcast_to(np.asarray(a, dtype=np.float64), shape)
    fields = {"manning": coarsen_mean(full(storm.manning), f).astype(np.float32),
              "storage": coarsen_mean(full(storm.storage if storm.storage is not None else 0.0), f).astype(np.float32)}
    if storm.horton is not None:
        for name, a in zip(("horton_f0", "horton_fc", "horton_k"), storm.horton[:3]):
            fields[name] = coarsen_mean(full(a), f).astype(np.float32)
    fo = storm.forcing
    ts = np.linspace(0.0, storm.t_end, forcing_steps)
    ledger = {}
    if "ledger" in res.extras:
        L = res.extras["ledger"]
        ledger = {k: np.array([row[k] for row in L], np.float64) for k in L[0]} if L else {}
        ledger["v2d_coarse"] = h[:, :(ter.ny // f) * f, :(ter.nx // f) * f].astype(np.float64).sum(axis=(1, 2)) * \
            ter.dx * ter.dx
    run = res.extras.get("run")
    rec = {
        "meta": {"key": storm.key, "ny": ter.ny, "nx": ter.nx, "dx": ter.dx, "t_end": float(storm.t_end),
                 "bc": list(storm.bc)},
        "mass_balance_error": float(res.mass_balance_error),
        "times": res.times.numpy().astype(np.float32),
        "h": hc.astype(np.float32), "u": uc.astype(np.float32), "v": vc.astype(np.float32),
        "depth_max_full": h.max(0).astype(np.float32) if len(h) else np.zeros(shape, np.float32),
        "eta1": res.channel_eta.numpy(), "q1": res.channel_q.numpy(),
        "fields": fields,
        "forcing": {"rain_mmh": np.array([fo.rain_rate(t) * 3.6e6 for t in ts], np.float32),
                    "tide_m": np.array([fo.tide(t) for t in ts], np.float32),
                    "inflow_m3s": np.array([fo.inflow(t) for t in ts], np.float32),
                    "t_end": float(storm.t_end)},
        "volumes": {"infiltrated_m3": float(res.infiltrated_volume_m3), "stored_m3": float(res.stored_volume_m3),
                    "sources": dict(res.extras.get("sources", {}))},
        "ledger": ledger,
        "run_log": {} if run is None else {"steps": run.steps, "dt_min": run.dt_min, "dt_max": run.dt_max,
                                           "n_sub_max": run.n_sub_max, "n_dt_clamped": run.n_dt_clamped,
                                           "status": run.status},
        "store_coarsen": f,
    }
    return _tensors(rec)


def write_records(items, out_dir, store_factor: int = 1, compress: bool = True, first_id: int = 0) -> Path:
    """Write (storm, FloodResult) pairs as records sim_{first_id + i} and merge their
    entries into out_dir/index.json; returns the index path."""
    out = Path(out_dir)
    out.mkdir(parents=True, exist_ok=True)
    index_path = out / "index.json"
    index = json.loads(index_path.read_text()) if index_path.exists() else {}
    for i, (storm, res) in enumerate(items):
        sim_id = first_id + i
        path = record_path(out, sim_id, compress)
        save_record(flood_record(storm, res, store_factor), path)
        h = res.depth_series
        index[str(sim_id)] = {"key": storm.key, "record": path.name, "bytes": path.stat().st_size,
                              "store_coarsen": int(store_factor), "mass_err": float(res.mass_balance_error),
                              "outputs": int(h.shape[0]), "peak_depth": float(h.max()) if h.numel() else 0.0}
    tmp = index_path.with_suffix(".json.tmp")
    tmp.write_text(json.dumps(index, indent=1))
    tmp.replace(index_path)
    return index_path


__all__ = ["coarsen_mean", "flood_record", "write_records", "save_record", "load_record", "record_path"]
