"""Work-decomposition tuner of the 2-D stage kernels.

The strip kernels split every member's grid into strips of at most ``tile_x``
columns (CTAs of 64, 128, 224 or 352 threads for up to 58, 122, 218 or 346
columns) and chunks of at most ``tile_y`` rows (``his_grid_create``).  The fastest split depends on the
grid sizes, the batch and the precision: narrow strips recompute more halo
columns, short chunks more halo rows, and the number of strip-chunks decides how
evenly the CTAs fill the GPU (152 SMs, 14 resident 64-thread CTAs each in float32).

``choose_tile`` times every candidate the way the engine runs it: the members split
into that decomposition's default number of chains (``his_engine_default_chains``,
at tile-balanced member boundaries), one grid set per chain stepped on its own
stream, all side by side.  It works on throw-away copies of the members' state (the
fields are shared read-only), keeps the fastest and caches the choice per device,
precision, spatial order and batch shape, in memory and in a JSON file
(``$HIS_GB300_TUNE_CACHE``, default ``~/.cache/his_gb300/tiles.json``).

The decomposition changes only the order in which the volume partials are summed
(in the compute type within a strip-chunk, in float64 across them), never a cell's
arithmetic: every candidate gives the same state.
"""
from __future__ import annotations

import ctypes as C
import json
import os
import threading
from collections import Counter
from pathlib import Path

import numpy as np
import torch

from . import _lib

CANDIDATES_X = (58, 122, 218, 346)
CANDIDATES_Y = (16, 24, 32, 40, 48, 64, 96, 128)
WARMUP_MS = 200.0        # busy the GPU before timing, so no candidate runs at ramping clocks
TIMED_STEPS = 5          # steps per timing; each candidate keeps its best of ROUNDS timings
ROUNDS = 3

_MEM: dict[str, tuple[int, int]] = {}
_LOCK = threading.Lock()


def cache_path() -> Path:
    p = os.environ.get("HIS_GB300_TUNE_CACHE")
    return Path(p) if p else Path.home() / ".cache" / "his_gb300" / "tiles.json"


def tune_key(device: torch.device, prec: int, order: int, shapes: list[tuple[int, int]]) -> str:
    name = torch.cuda.get_device_name(device)
    hist = sorted(Counter(shapes).items())
    return f"{name}|prec{prec}|o{order}|" + ";".join(f"{ny}x{nx}*{k}" for (ny, nx), k in hist)


def _load_file() -> dict:
    try:
        return json.loads(cache_path().read_text())
    except (OSError, ValueError):
        return {}


def _store_file(key: str, tile: tuple[int, int], times: dict) -> None:
    p = cache_path()
    try:
        p.parent.mkdir(parents=True, exist_ok=True)
        data = _load_file()
        data[key] = {"tile": list(tile), "ms": times}
        tmp = p.with_suffix(f".{os.getpid()}.tmp")
        tmp.write_text(json.dumps(data, indent=1, sort_keys=True))
        os.replace(tmp, p)
    except OSError:
        pass                                   # a read-only home only loses the cache


def strip_threads(tx: int) -> int:
    """Threads of a strip CTA for strips of at most tx columns (3-column halo each side)."""
    for nt in (64, 128, 224, 352):
        if tx <= nt - 6:
            return nt
    raise ValueError(f"strip width {tx} above 346")


def candidates(shapes: list[tuple[int, int]]) -> list[tuple[int, int]]:
    """Distinct decompositions: candidates that give the same strips and chunks for every
    member are timed once."""
    seen, out = set(), []
    for tx in CANDIDATES_X:
        for ty in CANDIDATES_Y:
            sig = []
            for ny, nx in set(shapes):
                ns = -(-nx // tx)
                nch = -(-ny // ty)
                sig.append((ny, nx, -(-nx // ns), -(-ny // nch), strip_threads(tx)))
            sig = tuple(sorted(sig))
            if sig not in seen:
                seen.add(sig)
                out.append((tx, ty))
    return out


def tiles_per_member(shapes: list[tuple[int, int]], tile: tuple[int, int]) -> list[int]:
    """Strip-chunks of each member for a decomposition (his_grid_create's split)."""
    tx, ty = tile
    return [(-(-nx // tx)) * (-(-ny // ty)) for ny, nx in shapes]


def chain_bounds(counts: list[int], k: int) -> list[int]:
    """Member boundaries of k chains at the nearest shares of the tiles, every chain
    at least one member (the engine's split)."""
    n = len(counts)
    tile0 = np.concatenate([[0], np.cumsum(counts)]).astype(np.int64)
    total = int(tile0[-1])
    bounds, m = [0], 0
    for c in range(1, k):
        want = total * c // k
        m = max(m + 1, 1)
        while m < n - (k - c) and tile0[m] < want:
            m += 1
        bounds.append(m)
    bounds.append(n)
    return bounds


def _time_chained(lib, sets, streams, main, steps) -> float:
    """Mean device time of one step of every grid set, the sets side by side on
    their own streams."""
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(main)
    for s in streams[:len(sets)]:
        s.wait_event(e0)
    for _ in range(steps):
        for (g, params), s in zip(sets, streams):
            _lib.check(lib.his_grid_step_async(g, params, None, s.cuda_stream), "his_grid_step_async")
    for s in streams[:len(sets)]:
        ev = torch.cuda.Event()
        ev.record(s)
        main.wait_event(ev)
    e1.record(main)
    e1.synchronize()
    return e0.elapsed_time(e1) / steps


def choose_tile(device: torch.device, prec: int, cfg, descs, states: list[list[torch.Tensor]],
                use_cache: bool = True) -> tuple[int, int]:
    """Fastest (tile_x, tile_y) for a grid set described by ``descs`` (GridDesc array)
    whose per-member state tensors are ``states[b] = [h, hu, hv, s_filled, infil_cum]``."""
    n = len(states)
    shapes = [(int(descs[b].ny), int(descs[b].nx)) for b in range(n)]
    key = tune_key(device, prec, int(cfg.spatial_order), shapes)
    with _LOCK:
        if use_cache:
            if key in _MEM:
                return _MEM[key]
            hit = _load_file().get(key)
            if hit:
                _MEM[key] = tuple(hit["tile"])
                return _MEM[key]
        lib = _lib.load()
        cfgc = _lib.solver_cfg(cfg)
        copies = []
        tdesc = (_lib.GridDesc * n)()
        with torch.cuda.device(device):
            for b in range(n):
                c = [x.clone() for x in states[b]]
                copies.append(c)
                d = _lib.GridDesc.from_buffer_copy(descs[b])
                d.h, d.hu, d.hv, d.s_filled, d.infil_cum = (x.data_ptr() for x in c)
                d.peak_h = d.peak_speed = None
                tdesc[b] = d
            # a representative step: each member's own CFL step of its current state
            probe = C.c_void_p()
            _lib.check(lib.his_grid_create(prec, C.byref(cfgc), n, tdesc, 0, 0, C.byref(probe)), "his_grid_create")
            rate = np.zeros(n)
            stream = torch.cuda.current_stream(device)
            try:
                _lib.check(lib.his_grid_max_rate(probe, _lib.as_p(rate), stream.cuda_stream), "his_grid_max_rate")
            finally:
                lib.his_grid_destroy(probe)
            params = (_lib.StepParams * n)()
            for b in range(n):
                dt = cfg.cfl / rate[b] if rate[b] > 0 else cfg.dt_max
                params[b].dt = float(min(max(dt, cfg.dt_min), cfg.dt_max))
                params[b].t = 0.0
                params[b].rain = 1e-5
            cands = candidates(shapes)
            streams = [torch.cuda.Stream(device) for _ in range(8)]
            sets = {}
            try:
                for tile in cands:
                    counts = tiles_per_member(shapes, tile)
                    k = int(lib.his_engine_default_chains(n, sum(counts)))
                    bounds = chain_bounds(counts, k)
                    sets[tile] = []
                    for b0, b1 in zip(bounds[:-1], bounds[1:]):
                        sub_desc = (_lib.GridDesc * (b1 - b0))(*[tdesc[b] for b in range(b0, b1)])
                        sub_par = (_lib.StepParams * (b1 - b0))(*[params[b] for b in range(b0, b1)])
                        g = C.c_void_p()
                        _lib.check(lib.his_grid_create(prec, C.byref(cfgc), b1 - b0, sub_desc, tile[0], tile[1],
                                                       C.byref(g)), "his_grid_create")
                        sets[tile].append((g, sub_par))
                # warm up on the first candidate until the clocks have settled
                first = sets[cands[0]]
                per = _time_chained(lib, first, streams, stream, 1)
                _time_chained(lib, first, streams, stream, max(1, int(WARMUP_MS / max(per, 1e-3))))
                best = {tile: float("inf") for tile in cands}
                for _ in range(ROUNDS):                      # interleaved rounds, best per candidate
                    for tile in cands:
                        best[tile] = min(best[tile], _time_chained(lib, sets[tile], streams, stream, TIMED_STEPS))
            finally:
                torch.cuda.synchronize(device)
                for grid_sets in sets.values():
                    for g, _ in grid_sets:
                        lib.his_grid_destroy(g)
            times = {f"{tx}x{ty}": ms for (tx, ty), ms in best.items()}
        del copies
        best = min(times, key=times.get)
        tile = tuple(int(v) for v in best.split("x"))
        _MEM[key] = tile
        if use_cache:
            _store_file(key, tile, times)
        return tile


ENGINE_CANDIDATES_X = (58, 122)   # wider strips were never the fastest for the engine
ENGINE_STEPS = 32                  # timed engine steps per candidate and round (two captured graphs)


def choose_tile_engine(storms, cfg, precision: str, device: torch.device, couple: bool = True,
                       use_cache: bool = True) -> tuple[int, int]:
    """Fastest (tile_x, tile_y) for a device-resident engine over ``storms``, timed as
    the engine itself runs: for every distinct decomposition an engine is built over
    one throw-away copy of the members (state, fields and network), in that
    decomposition's default member chains, and the advance of ENGINE_STEPS captured
    steps is timed with CUDA events, best of ROUNDS interleaved rounds.  Timing the
    grid step alone (``choose_tile``) misses how each chain's per-step kernels and
    the side-stream network interleave with the 2-D stages, and ranked the
    decompositions differently.  Cached like ``choose_tile`` under its own key."""
    from .engine import FloodEngine, Member
    dtype = torch.float64 if precision == "fp64" else torch.float32
    prec = _lib.PREC_F64 if precision == "fp64" else _lib.PREC_F32
    shapes = [(int(s.terrain.ny), int(s.terrain.nx)) for s in storms]
    key = tune_key(device, prec, int(cfg.spatial_order), shapes) + f"|engine|coupled{int(bool(couple))}"
    with _LOCK:
        if use_cache:
            if key in _MEM:
                return _MEM[key]
            hit = _load_file().get(key)
            if hit:
                _MEM[key] = tuple(hit["tile"])
                return _MEM[key]
    cands = [t for t in candidates(shapes) if t[0] in ENGINE_CANDIDATES_X]
    zcache: dict = {}
    members = [Member(s, dtype, device, couple, False, zcache) for s in storms]
    stream = torch.cuda.current_stream(device)
    best = {tile: float("inf") for tile in cands}
    engines = {}
    try:
        for tile in cands:
            fe = FloodEngine(members, cfg, precision, device, tile=tile, graph_steps=16)
            fe.prepare(ENGINE_STEPS)
            engines[tile] = fe
        # warm up on the first candidate until the clocks have settled
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        first = engines[cands[0]]
        e0.record(stream)
        first.advance(ENGINE_STEPS)
        e1.record(stream)
        e1.synchronize()
        per = max(e0.elapsed_time(e1) / ENGINE_STEPS, 1e-3)
        first.advance(max(ENGINE_STEPS, int(WARMUP_MS / per) // 16 * 16))
        for _ in range(ROUNDS):
            for tile in cands:
                e0.record(stream)
                engines[tile].advance(ENGINE_STEPS)
                e1.record(stream)
                e1.synchronize()
                best[tile] = min(best[tile], e0.elapsed_time(e1) / ENGINE_STEPS)
    finally:
        torch.cuda.synchronize(device)
        for fe in engines.values():
            fe.close()
        del members
    times = {f"{tx}x{ty}": ms for (tx, ty), ms in best.items()}
    tile = tuple(int(v) for v in min(times, key=times.get).split("x"))
    with _LOCK:
        _MEM[key] = tile
        if use_cache:
            _store_file(key, tile, times)
    return tile


__all__ = ["choose_tile", "choose_tile_engine", "candidates", "tune_key", "cache_path", "tiles_per_member",
           "chain_bounds"]
