"""Serving form: continuous batching of storm requests on one GPU.

Requests (storms) arrive over time.  A request is admitted as soon as its device
footprint fits the HBM budget and a member slot is free (first come, first served);
its state is built on the device once and stays there until it finishes.  The
engine advances every admitted member in chunks of ``chunk_steps`` steps (CUDA
graphs, each member with its own dt).  Between chunks, finished members retire --
their mass balance, clock and peak fields are read back -- and waiting requests join.
A membership change rebuilds the engine's tables over the same member objects: every
continuing member resumes its clock and accumulators exactly, and every batch uses
the same work decomposition, so a request's result is the same whichever requests
shared the GPU with it.

This replaces the per-storm loop of the reference's dataset generator and batch API
(hydrointel/api.py:256-324 simulate_batch, data/generate.py:229-300), which runs a
fixed batch to its end before starting the next.

    python -m his_gb300.serving --minutes 10 --rate 2
"""
from __future__ import annotations

import argparse
import json
import time
from pathlib import Path
from dataclasses import dataclass, field

import numpy as np
import torch

from .config import SolverConfig
from .engine import FloodEngine, FloodResult, Member, MemberResult, output_count
from .records import write_records
from .swe2d import cuda_device
from .workloads import Storm, served_requests, uneven_member


def estimate_bytes(storm: Storm, dtype: torch.dtype, track_peaks: bool = True,
                   output_interval: float | None = None) -> int:
    """Device bytes a storm needs as a member: 5 state planes, up to 6 field planes,
    3 stage planes, 2 peak planes, its channel network and tables, and with outputs
    three float32 planes and two channel rows per output time."""
    planes = 5 + 2 + 3 + (3 if storm.horton is not None else 0) + (1 if storm.storage is not None else 0) + \
        (2 if track_peaks else 0)
    elem = torch.tensor([], dtype=dtype).element_size()
    net = cells1d = 0
    if storm.network is not None:
        cells1d = sum(r.n for r in storm.network.reaches) + 8 * len(storm.network.reaches)
        net = 64 * 1024 + 40 * 8 * cells1d
    out = 0
    if output_interval is not None:
        n_out = output_count(float(storm.t_end), float(output_interval))
        out = n_out * (3 * 4 * storm.cells + 2 * 4 * cells1d + 8)
    return planes * storm.cells * elem + net + out + 64 * 1024


@dataclass
class Request:
    rid: int
    storm: Storm
    arrival: float                       # seconds after the server started
    admitted: float | None = None
    finished: float | None = None
    result: MemberResult | None = None
    flood: FloodResult | None = None
    peak_h: np.ndarray | None = None
    peak_speed: np.ndarray | None = None
    h: np.ndarray | None = None

    @property
    def latency(self) -> float | None:
        return None if self.finished is None else self.finished - self.arrival


@dataclass
class ServeStats:
    requests: int
    finished: int
    wall_s: float
    storms_per_hour: float
    cell_steps_per_s: float
    latency_p50_s: float
    latency_p99_s: float
    queue_p50_s: float
    queue_p99_s: float
    max_members: int
    rebuilds: int
    max_mass_error: float
    statuses: dict = field(default_factory=dict)


class FloodServer:
    def __init__(self, cfg: SolverConfig | None = None, precision: str = "fp32", device=None,
                 hbm_budget: int | None = None, max_members: int = 512, chunk_steps: int = 256,
                 graph_steps: int = 16, tile=(58, 16), track_peaks: bool = True, keep_state: bool = False,
                 output_interval: float | None = None, record_dir=None, store_factor: int = 1):
        """hbm_budget: device bytes the members may hold (default: 80 % of the free memory
        at start).  tile: the one work decomposition every batch uses; short 16-row
        chunks by default, because a served batch is small and each step is bound by
        the latency of one CTA's march up its chunk (at 2 requests/s: p50 latency 0.86
        s against 1.66 s with 48-row chunks).  keep_state:
        copy each finished member's final depth to the host with its result.
        output_interval: seconds between the outputs of each request; a finished request
        then carries a FloodResult with its series.  record_dir: with outputs, write each
        finished request as a dataset record there (store_factor: its storage grid)."""
        self.cfg = cfg or SolverConfig()
        self.precision = precision
        self.dtype = torch.float64 if precision == "fp64" else torch.float32
        self.device = cuda_device(device)
        if hbm_budget is None:
            free, _ = torch.cuda.mem_get_info(self.device)
            hbm_budget = int(0.8 * free)
        self.hbm_budget = int(hbm_budget)
        self.max_members = int(max_members)
        self.chunk_steps = int(chunk_steps)
        self.graph_steps = int(graph_steps)
        self.tile = tuple(tile)
        self.track_peaks = track_peaks
        self.keep_state = keep_state
        self.output_interval = output_interval
        self.record_dir = None if record_dir is None else Path(record_dir)
        self.store_factor = int(store_factor)
        self.queue: list[Request] = []
        self.active: list[tuple[Request, Member]] = []
        self.done: list[Request] = []
        self.engine: FloodEngine | None = None
        self.used_bytes = 0
        self.rebuilds = 0
        self.cell_steps = 0
        self.max_batch = 0

    # ------------------------------------------------------------ admission
    def _footprint(self, req: Request) -> int:
        return estimate_bytes(req.storm, self.dtype, self.track_peaks, self.output_interval)

    def _admit(self, now: float, n_active: int) -> list[tuple[Request, Member]]:
        joined = []
        while self.queue and n_active + len(joined) < self.max_members:
            req = self.queue[0]
            need = self._footprint(req)
            if self.used_bytes + need > self.hbm_budget:
                if not n_active and not joined:
                    raise ValueError(f"request {req.rid} needs {need} bytes, more than the whole HBM budget "
                                     f"({self.hbm_budget})")
                break
            self.queue.pop(0)
            member = Member(req.storm, self.dtype, self.device, True, self.track_peaks,
                            output_interval=self.output_interval)
            req.admitted = now
            self.used_bytes += need
            joined.append((req, member))
        return joined

    def _retire(self, reps, now: float) -> list[int]:
        results = self.engine.results(reps)
        done = [b for b in range(len(self.active)) if reps[b].status != 0]
        floods = {}
        if self.output_interval is not None and done:
            floods = dict(zip(done, self.engine.flood_results(reps, only=done)))
        gone = []
        for b, (req, member) in enumerate(self.active):
            r = reps[b]
            if r.status == 0:
                continue
            req.finished = now
            req.result = results[b]
            req.flood = floods.get(b)
            if req.flood is not None and self.record_dir is not None:
                write_records([(req.storm, req.flood)], self.record_dir, self.store_factor, first_id=req.rid)
            if member.peak_h is not None:
                req.peak_h = member.peak_h.cpu().numpy()
                req.peak_speed = member.peak_speed.cpu().numpy()
            if self.keep_state:
                req.h = member.h.cpu().numpy()
            self.cell_steps += member.cells * int(r.steps)
            self.used_bytes -= self._footprint(req)
            self.done.append(req)
            gone.append(b)
        return gone

    def _rebuild(self, keep: list[tuple[Request, Member]], joined: list[tuple[Request, Member]]) -> None:
        if self.engine is not None:
            self.engine.detach()
            self.engine = None
        self.active = keep + joined
        self.max_batch = max(self.max_batch, len(self.active))
        if self.active:
            self.engine = FloodEngine([m for _, m in self.active], self.cfg, self.precision, self.device,
                                      tile=self.tile, graph_steps=self.graph_steps)
            self.rebuilds += 1

    # ------------------------------------------------------------ serving loop
    def serve(self, requests: list[tuple[float, Storm]], max_wall_s: float | None = None) -> ServeStats:
        """Serve (arrival seconds, storm) requests in real time until all are finished
        (or max_wall_s passes) and return the statistics."""
        reqs = [Request(i, s, float(a)) for i, (a, s) in enumerate(sorted(requests, key=lambda x: x[0]))]
        t0 = time.perf_counter()
        nxt = 0
        reps = None
        while nxt < len(reqs) or self.queue or self.active:
            now = time.perf_counter() - t0
            if max_wall_s is not None and now > max_wall_s:
                break
            while nxt < len(reqs) and reqs[nxt].arrival <= now:
                self.queue.append(reqs[nxt])
                nxt += 1
            # retire the members the last chunk finished, then admit; one rebuild for both
            keep = self.active
            if reps is not None and any(r.status != 0 for r in reps):
                gone = set(self._retire(reps, now))
                keep = [am for b, am in enumerate(self.active) if b not in gone]
            reps = None
            joined = self._admit(now, len(keep))
            if joined or len(keep) != len(self.active):
                self._rebuild(list(keep), joined)
            if not self.active:
                if nxt < len(reqs):
                    time.sleep(max(0.0, min(reqs[nxt].arrival - (time.perf_counter() - t0), 0.05)))
                continue
            self.engine.advance(self.chunk_steps)
            reps = self.engine.reports()
        wall = time.perf_counter() - t0
        if self.engine is not None:
            reps = self.engine.reports()
            for b, (req, member) in enumerate(self.active):
                self.cell_steps += member.cells * int(reps[b].steps)
        return self.stats(len(reqs), wall)

    def stats(self, n_requests: int, wall: float) -> ServeStats:
        lat = np.array([r.latency for r in self.done]) if self.done else np.zeros(1)
        qs = np.array([r.admitted - r.arrival for r in self.done]) if self.done else np.zeros(1)
        statuses = {}
        for r in self.done:
            statuses[r.result.status] = statuses.get(r.result.status, 0) + 1
        return ServeStats(
            requests=n_requests, finished=len(self.done), wall_s=wall,
            storms_per_hour=3600.0 * len(self.done) / wall if wall > 0 else 0.0,
            cell_steps_per_s=self.cell_steps / wall if wall > 0 else 0.0,
            latency_p50_s=float(np.percentile(lat, 50)), latency_p99_s=float(np.percentile(lat, 99)),
            queue_p50_s=float(np.percentile(qs, 50)), queue_p99_s=float(np.percentile(qs, 99)),
            max_members=self.max_batch, rebuilds=self.rebuilds,
            max_mass_error=max((r.result.mass_error for r in self.done), default=0.0), statuses=statuses)


def shard_requests(requests: list, rank: int, world: int) -> list:
    """The requests one of `world` independent replicas serves (round robin by arrival
    order; the replicas share nothing, as the reference's process-per-GPU --shard i/n,
    cli.py:190-198)."""
    if not 0 <= rank < world:
        raise ValueError(f"rank {rank} outside a world of {world}")
    return list(requests[rank::world])


def request_stream(rate_per_s: float = 2.0, horizon_s: float = 600.0, key: str = "served"):
    """The served workload: Poisson arrivals of storms drawn from the three grid sizes,
    durations U(0.5, 6) h, built ahead of time (the request payloads)."""
    return [(t, uneven_member(f"{key}/{i}", size, dur))
            for i, (t, size, dur) in enumerate(served_requests(rate_per_s, horizon_s, key))]


def main():
    p = argparse.ArgumentParser(description="Serve a Poisson stream of storm requests on one GPU")
    p.add_argument("--minutes", type=float, default=10.0)
    p.add_argument("--rate", type=float, default=2.0)
    p.add_argument("--precision", default="fp32", choices=["fp32", "fp64"])
    p.add_argument("--chunk-steps", type=int, default=256)
    p.add_argument("--hbm-gb", type=float, default=None)
    p.add_argument("--tile", default="58x16")
    args = p.parse_args()
    reqs = request_stream(args.rate, 60.0 * args.minutes)
    tx, ty = (int(v) for v in args.tile.split("x"))
    srv = FloodServer(precision=args.precision, chunk_steps=args.chunk_steps, tile=(tx, ty),
                      hbm_budget=None if args.hbm_gb is None else int(args.hbm_gb * 2**30))
    st = srv.serve(reqs)
    print(json.dumps(st.__dict__))


if __name__ == "__main__":
    main()


__all__ = ["FloodServer", "Request", "ServeStats", "estimate_bytes", "request_stream", "shard_requests"]
