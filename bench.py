"""Benchmark of the GB300-native flood-engine step.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl reference]

Workload (one rank): the batched production form -- 64 storms on the seeded
400 x 325 @ 20 m terrain, float32 state and fluxes with float64 accumulators, each
member with its own CFL step, coupled 1-D network and weir exchange -- advanced by
the device-resident engine (CUDA graphs).  A "step" is one engine step of every
member.  Inputs (about 0.5 GB of state and fields touched per step) exceed the
129 MB L2, so no flush is needed between steps.

Printed (rank 0, one JSON line): cell-steps/s (whole job), storms/hour of the
batch and of the plain float64 single-storm engine at the same resolution, the
end-to-end rate through the drop-in C-ABI path with host buffers, the roofline of
the dominant kernel against the measured HBM peak, SM clocks sampled during the
timed region, the float32 form's error against float64 on the 100 x 81 storm (peak
depth, arrival time, volume), and the oracle's CPU float64 rate on this host as a
baseline.

--impl reference times the CPU restatement of the reference's float64 step (the
oracle, all host threads) on a bounded sample of the same workload.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time
from pathlib import Path

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

ALG_BYTES_F32 = 64      # per member-cell-step: 11 fields read + 5 written, float32
ALG_BYTES_F64 = 128
LAUNCHES_PER_STEP = 5   # pre, stage 1, stage 2, 1-D substeps, post: per member chain


def parse():
    p = argparse.ArgumentParser()
    p.add_argument("--gpus", type=int, default=1)
    p.add_argument("--steps", type=int, default=2000)
    p.add_argument("--warmup", type=int, default=30)
    p.add_argument("--impl", default="ours", choices=["ours", "reference"])
    p.add_argument("--members", type=int, default=64)
    p.add_argument("--storm-seconds", type=float, default=45.0, help="wall budget of the storms/hour legs")
    p.add_argument("--cpu-seconds", type=float, default=10.0)
    p.add_argument("--serve-seconds", type=float, default=60.0, help="arrival window of the serving leg")
    p.add_argument("--quick", action="store_true")
    p.add_argument("--tile", default="auto", help="strip width x chunk height of the 2-D kernels, or auto")
    p.add_argument("--chains", type=int, default=None, help="independent member chains of the engine (1..8)")
    return p.parse_args()


_REDUCE_DEVICE = "cuda"


def dist_init(backend: str | None = None):
    """One process per GPU (torchrun's RANK / LOCAL_RANK / WORLD_SIZE).  The ranks are
    independent replicas: the only communication is the barrier and the max-over-ranks
    of the timed region.  backend: "nccl" on GPUs (default), "gloo" for CPU tests."""
    global _REDUCE_DEVICE
    import torch
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    backend = backend or ("nccl" if torch.cuda.is_available() else "gloo")
    _REDUCE_DEVICE = "cuda" if backend == "nccl" else "cpu"
    if world > 1:
        import torch.distributed as dist
        if backend == "nccl":
            torch.cuda.set_device(local)
            dist.init_process_group("nccl", device_id=torch.device("cuda", local))
        else:
            dist.init_process_group("gloo")
    elif torch.cuda.is_available():
        torch.cuda.set_device(0)
    return world, rank, local


def barrier(world):
    if world > 1:
        import torch.distributed as dist
        dist.barrier()


def max_over_ranks(x: float, world: int) -> float:
    if world == 1:
        return x
    import torch
    import torch.distributed as dist
    t = torch.tensor([x], dtype=torch.float64, device=_REDUCE_DEVICE)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def rank_storms(members: int, rank: int):
    """The batch a rank advances: rank 0 the named workload, every other rank its own
    seeded storms of the same configuration (the ranks share no data)."""
    from his_gb300 import workloads as W
    return W.batched_uniform(members) if rank == 0 else W.batched_uniform(members, key=f"plain_full/rank{rank}")


def peaks():
    try:
        d = json.loads((ROOT / "MEASURED_PEAKS.json").read_text())
        return float(d["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


class ClockSampler:
    """SM clocks and throttle reasons sampled during the timed region.

    NVML (the driver's libnvidia-ml, read-only queries) is polled every 0.2 ms from a
    host thread (a read itself takes about 0.3 ms), so even a timed region of a few
    milliseconds gets a dozen or more samples; without NVML, nvidia-smi every 200 ms."""

    REASONS = {0x4: "sw_power_cap", 0x8: "hw_slowdown", 0x20: "sw_thermal_slowdown", 0x40: "hw_thermal_slowdown"}
    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index: int, period_s: float = 0.0002):
        self.gpu = gpu_index
        self.period = period_s
        self.samples = []            # (sm_mhz, reason bits)
        self.max_mhz = None
        self.source = None
        self._nvml = None
        self._stop = None
        self._thread = None
        self.proc = None
        self.path = None

    def _nvml_open(self):
        import ctypes as C
        try:
            lib = C.CDLL("libnvidia-ml.so.1")
        except OSError:
            return None
        if lib.nvmlInit_v2() != 0:
            return None
        h = C.c_void_p()
        if lib.nvmlDeviceGetHandleByIndex_v2(C.c_uint(self._nvml_index()), C.byref(h)) != 0:
            return None
        mx = C.c_uint()
        if lib.nvmlDeviceGetMaxClockInfo(h, C.c_int(1), C.byref(mx)) == 0:
            self.max_mhz = float(mx.value)
        reasons = getattr(lib, "nvmlDeviceGetCurrentClocksEventReasons", None) or \
            getattr(lib, "nvmlDeviceGetCurrentClocksThrottleReasons")
        return lib, h, reasons

    def _nvml_index(self) -> int:
        vis = os.environ.get("CUDA_VISIBLE_DEVICES", "")
        ids = [v.strip() for v in vis.split(",") if v.strip()]
        if ids and all(v.isdigit() for v in ids) and self.gpu < len(ids):
            return int(ids[self.gpu])
        return self.gpu

    def _poll(self):
        import ctypes as C
        lib, h, reasons = self._nvml
        mhz, bits = C.c_uint(), C.c_ulonglong()
        while not self._stop.is_set():
            if lib.nvmlDeviceGetClockInfo(h, C.c_int(1), C.byref(mhz)) == 0 and reasons(h, C.byref(bits)) == 0:
                self.samples.append((float(mhz.value), int(bits.value)))
            self._stop.wait(self.period)

    def __enter__(self):
        import threading
        try:
            self._nvml = self._nvml_open()
        except Exception:
            self._nvml = None
        if self._nvml is not None:
            self.source = f"nvml, {self.period * 1e3:g} ms"
            self._stop = threading.Event()
            self._thread = threading.Thread(target=self._poll, daemon=True)
            self._thread.start()
            return self
        fd, self.path = tempfile.mkstemp(suffix=".csv")
        os.close(fd)
        try:
            self.proc = subprocess.Popen(["nvidia-smi", f"--id={self.gpu}", f"--query-gpu={self.FIELDS}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=open(self.path, "w"), stderr=subprocess.DEVNULL)
            self.source = "nvidia-smi, 200 ms"
        except Exception:
            self.proc = None
        return self

    def __exit__(self, *exc):
        if self._thread is not None:
            self._stop.set()
            self._thread.join(timeout=5)
        if self.proc is not None:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()

    def summary(self):
        if self._nvml is not None:
            if not self.samples:
                return None
            sm = [m for m, _ in self.samples]
            reasons = sorted({n for _, b in self.samples for bit, n in self.REASONS.items() if b & bit})
            return {"sm_mhz": statistics.median(sm), "sm_max_mhz": self.max_mhz or max(sm), "samples": len(sm),
                    "reasons": reasons, "source": self.source}
        if not self.path or not Path(self.path).exists():
            return None
        rows = [r.split(",") for r in Path(self.path).read_text().strip().splitlines() if r.strip()]
        Path(self.path).unlink(missing_ok=True)
        sm, mx, reasons = [], [], set()
        names = ("hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap")
        for r in rows:
            r = [x.strip() for x in r]
            if len(r) < 9:
                continue
            try:
                sm.append(float(r[1]))
                mx.append(float(r[2]))
            except ValueError:
                continue
            for n, v in zip(names, r[5:9]):
                if v.lower() == "active":
                    reasons.add(n)
        if not sm:
            return None
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(mx), "samples": len(sm),
                "reasons": sorted(reasons), "source": self.source}


TRAFFIC_PROFILE = "profiles/strip_kernel_f32_batched_uniform.md"


def read_traffic():
    """Per-cell DRAM traffic of the dominant kernel, as measured by the ncu capture that
    the committed summary records (not by this run: counters are not read live)."""
    p = ROOT / TRAFFIC_PROFILE
    if not p.exists():
        return None
    for line in p.read_text().splitlines():
        if line.strip().startswith("traffic_bytes_per_cell:"):
            try:
                return float(line.split(":", 1)[1].split()[0])
            except ValueError:
                return None
    return None


def storm_rate(engine, budget_s: float):
    """Advance until every member is done or the wall budget is spent; storms/hour from the
    simulated-time progress (exact when the batch completes)."""
    import torch
    t_end = [s.t_end for s in engine.storms]
    r0 = engine.reports()
    t_start = [r.t for r in r0]
    torch.cuda.synchronize()
    w0 = time.perf_counter()
    done = False
    while time.perf_counter() - w0 < budget_s:
        engine.advance(256)
        reps = engine.reports()
        if all(r.status != 0 for r in reps):
            done = True
            break
    wall = time.perf_counter() - w0
    reps = engine.reports()
    frac = sum((r.t - t0) / te for r, t0, te in zip(reps, t_start, t_end))
    return {"storms_per_hour": 3600.0 * frac / wall, "wall_s": wall, "completed": done,
            "status": sorted({int(r.status) for r in reps}), "steps": [int(r.steps) for r in reps]}


def cpu_oracle_rate(storm, seconds: float, threads: int):
    """The oracle (C, OpenMP) float64 coupled step on one member, on this host's cores."""
    sys.path.insert(0, str(ROOT / "tests"))
    sys.path.insert(0, str(ROOT / "tests" / "golden"))
    from oracle import oracle as O
    import harness as H
    O.set_threads(threads)
    orc = H.oracle_from_storm(storm)
    t, steps = 0.0, 0
    orc.step(t, storm.t_end)                 # warm-up step (builds the library, pages memory in)
    w0 = time.perf_counter()
    while time.perf_counter() - w0 < seconds and steps < 10000:
        t = orc.step(t, storm.t_end)
        steps += 1
    wall = time.perf_counter() - w0
    return {"value": storm.cells * steps / wall, "steps": steps, "wall_s": wall}


def uneven_leg(budget_s: float):
    """48 storms of three grid sizes and their own durations in one engine (one launch per
    stage over every member's strips, per-member dt, tuned decomposition), run to the end."""
    import numpy as np
    from his_gb300 import workloads as W
    from his_gb300.config import SolverConfig
    from his_gb300.engine import FloodEngine
    storms = W.batched_uneven(16)
    eng = FloodEngine(storms, SolverConfig(), precision="fp32", graph_steps=16)
    sr = storm_rate(eng, budget_s)
    cell_steps = sum(s.cells * st for s, st in zip(storms, sr["steps"]))
    out = {"workload": "batched uneven: 16 x 100x81 @ 80 m + 16 x 200x163 @ 40 m + 16 x 400x325 @ 20 m, "
                       "durations U(1, 6) h, coupled, per-member dt", "members": len(storms),
           "tile": list(eng.tile), "storms_per_hour": sr["storms_per_hour"], "completed": sr["completed"],
           "wall_s": sr["wall_s"], "cell_steps_per_s": cell_steps / sr["wall_s"],
           "steps_min_max": [int(np.min(sr["steps"])), int(np.max(sr["steps"]))]}
    if sr["completed"]:
        out["mass_error_max"] = max(r.mass_error for r in eng.results())
    return out


def serving_leg(window_s: float):
    """Poisson arrivals (2 requests/s over the window) of storms drawn from the three grid
    sizes with durations U(0.5, 6) h, served in real time by the continuous-batching loop;
    latency is arrival to result."""
    from his_gb300.serving import FloodServer, request_stream
    reqs = request_stream(2.0, window_s)
    srv = FloodServer(precision="fp32", chunk_steps=256, tile=(58, 16))
    st = srv.serve(reqs, max_wall_s=window_s + 240.0)
    d = dict(st.__dict__)
    d["workload"] = (f"served: Poisson 2 req/s over {window_s:.0f} s, grids 100x81 @ 80 m / 200x163 @ 40 m / "
                     "400x325 @ 20 m, durations U(0.5, 6) h, fp32, admission by HBM footprint")
    return d


def accuracy_leg(interval_s: float = 60.0) -> dict:
    """Error of the float32 production form against the plain float64 method on the
    100x81 @ 80 m storm run to its end: peak depth, arrival time (first output at
    0.1 m, outputs every interval_s) and volume (his_gb300.accuracy.compare)."""
    from his_gb300 import workloads as W
    from his_gb300.accuracy import compare
    from his_gb300.config import SolverConfig
    from his_gb300.engine import FloodEngine
    storm = W.plain_small()
    res = {}
    for prec in ("fp64", "fp32"):
        fe = FloodEngine([storm], SolverConfig(slot_width_frac=storm.slot_width_frac), precision=prec,
                         track_peaks=True, output_interval=interval_s)
        fe.run(chunk=512)
        res[prec] = fe.flood_results()[0]
        fe.close()
    m = compare(res["fp32"], res["fp64"])
    m["mass_error_fp32"] = float(res["fp32"].mass_balance_error)
    m["workload"] = "100x81 @ 80 m coupled storm to its end, float32 production form against float64"
    return m


def accuracy_c3_leg(members: int = 2, interval_s: float = 120.0) -> dict:
    """Error of the float32 production form against the float64 method at full
    resolution: the first ``members`` storms of the 64-storm batch (400 x 325 @ 20 m)
    run to their end in both precisions (his_gb300.accuracy.against_fp64): peak depth
    (max and RMSE over wet cells), arrival time at 0.1 m from the outputs, volume and
    both runs' mass-balance errors."""
    from his_gb300 import workloads as W
    from his_gb300.accuracy import against_fp64, reference_criteria
    w0 = time.perf_counter()
    rows = against_fp64(W.batched_uniform(members), interval_s)
    keep = ("member", "status_fp32", "status_fp64", "steps_fp32", "steps_fp64", "peak_depth_rmse_m",
            "peak_depth_max_m", "peak_every_step_rmse_m", "wet_cells", "arrival_rmse_s", "arrival_max_s",
            "arrival_cells", "arrival_cells_in_one_run_only", "final_volume_rel", "final_surface_volume_rel",
            "depth_rmse_wet_m", "depth_p99_abs_m", "depth_max_abs_m", "flooded_area_rel",
            "reach_peak_discharge_rel", "mass_error_fp32", "mass_error_fp64")
    crit = [reference_criteria(r) for r in rows]
    return {"workload": f"{members} members of the 64-storm batch, 400x325 @ 20 m, 8.5 h storms to their end, "
                        f"float32 production form against float64, outputs every {interval_s:.0f} s",
            "peak_depth_rmse_m_max": max(r["peak_depth_rmse_m"] for r in rows),
            "arrival_rmse_s_max": max(r["arrival_rmse_s"] for r in rows),
            "mass_error_fp32_max": max(r["mass_error_fp32"] for r in rows),
            "reach_peak_discharge_rel_max": max(r.get("reach_peak_discharge_rel", 0.0) for r in rows),
            "reference_fp32_criteria": {k: {"worst": max(c[k]["value"] for c in crit), "limit": crit[0][k]["limit"],
                                            "pass_all": all(c[k]["pass"] for c in crit)} for k in crit[0]},
            "members": [{k: r[k] for k in keep if k in r} for r in rows],
            "wall_s": time.perf_counter() - w0}


def e2e_dropin(storms, steps: int):
    """Same metric through the drop-in public API (batched CoupledEngine -> C ABI, host
    buffers): every step uploads its step parameters and 1-D forcing from host memory
    (staged through pinned slots) and reads back both models' CFL rates, the one wait
    of the step; the mass terms stay on the device, as the reference keeps them."""
    import numpy as np
    import torch
    from his_gb300.assembly import build_engine_batch
    eng = build_engine_batch(storms, dtype=torch.float32)
    B = len(storms)
    t = 0.0
    t_end = storms[0].t_end
    for _ in range(2):
        t = eng.step(t, t_end)
    torch.cuda.synchronize()
    w0 = time.perf_counter()
    for _ in range(steps):
        t = eng.step(t, t_end)
    torch.cuda.synchronize()
    wall = time.perf_counter() - w0
    n_sub = eng.log.n_sub_max
    # bytes moved per step by the drop-in calls (params in, results out)
    h2d = B * 88 + B * 2 * 8 * n_sub        # 2-D step params, 1-D substep forcing
    d2h = B * 8 + B * 16                    # 2-D rate, 1-D (rate, wet) per member
    cells = sum(s.cells for s in storms)
    return {"value": cells * steps / wall, "unit": "cell-steps/s", "h2d_bytes_per_step": int(h2d),
            "d2h_bytes_per_step": int(d2h), "steps": steps, "shared_dt": True}


def workload_config(members: int) -> dict:
    """The workload both arms report: the batched production form on the seeded terrain."""
    return {"workload": f"batched uniform: {members} storms x 400x325 @ 20 m, coupled 1-D/2-D, per-member dt",
            "members": members, "cells_per_step": members * 400 * 325, "grid": "400x325", "dx_m": 20.0,
            "precision": "fp32 2-D state and fluxes, fp32 1-D fluxes over fp64 1-D state, fp64 accumulators", "graph_steps": 16,
            "l2": "inputs larger than L2 (~0.5 GB touched per step), no flush"}


def run_ours(args, world, rank, local):
    import numpy as np
    import torch
    from his_gb300 import workloads as W
    from his_gb300.config import SolverConfig
    from his_gb300.engine import FloodEngine
    members = args.members
    storms = rank_storms(members, rank)
    cells = sum(s.cells for s in storms)
    tile = "auto" if args.tile == "auto" else tuple(int(v) for v in args.tile.split("x"))
    eng = FloodEngine(storms, SolverConfig(), precision="fp32", graph_steps=16, tile=tile, chains=args.chains)
    # graphs are captured before the steps they run: the warm-up's, then the timed
    # region's (a whole number of 16-step graphs plus one remainder graph per chain)
    eng.prepare(args.warmup)
    eng.advance(args.warmup)
    eng.prepare(args.steps)
    torch.cuda.synchronize()
    s = torch.cuda.current_stream()
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    with ClockSampler(local) as clk:
        barrier(world)
        torch.cuda.synchronize()
        ev0.record(s)
        eng.advance(args.steps)
        ev1.record(s)
        torch.cuda.synchronize()
        barrier(world)
    ms = max_over_ranks(ev0.elapsed_time(ev1), world)
    clocks = clk.summary()
    reps = eng.reports()
    assert all(r.status == 0 for r in reps), "a member finished or failed inside the timed region"
    value = world * cells * args.steps / (ms / 1e3)
    # per-kernel device times (events on the launching streams)
    prof_steps = min(args.steps, 50)
    kms = np.zeros(6)
    import ctypes as C
    from his_gb300 import _lib
    _lib.check(eng._lib.his_engine_profile(eng._engine, prof_steps, _lib.as_p(kms), _lib.stream_handle()),
               "his_engine_profile")
    hbm, peak_kind = peaks()
    stage2_s = kms[2] / prof_steps / 1e3
    achieved = ALG_BYTES_F32 * cells / stage2_s / 1e9
    step_s = ms / args.steps / 1e3          # the timed step, all chains side by side
    traffic = read_traffic()
    out = {"metric": "cell-steps/s", "value": value, "unit": "cell-steps/s", "n_gpus": world, "steps": args.steps,
           "warmup": args.warmup, "ms_per_step": ms / args.steps, "higher_is_better": True, "scaling": "weak",
           "vs_baseline": None, "dtype": "f32 (f64 accumulators, 1-D channel state and junction depths)",
           "data": "synthetic (seeded terrain, forcing and networks)",
           "config": workload_config(members),
           "gpu_launches": LAUNCHES_PER_STEP * eng.chains * args.steps, "tile": list(eng.tile), "chains": eng.chains,
           "roofline": {"bound": "hbm", "achieved": achieved, "peak": hbm, "unit": "GB/s",
                        "frac": achieved / hbm, "peak_kind": peak_kind,
                        "traffic": traffic * cells if traffic is not None else None,
                        "traffic_source": f"ncu capture of this kernel on this workload ({TRAFFIC_PROFILE}), "
                                          "not this run",
                        "kernel": "strip_kernel<float,64,2> (RK stage 2 + sources + friction + CFL)",
                        "alg_bytes_per_cell": ALG_BYTES_F32,
                        "step_achieved": ALG_BYTES_F32 * cells / step_s / 1e9,
                        "step_frac": ALG_BYTES_F32 * cells / step_s / 1e9 / hbm,
                        "ms_per_step_by_kernel": {"pre": kms[0] / prof_steps, "stage1": kms[1] / prof_steps,
                                                  "stage2": kms[2] / prof_steps, "net1d": kms[3] / prof_steps,
                                                  "post": kms[4] / prof_steps, "step": kms[5] / prof_steps},
                        "profile_note": "per-kernel times from one serial chain (CUDA events per kernel class); "
                                        "the timed step runs the member chains side by side"},
           "clocks": clocks}
    if rank == 0 and not args.quick:
        sr = storm_rate(eng, args.storm_seconds)
        out["storms_per_hour"] = sr["storms_per_hour"]
        out["storms_detail"] = {k: v for k, v in sr.items() if k != "steps"} | {
            "mean_steps": float(np.mean(sr["steps"]))}
        if sr["completed"]:
            errs = [r.mass_error for r in eng.results()]
            out["mass_error_max"] = max(errs)
        del eng
        torch.cuda.empty_cache()
        plain = W.plain_full()
        pe = FloodEngine([plain], SolverConfig(), precision="fp64", graph_steps=16)
        pr = storm_rate(pe, args.storm_seconds)
        out["plain_fp64_single"] = {"storms_per_hour": pr["storms_per_hour"], "completed": pr["completed"],
                                    "wall_s": pr["wall_s"], "steps": pr["steps"][0],
                                    "cell_steps_per_s": plain.cells * pr["steps"][0] / pr["wall_s"]}
        out["speedup_vs_plain_fp64_single"] = out["storms_per_hour"] / pr["storms_per_hour"]
        del pe
        torch.cuda.empty_cache()
        out["uneven_batch"] = uneven_leg(args.storm_seconds)
        torch.cuda.empty_cache()
        out["accuracy_c1"] = accuracy_leg()
        torch.cuda.empty_cache()
        out["accuracy_c3"] = accuracy_c3_leg()
        torch.cuda.empty_cache()
        if args.serve_seconds > 0:
            out["serving"] = serving_leg(args.serve_seconds)
            torch.cuda.empty_cache()
        out["e2e"] = e2e_dropin(storms[: min(members, 64)], steps=200)
        threads = os.cpu_count() or 1
        cpu = cpu_oracle_rate(storms[0], args.cpu_seconds, threads)
        out["cpu_baseline"] = {"value": cpu["value"], "unit": "cell-steps/s", "cores": threads, "kind": "port",
                               "sample": f"{cpu['steps']} coupled float64 steps of one 400x325 member "
                                         f"({cpu['wall_s']:.1f} s)"}
    else:
        out["e2e"] = None
    return out


def run_reference(args, world, rank):
    if rank != 0:
        return None
    from his_gb300 import workloads as W
    sys.path.insert(0, str(ROOT / "tests"))
    sys.path.insert(0, str(ROOT / "tests" / "golden"))
    from oracle import oracle as O
    import harness as H
    threads = os.cpu_count() or 1
    O.set_threads(threads)
    storm = W.batched_uniform(1)[0]
    orc = H.oracle_from_storm(storm)
    t = 0.0
    for _ in range(max(1, min(args.warmup, 3))):
        t = orc.step(t, storm.t_end)
    # a bounded sample: up to --steps steps of one member, at most about 20 s of host time
    steps = 0
    w0 = time.perf_counter()
    while steps < max(1, args.steps) and (steps == 0 or time.perf_counter() - w0 < 20.0):
        t = orc.step(t, storm.t_end)
        steps += 1
    wall = time.perf_counter() - w0
    value = storm.cells * steps / wall
    return {"impl": "reference", "metric": "cell-steps/s", "value": value, "unit": "cell-steps/s", "n_gpus": world,
            "steps": steps, "warmup": args.warmup, "ms_per_step": wall * 1e3 / steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded terrain, forcing "
            "and networks)", "config": workload_config(args.members) | {
                "sampled": "member 0 of the batch, one member-step per step (the rate is per member-cell-step)",
                "precision": "fp64 throughout (the reference's method on the host)"},
            "cpu_baseline": {"value": value, "unit": "cell-steps/s", "cores": threads, "kind": "port",
                             "sample": f"{steps} coupled float64 steps of member 0 of the batch (400x325), "
                                       "the oracle restatement of the reference's step on all host threads"},
            "e2e": {"value": value, "unit": "cell-steps/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
            "gpu_launches": 0}


def main():
    args = parse()
    if args.warmup < 3:
        args.warmup = 3
    if args.impl == "reference":
        world = int(os.environ.get("WORLD_SIZE", "1"))
        rank = int(os.environ.get("RANK", "0"))
        out = run_reference(args, world, rank)
        if out is not None:
            print(json.dumps(out))
        return
    world, rank, local = dist_init()
    out = run_ours(args, world, rank, local)
    if rank == 0:
        print(json.dumps(out))
    if world > 1:
        import torch.distributed as dist
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
