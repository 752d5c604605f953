"""The CUDA engine on the synthetic workloads: parity with the oracle at 1e-9, lake at
rest, mass balance, per-member time steps, batched == solo, float32 production form."""
import numpy as np
import pytest
import torch

import harness as H

pytestmark = pytest.mark.gpu


def _np(t):
    return t.detach().double().cpu().numpy()


def test_plain_small_1000_steps_match_oracle():
    """Plain float64 method, 100x81 @ 80 m coupled storm: after 1000 steps driven by the
    oracle's own CFL sequence, max |dh| <= 1e-9 m and max |d(hu, hv)| <= 1e-9 m^2/s."""
    from his_gb300 import workloads as W
    from his_gb300.assembly import build_engine
    storm = W.plain_small()
    eng = build_engine(storm)
    orc = H.oracle_from_storm(storm)
    t = 0.0
    for k in range(1000):
        dt = min(orc.two.max_dt(), storm.t_end - t)
        n_sub = max(1, int(np.ceil(dt / orc.one.max_dt() - 1e-9)))
        orc.step(t, storm.t_end, dt=dt, n_sub=n_sub)
        t = eng.step(t, storm.t_end, dt=dt, n_sub=n_sub)
    dh = H.max_abs(_np(eng.two.h), orc.two.h[0])
    dhu = H.max_abs(_np(eng.two.hu), orc.two.hu[0])
    dhv = H.max_abs(_np(eng.two.hv), orc.two.hv[0])
    dA = H.max_abs(_np(eng.one.A), orc.one.A[0])
    print(f"after 1000 steps (t = {t:.1f} s): |dh| {dh:.3e} m, |dhu| {dhu:.3e}, |dhv| {dhv:.3e}, |dA| {dA:.3e}")
    assert dh <= 1e-9 and dhu <= 1e-9 and dhv <= 1e-9
    assert dA <= 1e-8
    src = eng.mb.sources()
    for term, v in orc.acc.items():
        assert src[term] == pytest.approx(float(v[0]), rel=1e-9, abs=1e-6), term
    assert eng.mb.check(eng.total_volume(), t, record=False) < 1e-3


@pytest.mark.parametrize("dtype,tol", [(torch.float64, 1e-10), (torch.float32, 1e-5)])
def test_lake_at_rest_over_synthetic_dem(dtype, tol):
    """Still water over the full-resolution seeded DEM, partly dry, closed edges: after 500
    steps the spurious velocity stays below 1e-10 m/s (float64; 1e-5 for float32)."""
    from his_gb300 import workloads as W
    from his_gb300.boundaries import all_edges
    from his_gb300.config import SolverConfig
    from his_gb300.swe2d import SWE2D
    ter = W.make_terrain(400, 325, 20.0, 24, "plain_full", "triple")
    eta0 = float(np.quantile(ter.z, 0.6))
    sim = SWE2D(ter.z, 0.035, ter.dx, SolverConfig(), all_edges("closed"), dtype=dtype)
    sim.set_level(eta0)
    wet0 = _np(sim.h) > 0
    for _ in range(500):
        sim.step(sim.max_dt(), 0.0, 0.0)
    u, v = sim.velocities(sim.h, sim.hu, sim.hv)
    umax = max(float(u.abs().max()), float(v.abs().max()))
    deta = float(np.abs((_np(sim.h) + ter.z - eta0) * wet0).max())
    speed = np.hypot(_np(u), _np(v))
    j, i = np.unravel_index(np.argmax(speed), speed.shape)
    h = _np(sim.h)
    print(f"{dtype}: wet fraction {wet0.mean():.2f}, max |u|,|v| {umax:.3e} m/s at depth {h[j, i]:.4g} m "
          f"(cell {j},{i}), 99th pct speed {np.quantile(speed[wet0], 0.99):.3e}, "
          f"max |eta - eta0| {deta:.3e} m")
    assert umax < tol and deta < tol


def test_engine_matches_dropin_path_fp64():
    """The device-resident engine (dt, forcing and accounting on the GPU, graphs) takes the
    same steps as the drop-in path on the plain small storm."""
    from his_gb300 import workloads as W
    from his_gb300.assembly import build_engine
    from his_gb300.config import SolverConfig
    from his_gb300.engine import FloodEngine
    storm = W.plain_small()
    fe = FloodEngine([storm], SolverConfig(slot_width_frac=storm.slot_width_frac), precision="fp64",
                     graph_steps=8)
    eng = build_engine(storm)
    t = 0.0
    for _ in range(100):
        t = eng.step(t, storm.t_end)
    fe.advance(100)
    r = fe.reports()[0]
    assert r.steps == 100 and r.t == pytest.approx(t, rel=1e-12)
    assert H.max_abs(_np(fe.h[0]), _np(eng.two.h)) <= 1e-12
    assert H.max_abs(_np(fe.A[0]), _np(eng.one.A)) <= 1e-10
    src = eng.mb.sources()
    for j, term in enumerate(("rain", "infiltration", "bnd2d_in", "bnd2d_out", "bnd1d_in", "bnd1d_out", "clip")):
        assert r.acc[j] == pytest.approx(src[term], rel=1e-9, abs=1e-6), term


def test_batched_member_is_bit_identical_to_solo():
    """Per-member dt: a member advanced inside an uneven batch equals the same storm alone,
    bit for bit (float32 production form)."""
    from his_gb300 import workloads as W
    from his_gb300.engine import FloodEngine
    storms = [W.uneven_member(f"solo-vs-batch/{k}", k % 3, 1800.0 + 600.0 * k) for k in range(4)]
    # one decomposition for both (a tuned one could differ between the two batches and
    # change the summation order of the volume partials, not the state)
    batch = FloodEngine(storms, precision="fp32", tile=(58, 48))
    solo = FloodEngine([storms[2]], precision="fp32", tile=(58, 48))
    batch.advance(150)
    solo.advance(150)
    rb, rs = batch.reports()[2], solo.reports()[0]
    assert rb.steps == rs.steps == 150 and rb.t == rs.t
    assert torch.equal(batch.h[2], solo.h[0]) and torch.equal(batch.hu[2], solo.hu[0])
    assert torch.equal(batch.A[2], solo.A[0]) and torch.equal(batch.Q[2], solo.Q[0])
    assert list(rb.acc) == list(rs.acc)
    # members really take different steps
    dts = {round(r.dt_last, 9) for r in batch.reports()}
    assert len(dts) > 1


@pytest.mark.parametrize("precision", ["fp64", "fp32"])
def test_full_storm_mass_balance(precision):
    """The plain small storm run to its end through the engine: per-member mass error < 1e-3."""
    from his_gb300 import workloads as W
    from his_gb300.config import SolverConfig
    from his_gb300.engine import FloodEngine
    storm = W.plain_small()
    fe = FloodEngine([storm], SolverConfig(slot_width_frac=storm.slot_width_frac), precision=precision)
    reps = fe.run(chunk=512)
    assert reps[0].status == 1, f"member ended with status {reps[0].status}"
    errs = fe.assert_mass_ok()
    res = fe.results()[0]
    print(f"{precision}: {res.steps} steps, dt {res.dt_min:.3f}..{res.dt_max:.3f} s, mass error {errs[0]:.3e}, "
          f"sources {res.sources}")
    assert res.sources["rain"] > 0 and res.sources["bnd2d_out"] >= 0


def test_fp32_production_form_against_fp64():
    """Production form (float32 state and fluxes, float64 accumulators) against the plain
    float64 method on the same storm run to its end: peak-depth RMSE <= 1 cm, mass
    error < 1e-3, flood arrival (first 60-s output at 0.1 m) within one output interval
    in RMSE, and the volume error reported."""
    from his_gb300 import workloads as W
    from his_gb300.accuracy import compare
    from his_gb300.config import SolverConfig
    from his_gb300.engine import FloodEngine
    storm = W.plain_small()
    runs, floods = {}, {}
    for prec in ("fp64", "fp32"):
        fe = FloodEngine([storm], SolverConfig(slot_width_frac=storm.slot_width_frac), precision=prec,
                         track_peaks=True, output_interval=60.0)
        reps = fe.run(chunk=512)
        assert reps[0].status == 1
        fe.assert_mass_ok()
        runs[prec] = (fe, fe.results()[0])
        floods[prec] = fe.flood_results()[0]
    p64 = _np(runs["fp64"][0].peak_h[0])
    p32 = _np(runs["fp32"][0].peak_h[0])
    wet = (p64 > 1e-3) | (p32 > 1e-3)
    rmse = float(np.sqrt(np.mean((p32 - p64)[wet] ** 2)))
    dmax = float(np.abs(p32 - p64).max())
    r64, r32 = runs["fp64"][1], runs["fp32"][1]
    vol_err = abs(r32.volume - r64.volume) / max(r64.volume, 1.0)
    print(f"peak depth: RMSE {rmse * 1e3:.3f} mm, max {dmax * 1e3:.2f} mm over {int(wet.sum())} wet cells; "
          f"final volume rel. error {vol_err:.2e}; steps fp64 {r64.steps} fp32 {r32.steps}")
    assert rmse <= 0.01
    assert vol_err < 1e-3
    m = compare(floods["fp32"], floods["fp64"])
    print({k: v for k, v in m.items()})
    assert m["arrival_cells"] > 0
    assert m["arrival_rmse_s"] <= 60.0
    assert m["arrival_cells_in_one_run_only"] <= 0.01 * m["arrival_cells"] + 1
    assert m["peak_depth_rmse_m"] <= 0.01


@pytest.mark.parametrize("dtype,tol", [(torch.float64, 1e-9), (torch.float32, 1e-5)])
def test_batched_dropin_equals_members_run_alone(dtype, tol):
    """The batched drop-in engine (one shared CFL step, the reference's
    build_engine_batch) against each member built alone and driven through the
    batch's dt and substep sequence: the same states and mass terms per member."""
    from his_gb300 import workloads as W
    from his_gb300.assembly import build_engine, build_engine_batch
    storms = W.batched_uniform(3)
    eb = build_engine_batch(storms, dtype=dtype)
    singles = [build_engine(s, dtype=dtype) for s in storms]
    t_end = min(s.t_end for s in storms)
    t = 0.0
    for k in range(60):
        dt = min(eb.two.max_dt(), t_end - t)
        n_sub = max(1, int(np.ceil(dt / eb.one.max_dt() - 1e-9)))
        t_next = eb.step(t, t_end)
        assert eb._last_dt == dt, f"step {k}: the step chose another dt"
        for e in singles:
            e.step(t, t_end, dt=dt, n_sub=n_sub)
        t = t_next
    for b, e in enumerate(singles):
        for f in ("h", "hu", "hv"):
            d = H.max_abs(_np(getattr(eb.two, f)[b]), _np(getattr(e.two, f)))
            assert d <= tol, f"member {b}: {f} differs by {d}"
        assert H.max_abs(_np(eb.one.A[b]), _np(e.one.A)) <= 10 * tol
    sb = eb.mb.sources()
    for b, e in enumerate(singles):
        s1 = e.mb.sources()
        for term in s1:
            assert sb[term][b] == pytest.approx(s1[term], rel=1e-6, abs=1e-3), (b, term)


def test_member_chains_do_not_change_results():
    """Members split into 1, 3 or 4 independent chains (own streams and graphs, split
    at tile-balanced member boundaries of an uneven batch) step bit for bit alike."""
    from his_gb300 import workloads as W
    from his_gb300.config import SolverConfig
    from his_gb300.engine import FloodEngine
    storms = [W.uneven_member(f"chains/{k}", k % 3, 1800.0) for k in range(7)]
    states = {}
    for chains in (1, 3, 4):
        fe = FloodEngine(storms, SolverConfig(), precision="fp32", graph_steps=8, tile=(58, 32), chains=chains)
        assert fe.chains == chains
        fe.advance(37)                                  # graphs plus an uncaptured remainder
        reps = fe.reports()
        states[chains] = ([_np(h) for h in fe.h], [r.t for r in reps], [list(r.acc) for r in reps])
        fe.close()
    for chains in (3, 4):
        for a, b in zip(states[1][0], states[chains][0]):
            assert np.array_equal(a, b), f"{chains} chains: state differs"
        assert states[1][1] == states[chains][1] and states[1][2] == states[chains][2]


@pytest.mark.parametrize("order", [1, 2])
def test_grid_step_parts_match_members_alone(order):
    """A drop-in grid step large enough to run its stage launches as parts (48 members
    of 100 x 81 cells in 58 x 16 tiles: 576 tiles, 2 parts) equals each member
    stepped alone, bit for bit, at first order (stage copy per part) and second."""
    from his_gb300 import workloads as W
    from his_gb300.boundaries import all_edges
    from his_gb300.config import SolverConfig
    from his_gb300.swe2d import SWE2D
    ter = W.plain_small().terrain
    z = ter.z
    B = 48
    cfg = SolverConfig(spatial_order=order)
    rng = np.random.default_rng(5)
    n = rng.uniform(0.02, 0.06, B)[:, None, None] * np.ones((B,) + z.shape)
    eta = float(np.quantile(z, 0.3)) + rng.uniform(0.0, 2.0, B)
    h0 = np.maximum(eta[:, None, None] - z[None], 0.0)
    bcs = all_edges("transmissive")
    batched = SWE2D(z, n, ter.dx, cfg, bcs, batch=B, tile=(58, 16))
    batched.set_state(h0)
    dts, vols = [], []
    for k in range(12):
        dt = batched.max_dt()
        dts.append(dt)
        v = batched.step(dt, 60.0 * k, 2e-5)
        vols.append(np.stack([_np(getattr(v, f)) for f in ("bnd_in", "bnd_out", "rain", "infil", "clip")]))
    for b in range(0, B, 7):
        one = SWE2D(z, n[b], ter.dx, cfg, bcs, tile=(58, 16))
        one.set_state(h0[b])
        for k, dt in enumerate(dts):
            v = one.step(dt, 60.0 * k, 2e-5)
            got = np.array([float(getattr(v, f)) for f in ("bnd_in", "bnd_out", "rain", "infil", "clip")])
            assert np.array_equal(got, vols[k][:, b]), f"member {b}, step {k}: volumes"
        for f in ("h", "hu", "hv"):
            assert np.array_equal(_np(getattr(one, f)), _np(getattr(batched, f)[b])), f"member {b}: {f}"
