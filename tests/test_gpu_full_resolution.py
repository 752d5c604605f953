"""The full-resolution configurations on the CUDA path: the plain float64 method on the
400 x 325 @ 20 m storm (three reaches meeting at a level-pool junction, ~1,500 bank
links, Horton infiltration, a 5 mm retention store, the M2 tide on both models and the
inflow hydrograph) against the oracle over 1000 steps, and the float32 production form
against the float64 method on members of the 64-storm batch run to their end."""
import numpy as np
import pytest

import harness as H

pytestmark = pytest.mark.gpu


def _np(t):
    return t.detach().double().cpu().numpy()


def test_plain_full_1000_steps_match_oracle():
    """400 x 325 @ 20 m, float64, B = 1, driven by the oracle's own CFL sequence (dt and
    1-D substep count per step): after 1000 steps max |dh| <= 1e-9 m, max |d(hu, hv)|
    <= 1e-9 m^2/s, max |dA| <= 1e-8 m^2, every accumulated volume term within 1e-9
    relative, and the mass-balance error < 1e-3.  The run exercises the junction, the
    weir links in both directions, infiltration, the retention store and both models'
    boundaries (checked on the oracle's tallies)."""
    from his_gb300 import workloads as W
    from his_gb300.assembly import build_engine
    storm = W.plain_full()
    assert storm.network is not None and len(storm.network.junctions) >= 1
    eng = build_engine(storm)
    orc = H.oracle_from_storm(storm)
    t = 0.0
    for _ in range(1000):
        dt = min(orc.two.max_dt(), storm.t_end - t)
        n_sub = max(1, int(np.ceil(dt / orc.one.max_dt() - 1e-9)))
        orc.step(t, storm.t_end, dt=dt, n_sub=n_sub)
        t = eng.step(t, storm.t_end, dt=dt, n_sub=n_sub)
    d = {f: H.max_abs(_np(getattr(eng.two, f)), getattr(orc.two, f)[0]) for f in ("h", "hu", "hv", "s_filled",
                                                                                    "infil_cum")}
    dA = H.max_abs(_np(eng.one.A), orc.one.A[0])
    dQ = H.max_abs(_np(eng.one.Q), orc.one.Q[0])
    src = eng.mb.sources()
    print(f"after 1000 steps (t = {t:.1f} s): " + ", ".join(f"|d{k}| {v:.3e}" for k, v in d.items()) +
          f", |dA| {dA:.3e}, |dQ| {dQ:.3e}; exchanged 2-D->1-D {orc.exch[0, 0]:.1f} m^3, 1-D->2-D "
          f"{orc.exch[0, 1]:.1f} m^3 over {int(orc.links_active.sum())}/{orc.links.n_links} links; sources {src}")
    assert d["h"] <= 1e-9 and d["hu"] <= 1e-9 and d["hv"] <= 1e-9
    assert d["s_filled"] <= 1e-12 and d["infil_cum"] <= 1e-12
    assert dA <= 1e-8 and dQ <= 1e-8
    for term, v in orc.acc.items():
        assert src[term] == pytest.approx(float(v[0]), rel=1e-9, abs=1e-6), term
    assert eng.mb.check(eng.total_volume(), t, record=False) < 1e-3
    # what the first 1000 steps exercise (the weir links start later: see the next test)
    assert src["infiltration"] > 0 and src["rain"] > 0 and src["bnd2d_in"] > 0 and src["bnd1d_out"] > 0
    assert float(orc.two.s_filled.max()) > 0, "retention store filled"


def test_plain_full_mid_storm_1000_steps_match_oracle():
    """The same storm from t = 5400 s (1.5 h, rising limb: the channel overtops into the
    floodplain and the floodplain drains back over other banks): the CUDA float64 engine
    runs there on its own CFL steps, the oracle takes over its state, and both then take
    1000 steps on the oracle's dt and substep sequence.  Same bounds as from t = 0, on
    the states and on the volume terms accumulated over the 1000 steps; the weir links
    move water in both directions."""
    from his_gb300 import workloads as W
    from his_gb300.assembly import build_engine
    from his_gb300.massbalance import TERMS
    storm = W.plain_full()
    eng = build_engine(storm)
    t = 0.0
    while t < 5400.0:
        t = eng.step(t, storm.t_end)
    orc = H.oracle_from_storm(storm)
    for f in ("h", "hu", "hv", "s_filled", "infil_cum"):
        getattr(orc.two, f)[0][...] = _np(getattr(eng.two, f))
    orc.one.A[0][...] = _np(eng.one.A)
    orc.one.Q[0][...] = _np(eng.one.Q)
    src0 = eng.mb.sources()
    t0 = t
    for _ in range(1000):
        dt = min(orc.two.max_dt(), storm.t_end - t)
        n_sub = max(1, int(np.ceil(dt / orc.one.max_dt() - 1e-9)))
        orc.step(t, storm.t_end, dt=dt, n_sub=n_sub)
        t = eng.step(t, storm.t_end, dt=dt, n_sub=n_sub)
    d = {f: H.max_abs(_np(getattr(eng.two, f)), getattr(orc.two, f)[0]) for f in ("h", "hu", "hv")}
    dA = H.max_abs(_np(eng.one.A), orc.one.A[0])
    dQ = H.max_abs(_np(eng.one.Q), orc.one.Q[0])
    src = eng.mb.sources()
    inc = {k: src[k] - src0[k] for k in TERMS}
    print(f"t {t0:.1f} -> {t:.1f} s: " + ", ".join(f"|d{k}| {v:.3e}" for k, v in d.items()) +
          f", |dA| {dA:.3e}, |dQ| {dQ:.3e}; exchanged 2-D->1-D {orc.exch[0, 0]:.1f} m^3, 1-D->2-D "
          f"{orc.exch[0, 1]:.1f} m^3 over {int(orc.links_active.sum())}/{orc.links.n_links} links; "
          f"terms over the segment {inc}")
    assert d["h"] <= 1e-9 and d["hu"] <= 1e-9 and d["hv"] <= 1e-9
    assert dA <= 1e-8 and dQ <= 1e-8
    for term, v in orc.acc.items():
        assert inc[term] == pytest.approx(float(v[0]), rel=1e-9, abs=1e-6), term
    assert orc.exch[0, 0] > 0 and orc.exch[0, 1] > 0, "weir exchange in both directions"
    assert eng.mb.check(eng.total_volume(), t, record=False) < 1e-3


def test_fp32_against_fp64_full_resolution_members():
    """Four members of the 64-storm batch (400 x 325 @ 20 m, own roughness, retention,
    infiltration, conveyance, rain, tide and inflow) run to their end in the float32
    production form and in the float64 method, outputs every 120 s: per member
    peak-depth RMSE <= 1 cm, mass-balance error < 1e-3 in both runs, flood arrival
    (first output at 0.1 m) within one output interval in RMSE, final volume within
    1e-3 relative."""
    from his_gb300 import workloads as W
    from his_gb300.accuracy import against_fp64, reference_criteria
    storms = W.batched_uniform(4)
    rows = against_fp64(storms, 120.0)
    for m in rows:
        print({k: (round(v, 9) if isinstance(v, float) else v) for k, v in m.items()})
        print("  reference fp32 criteria:", {k: (f"{v['value']:.3g}", v["pass"]) for k, v in
                                              reference_criteria(m).items()})
    for m in rows:
        assert m["status_fp32"] == "done" and m["status_fp64"] == "done", m["member"]
        assert m["peak_depth_rmse_m"] <= 0.01, m["member"]
        assert m["mass_error_fp32"] < 1e-3 and m["mass_error_fp64"] < 1e-3, m["member"]
        assert m["arrival_cells"] > 0 and m["arrival_rmse_s"] <= 120.0, m["member"]
        assert m["arrival_cells_in_one_run_only"] <= 0.01 * m["arrival_cells"] + 1, m["member"]
        assert m["final_volume_rel"] < 1e-3, m["member"]
        # the channel network runs in float32 too: its peak discharge per reach within
        # the reference's 2 % agreement bar (criteria.py:45)
        assert m["reach_peak_discharge_rel"] <= 0.02, m["member"]
