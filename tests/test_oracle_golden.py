"""Pin the oracle: the C restatement against vectors produced by the reference solver itself.

Every case replays the reference's own time-step sequence.  States are compared
at the recorded snapshots; per-step volumes at every step.  The reference runs in
torch (vectorised pow/exp and pairwise sums), the oracle in libm with sequential
sums, so the bound is a few ulp of the state scale, not bit equality.
"""
import numpy as np
import pytest

import golden_cases as GC
import harness as H

STATE_TOL = 1e-12      # absolute, on states of order 1 (m, m^2/s)
VOL_REL = 1e-11        # relative, per-step volumes


@pytest.mark.parametrize("name", list(GC.SWE2D_CASES))
def test_swe2d_matches_reference(name):
    sim, spec, fx = H.oracle_swe2d(name)
    for k in range(spec["steps"]):
        dt, t = float(fx["dt"][k]), float(fx["t"][k])
        rate = sim.max_rate()
        assert rate == pytest.approx(float(fx["rate"][k]), rel=1e-13, abs=1e-300), f"step {k}: CFL rate"
        vol = sim.step(dt, t, GC.rain_value(spec, t))
        for key in ("bnd_in", "bnd_out", "rain", "infil", "clip"):
            want = fx[key][k]
            scale = max(float(np.max(np.abs(want))), 1e-9)
            assert H.max_abs(vol[key], want) <= VOL_REL * scale + 1e-13, f"step {k}: volume {key}"
        if k + 1 in spec["snap_at"]:
            for f in ("h", "hu", "hv", "s_filled", "infil_cum"):
                got = getattr(sim, f).reshape(fx[f"{f}_{k + 1}"].shape)
                assert H.max_abs(got, fx[f"{f}_{k + 1}"]) <= STATE_TOL, f"step {k + 1}: {f}"


@pytest.mark.parametrize("name", list(GC.SWE1D_CASES))
def test_swe1d_matches_reference(name):
    one, spec, fx = H.oracle_swe1d(name)
    for k in range(spec["steps"]):
        dt, t = float(fx["dt"][k]), float(fx["t"][k])
        assert one.max_dt() == pytest.approx(float(fx["max_dt"][k]), rel=1e-13), f"step {k}: 1-D dt"
        v = one.step(dt, t)
        for key in ("bnd_in", "bnd_out", "clip"):
            want = fx[key][k]
            assert H.max_abs(v[key], want) <= VOL_REL * max(float(np.max(np.abs(want))), 1.0), f"step {k}: {key}"
        if k + 1 in spec["snap_at"]:
            assert H.max_abs(one.A.reshape(fx[f"A_{k + 1}"].shape), fx[f"A_{k + 1}"]) <= STATE_TOL * 10
            assert H.max_abs(one.Q.reshape(fx[f"Q_{k + 1}"].shape), fx[f"Q_{k + 1}"]) <= STATE_TOL * 10


def test_sections_match_reference():
    from his_gb300 import topology as T
    from his_gb300.channels import apply_gamma
    import his_gb300.channels as CH
    for name, spec in GC.SWE1D_CASES.items():
        fx = H.load(name)
        net = GC.network(spec, CH)
        nets = [apply_gamma(net, np.asarray(g)) for g in spec["gammas"]] if spec.get("batch") else [net]
        topos = [T.build_topology(n) for n in nets]
        tp = topos[0]
        for k in ("kind", "reach_of", "ghost_src", "ghost_sign", "face_l", "face_r", "m", "zbank", "n", "dx", "x",
                  "y", "chain"):
            assert np.array_equal(np.asarray(getattr(tp, k)), fx[f"topo_{k}"]), f"{name}: topology field {k}"
        z = np.stack([t.z for t in topos]).reshape(fx["z_members"].shape)
        b = np.stack([t.b for t in topos]).reshape(fx["sec_b"].shape)
        assert np.array_equal(z, fx["z_members"])
        sec = T.sections(tp, spec["slot_width_frac"], z, b)
        for k in ("b", "m", "yb", "ts"):
            assert np.array_equal(sec[k], np.broadcast_to(fx[f"sec_{k}"], sec[k].shape)), f"{name}: sec {k}"
        for k, fk in (("fb", "b"), ("fm", "m"), ("fyb", "yb"), ("fts", "ts")):
            assert np.array_equal(sec[k], np.broadcast_to(fx[f"fsec_{fk}"], sec[k].shape)), f"{name}: face sec {k}"


def test_exchange_matches_reference():
    from oracle.oracle import exchange
    fx = H.load("exchange_overtop")
    spec = GC.EXCHANGE_CASES["exchange_overtop"]
    one, two, links, _ = H.oracle_overtop(fx)
    for i in range(spec["calls"]):
        two.set_state(fx[f"h_in_{i}"], fx[f"hu_in_{i}"], fx[f"hv_in_{i}"])
        one.A = np.ascontiguousarray(fx[f"A_in_{i}"].reshape(one.A.shape))
        V = exchange(one, two, links, spec["dt"])
        assert H.max_abs(V.reshape(-1), fx[f"V_{i}"]) <= 1e-12 * max(1.0, float(np.abs(fx[f"V_{i}"]).max()))
        for f in ("h", "hu", "hv"):
            assert H.max_abs(getattr(two, f).reshape(fx[f"{f}_out_{i}"].shape), fx[f"{f}_out_{i}"]) <= 1e-13
        assert H.max_abs(one.A.reshape(-1), fx[f"A_out_{i}"]) <= 1e-12


def test_coupled_matches_reference():
    from oracle.oracle import OracleCoupled
    fx_x = H.load("exchange_overtop")
    fx = H.load("coupled_overtop")
    spec = GC.COUPLED_CASES["coupled_overtop"]
    one, two, links, _ = H.oracle_overtop(fx_x)
    two.set_state(fx["h0"])
    one.A = np.ascontiguousarray(fx["A0"].reshape(one.A.shape))
    one.Q = np.ascontiguousarray(fx["Q0"].reshape(one.Q.shape))
    eng = OracleCoupled(two, one, links, two.cfg, rain=GC.rain_fn_coupled(spec))
    t = 0.0
    for k in range(spec["steps"]):
        # the oracle's own CFL choices must reproduce the reference's sequence
        dt = min(two.max_dt(), spec["t_end"] - t)
        assert dt == pytest.approx(float(fx["dt"][k]), rel=1e-12), f"step {k}: dt"
        t = eng.step(t, spec["t_end"], dt=float(fx["dt"][k]), n_sub=int(fx["n_sub"][k]))
        if k + 1 in spec["snap_at"]:
            for f in ("h", "hu", "hv"):
                assert H.max_abs(getattr(two, f).reshape(fx[f"{f}_{k + 1}"].shape), fx[f"{f}_{k + 1}"]) <= 1e-11
            assert H.max_abs(one.A.reshape(-1), fx[f"A_{k + 1}"]) <= 1e-10
            assert H.max_abs(one.Q.reshape(-1), fx[f"Q_{k + 1}"]) <= 1e-10
    for term in GC_TERMS:
        want = float(fx[f"src_{term}"])
        assert float(eng.acc[term][0]) == pytest.approx(want, rel=1e-10, abs=1e-9), term
    assert float(eng.mass_error()[0]) < 1e-12


GC_TERMS = ("rain", "infiltration", "bnd2d_in", "bnd2d_out", "bnd1d_in", "bnd1d_out", "clip")


def test_batched_coupled_members_match_reference():
    """Each member of the reference's batched coupled run (shared dt; per-member
    roughness, channel conveyance, states, inflow and rain), replayed by the oracle
    member by member through the reference's dt and substep sequence."""
    import his_gb300.channels as CH
    from his_gb300.boundaries import all_edges
    from his_gb300.topology import build_topology
    from oracle.oracle import OracleCoupled, OracleLinks, OracleSWE1D, OracleSWE2D
    fx_x = H.load("exchange_overtop")
    fx = H.load("coupled_overtop_b2")
    spec = GC.COUPLED_BATCH_CASES["coupled_overtop_b2"]
    p = H.overtop_parts(fx_x)
    rain, inflow = GC.rain_fn_batch(spec), GC.inflow_batch(spec)
    for b, (gamma, manning) in enumerate(zip(spec["gamma"], spec["manning"])):
        two = OracleSWE2D(p.z2d, np.full(p.z2d.shape, manning), p.dx, p.cfg, all_edges("closed"))
        tp = build_topology(CH.apply_gamma(H.overtop_network(CH), [gamma]))
        one = OracleSWE1D(tp, p.cfg, inflow=lambda t, b=b: float(inflow(t)[b]), stage=p.stage)
        links = OracleLinks(**p.links)
        two.set_state(fx["h0"][b])
        one.A = np.ascontiguousarray(fx["A0"][b].reshape(one.A.shape))
        one.Q = np.ascontiguousarray(fx["Q0"][b].reshape(one.Q.shape))
        eng = OracleCoupled(two, one, links, p.cfg, rain=lambda t, b=b: float(rain(t)[b]))
        t = 0.0
        for k in range(spec["steps"]):
            t = eng.step(t, spec["t_end"], dt=float(fx["dt"][k]), n_sub=int(fx["n_sub"][k]))
            if k + 1 in spec["snap_at"]:
                for f in ("h", "hu", "hv"):
                    want = fx[f"{f}_{k + 1}"][b]
                    assert H.max_abs(getattr(two, f).reshape(want.shape), want) <= 1e-11, (b, k + 1, f)
                assert H.max_abs(one.A.reshape(-1), fx[f"A_{k + 1}"][b]) <= 1e-10, (b, k + 1)
                assert H.max_abs(one.Q.reshape(-1), fx[f"Q_{k + 1}"][b]) <= 1e-10, (b, k + 1)
        for term in GC_TERMS:
            want = float(fx[f"src_{term}"][b])
            assert float(eng.acc[term][0]) == pytest.approx(want, rel=1e-10, abs=1e-9), (b, term)
