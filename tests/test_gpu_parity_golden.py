"""CUDA path against the oracle and the reference's golden vectors (float64, plain method).

Every case replays the reference's own step sequence.  The kernels are built
without fused multiply-add and follow the reference's expression order, so the
states agree with the oracle to a few ulp; the bound is 1e-12 absolute on states of
order 1 m and 1e-11 relative on per-step volumes.
"""
import numpy as np
import pytest
import torch

import golden_cases as GC
import harness as H

pytestmark = pytest.mark.gpu

STATE_TOL = 1e-12
VOL_REL = 1e-11
FIELDS = ("h", "hu", "hv", "s_filled", "infil_cum")


def _np(t):
    return t.detach().double().cpu().numpy()


@pytest.mark.parametrize("tile", [(58, 48), (5, 3), (3, 1), (7, 2), (122, 16), (218, 7), (346, 5)])
@pytest.mark.parametrize("name", list(GC.SWE2D_CASES))
def test_swe2d_matches_oracle_and_reference(name, tile):
    sim, spec, fx = H.cuda_swe2d(name, tile=tile)
    orc, _, _ = H.oracle_swe2d(name, fx)
    for k in range(spec["steps"]):
        dt, t = float(fx["dt"][k]), float(fx["t"][k])
        rate = float(sim.member_rates().max())
        assert rate == pytest.approx(orc.max_rate(), rel=1e-13, abs=1e-300), f"step {k}: CFL rate"
        assert rate == pytest.approx(float(fx["rate"][k]), rel=1e-13, abs=1e-300), f"step {k}: CFL rate vs reference"
        rain = GC.rain_value(spec, t)
        vol = sim.step(dt, t, rain)
        ovol = orc.step(dt, t, rain)
        for key, okey in (("bnd_in", "bnd_in"), ("bnd_out", "bnd_out"), ("rain", "rain"), ("infil", "infil"),
                          ("clip", "clip")):
            got = _np(getattr(vol, key)).reshape(-1)
            want = ovol[okey]
            scale = max(float(np.abs(want).max()), 1e-9)
            assert H.max_abs(got, want) <= VOL_REL * scale + 1e-13, f"step {k}: {key}"
        for f in FIELDS:
            got = _np(getattr(sim, f)).reshape(getattr(orc, f).shape)
            assert H.max_abs(got, getattr(orc, f)) <= STATE_TOL, f"step {k + 1}: {f} vs oracle"
        if k + 1 in spec["snap_at"]:
            for f in FIELDS:
                want = fx[f"{f}_{k + 1}"]
                assert H.max_abs(_np(getattr(sim, f)).reshape(want.shape), want) <= STATE_TOL, \
                    f"step {k + 1}: {f} vs reference"


@pytest.mark.parametrize("name", list(GC.SWE1D_CASES))
def test_swe1d_matches_oracle_and_reference(name):
    import his_gb300.channels as CH
    from his_gb300.config import SolverConfig
    from his_gb300.swe1d import SWE1D
    spec = GC.SWE1D_CASES[name]
    fx = H.load(name)
    net = GC.network(spec, CH)
    nets = [CH.apply_gamma(net, np.asarray(g)) for g in spec["gammas"]] if spec.get("batch") else net
    one = SWE1D(nets, SolverConfig(slot_width_frac=spec["slot_width_frac"]), inflow=GC.inflow_fn(spec),
                stage=GC.stage_fn(spec))
    one.A = torch.as_tensor(fx["A0"])
    one.Q = torch.as_tensor(fx["Q0"])
    orc, _, _ = H.oracle_swe1d(name, fx)
    for k in range(spec["steps"]):
        dt, t = float(fx["dt"][k]), float(fx["t"][k])
        assert one.max_dt() == pytest.approx(orc.max_dt(), rel=1e-13)
        assert one.max_dt() == pytest.approx(float(fx["max_dt"][k]), rel=1e-13)
        v = one.step(dt, t)
        ov = orc.step(dt, t)
        for key in ("bnd_in", "bnd_out", "clip"):
            assert H.max_abs(_np(getattr(v, key)).reshape(-1), ov[key]) <= VOL_REL * max(
                float(np.abs(ov[key]).max()), 1.0), f"step {k}: {key}"
        assert H.max_abs(_np(one.A).reshape(orc.A.shape), orc.A) <= 1e-11, f"step {k + 1}: A"
        assert H.max_abs(_np(one.Q).reshape(orc.Q.shape), orc.Q) <= 1e-11, f"step {k + 1}: Q"
        if k + 1 in spec["snap_at"]:
            assert H.max_abs(_np(one.A).reshape(fx[f"A_{k + 1}"].shape), fx[f"A_{k + 1}"]) <= 1e-11
            assert H.max_abs(_np(one.Q).reshape(fx[f"Q_{k + 1}"].shape), fx[f"Q_{k + 1}"]) <= 1e-11


def test_links_and_exchange_match_reference():
    from his_gb300.config import SolverConfig
    from his_gb300.coupling import exchange
    fx = H.load("exchange_overtop")
    spec = GC.EXCHANGE_CASES["exchange_overtop"]
    one, two, links, p = H.cuda_overtop(fx)
    assert np.array_equal(links.cell1d.numpy(), fx["links_cell1d"])
    assert np.array_equal(links.inv.numpy(), fx["links_inv"])
    assert np.array_equal(links.uniq_dev.numpy(), fx["links_uniq"])
    assert np.array_equal(links.length.numpy(), fx["links_length"])
    assert np.array_equal(links.z2.numpy(), fx["links_z2"])
    for i in range(spec["calls"]):
        two.set_state(fx[f"h_in_{i}"], fx[f"hu_in_{i}"], fx[f"hv_in_{i}"])
        one.A = torch.as_tensor(fx[f"A_in_{i}"])
        V = exchange(one, two, links, spec["dt"], SolverConfig())
        assert H.max_abs(_np(V), fx[f"V_{i}"]) <= 1e-12 * max(1.0, float(np.abs(fx[f"V_{i}"]).max()))
        for f in ("h", "hu", "hv"):
            assert H.max_abs(_np(getattr(two, f)), fx[f"{f}_out_{i}"]) <= 1e-13, f"call {i}: {f}"
        assert H.max_abs(_np(one.A), fx[f"A_out_{i}"]) <= 1e-12


def test_coupled_engine_matches_reference():
    from his_gb300.coupling import CoupledEngine
    fx_x = H.load("exchange_overtop")
    fx = H.load("coupled_overtop")
    spec = GC.COUPLED_CASES["coupled_overtop"]
    one, two, links, p = H.cuda_overtop(fx_x)
    two.set_state(fx["h0"])
    one.A = torch.as_tensor(fx["A0"])
    one.Q = torch.as_tensor(fx["Q0"])
    eng = CoupledEngine(two, one, p.cfg, rain=GC.rain_fn_coupled(spec), links=links)
    t = 0.0
    for k in range(spec["steps"]):
        dt = min(two.max_dt(), spec["t_end"] - t)
        assert dt == pytest.approx(float(fx["dt"][k]), rel=1e-12), f"step {k}: dt"
        n_sub = max(1, int(np.ceil(dt / one.max_dt() - 1e-9)))
        assert n_sub == int(fx["n_sub"][k])
        t = eng.step(t, spec["t_end"], dt=float(fx["dt"][k]), n_sub=int(fx["n_sub"][k]))
        if k + 1 in spec["snap_at"]:
            for f in ("h", "hu", "hv"):
                assert H.max_abs(_np(getattr(two, f)), fx[f"{f}_{k + 1}"]) <= 1e-11, f"step {k + 1}: {f}"
            assert H.max_abs(_np(one.A), fx[f"A_{k + 1}"]) <= 1e-10
            assert H.max_abs(_np(one.Q), fx[f"Q_{k + 1}"]) <= 1e-10
    src = eng.mb.sources()
    for term in ("rain", "infiltration", "bnd2d_in", "bnd2d_out", "bnd1d_in", "bnd1d_out", "clip"):
        assert src[term] == pytest.approx(float(fx[f"src_{term}"]), rel=1e-10, abs=1e-9), term
    assert eng.mb.check(eng.total_volume(), t, record=False) < 1e-12


def test_coupled_engine_cfl_choice_matches_reference():
    """The step choosing its own dt and substep count (both CFL rates fetched with one
    wait, 1-D substeps on a side stream) reproduces the reference's dt and n_sub
    sequence and its states."""
    from his_gb300.coupling import CoupledEngine
    fx_x = H.load("exchange_overtop")
    fx = H.load("coupled_overtop")
    spec = GC.COUPLED_CASES["coupled_overtop"]
    one, two, links, p = H.cuda_overtop(fx_x)
    two.set_state(fx["h0"])
    one.A = torch.as_tensor(fx["A0"])
    one.Q = torch.as_tensor(fx["Q0"])
    eng = CoupledEngine(two, one, p.cfg, rain=GC.rain_fn_coupled(spec), links=links)
    t = 0.0
    for k in range(spec["steps"]):
        n_sub_before = eng.log.n_sub_max
        t = eng.step(t, spec["t_end"])
        assert eng._last_dt == pytest.approx(float(fx["dt"][k]), rel=1e-12), f"step {k}: dt"
        assert eng.log.n_sub_max == max(n_sub_before, int(fx["n_sub"][k])), f"step {k}: n_sub"
        if k + 1 in spec["snap_at"]:
            for f in ("h", "hu", "hv"):
                assert H.max_abs(_np(getattr(two, f)), fx[f"{f}_{k + 1}"]) <= 1e-11, f"step {k + 1}: {f}"
            assert H.max_abs(_np(one.A), fx[f"A_{k + 1}"]) <= 1e-10
            assert H.max_abs(_np(one.Q), fx[f"Q_{k + 1}"]) <= 1e-10
    src = eng.mb.sources()
    for term in ("rain", "infiltration", "bnd2d_in", "bnd2d_out", "bnd1d_in", "bnd1d_out", "clip"):
        assert src[term] == pytest.approx(float(fx[f"src_{term}"]), rel=1e-10, abs=1e-9), term


def test_async_entry_points_refuse_pageable_outputs():
    """Outputs of the asynchronous entry points must be device or page-locked memory;
    a pageable array is refused before any work is enqueued."""
    from his_gb300 import _lib
    fx_x = H.load("exchange_overtop")
    one, two, links, p = H.cuda_overtop(fx_x)
    lib = _lib.load()
    pageable = np.zeros(max(two.B, 8) * 8)
    with pytest.raises(ValueError, match="page-locked"):
        _lib.check(lib.his_grid_max_rate_async(two._handle, pageable.ctypes.data, _lib.stream_handle()), "rate")
    with pytest.raises(ValueError, match="page-locked"):
        _lib.check(lib.his_net_max_rate_async(one._handle, pageable.ctypes.data, _lib.stream_handle()), "rate")
    pinned = torch.zeros(2 * two.B, dtype=torch.float64, pin_memory=True)
    two.rates_async(pinned[: two.B])
    one.rates_async(pinned)
    torch.cuda.synchronize()
    assert float(pinned[0]) == pytest.approx(float(one.member_rates()[0][0]), rel=0, abs=0)


def test_coupled_step_sees_state_written_between_steps():
    """The 1-D rates reduced ahead at the end of a step are dropped when the 1-D state
    is written before the next one (through torch, or by a standalone exchange): the
    next step's substep count is that of the written state."""
    import math
    from his_gb300.coupling import CoupledEngine, exchange
    fx_x = H.load("exchange_overtop")
    fx = H.load("coupled_overtop")
    spec = GC.COUPLED_CASES["coupled_overtop"]
    one, two, links, p = H.cuda_overtop(fx_x)
    two.set_state(fx["h0"])
    one.A = torch.as_tensor(fx["A0"])
    one.Q = torch.as_tensor(fx["Q0"])
    eng = CoupledEngine(two, one, p.cfg, rain=GC.rain_fn_coupled(spec), links=links)
    t = 0.0
    for _ in range(3):
        t = eng.step(t, spec["t_end"])

    def expected(t):
        dt = min(two.dt_from_rate(float(two.member_rates().max())), spec["t_end"] - t)
        return dt, max(1, math.ceil(dt / one.max_dt() - 1e-9))

    one.A = one.A * 4.0                          # deeper channel: faster 1-D waves
    dt, n_sub = expected(t)
    t = eng.step(t, spec["t_end"])
    assert eng._last_dt == dt and eng._last_n_sub == n_sub
    exchange(one, two, links, 30.0, p.cfg)       # the library writes A itself
    dt, n_sub = expected(t)
    t = eng.step(t, spec["t_end"])
    assert eng._last_dt == dt and eng._last_n_sub == n_sub


def test_coupled_step_takes_the_2d_rate_from_its_last_step_while_the_state_is_unchanged():
    """The 2-D CFL rates at the start of a coupled step are those the last step's own
    last stage formed (no reduction) while h, hu and hv are unwritten: equal, in
    float64, to a fresh reduction of the same state.  A write through torch or by a
    standalone exchange makes the next step reduce afresh, and its dt is that of the
    written state."""
    from his_gb300.coupling import CoupledEngine, exchange
    fx_x = H.load("exchange_overtop")
    fx = H.load("coupled_overtop")
    spec = GC.COUPLED_CASES["coupled_overtop"]
    one, two, links, p = H.cuda_overtop(fx_x)
    two.set_state(fx["h0"])
    one.A = torch.as_tensor(fx["A0"])
    one.Q = torch.as_tensor(fx["Q0"])
    eng = CoupledEngine(two, one, p.cfg, rain=GC.rain_fn_coupled(spec), links=links)
    t = 0.0
    for _ in range(3):
        t = eng.step(t, spec["t_end"])
    calls, pairs = [], []
    step_rate, reduce = two.step_rate_async, two.rates_async

    def from_step(out, stream=None):
        calls.append("step")
        step_rate(out, stream)
        fresh = torch.empty(out.shape, dtype=torch.float64, pin_memory=True)
        reduce(fresh, stream)                   # behind the copy on the same stream
        pairs.append((out, fresh))

    def reduced(out, stream=None):
        calls.append("reduce")
        reduce(out, stream)

    two.step_rate_async, two.rates_async = from_step, reduced
    for _ in range(3):                          # unchanged state: the step's own rates
        t = eng.step(t, spec["t_end"])
        out, fresh = pairs[-1]
        assert calls[-1] == "step" and torch.equal(out.clone(), fresh)

    def expected(t):
        return min(two.dt_from_rate(float(two.member_rates().max())), spec["t_end"] - t)

    two.h = two.h * 1.5                         # written through torch
    dt = expected(t)
    t = eng.step(t, spec["t_end"])
    assert calls[-1] == "reduce" and eng._last_dt == dt
    t = eng.step(t, spec["t_end"])
    assert calls[-1] == "step"
    exchange(one, two, links, 30.0, p.cfg)      # the library writes h itself
    dt = expected(t)
    t = eng.step(t, spec["t_end"])
    assert calls[-1] == "reduce" and eng._last_dt == dt


def test_batched_coupled_engine_matches_reference():
    """The batched drop-in CoupledEngine (two members with their own roughness,
    channel conveyance, states, inflow and rain; one shared CFL step) against the
    reference's batched run: the same dt and substep sequence, chosen by the step
    itself, and the same states and per-member mass terms."""
    import his_gb300.channels as CH
    from his_gb300.boundaries import all_edges
    from his_gb300.coupling import CoupledEngine, build_links
    from his_gb300.swe1d import SWE1D
    from his_gb300.swe2d import SWE2D
    fx_x = H.load("exchange_overtop")
    fx = H.load("coupled_overtop_b2")
    spec = GC.COUPLED_BATCH_CASES["coupled_overtop_b2"]
    p = H.overtop_parts(fx_x)
    B = len(spec["gamma"])
    n_b = np.stack([np.full(p.z2d.shape, m) for m in spec["manning"]])
    two = SWE2D(p.z2d, n_b, p.dx, p.cfg, all_edges("closed"), batch=B)
    nets = [CH.apply_gamma(H.overtop_network(CH), [g]) for g in spec["gamma"]]
    one = SWE1D(nets, p.cfg, inflow=GC.inflow_batch(spec), stage=p.stage)
    links = build_links(one, two)
    two.set_state(fx["h0"])
    one.A = torch.as_tensor(fx["A0"])
    one.Q = torch.as_tensor(fx["Q0"])
    eng = CoupledEngine(two, one, p.cfg, rain=GC.rain_fn_batch(spec), links=links)
    t = 0.0
    for k in range(spec["steps"]):
        t = eng.step(t, spec["t_end"])
        assert eng._last_dt == pytest.approx(float(fx["dt"][k]), rel=1e-12), f"step {k}: dt"
        assert eng._last_n_sub == int(fx["n_sub"][k]), f"step {k}: n_sub"
        if k + 1 in spec["snap_at"]:
            for f in ("h", "hu", "hv"):
                assert H.max_abs(_np(getattr(two, f)), fx[f"{f}_{k + 1}"]) <= 1e-11, f"step {k + 1}: {f}"
            assert H.max_abs(_np(one.A), fx[f"A_{k + 1}"]) <= 1e-10
            assert H.max_abs(_np(one.Q), fx[f"Q_{k + 1}"]) <= 1e-10
    src = eng.mb.sources()
    for term in ("rain", "infiltration", "bnd2d_in", "bnd2d_out", "bnd1d_in", "bnd1d_out", "clip"):
        want = np.asarray(fx[f"src_{term}"], dtype=np.float64)
        assert np.allclose(np.asarray(src[term]), want, rtol=1e-10, atol=1e-9), term
