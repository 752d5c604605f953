"""Serving form (continuous batching) and the work-decomposition tuner on the GPU.

The serving loop rebuilds the engine whenever requests join or finish; every
continuing member resumes its clock and accumulators, and every batch uses one
decomposition.  Stated tolerance: a served request's final state, peak fields, clock
and float64 accumulators equal the same storm run alone, exactly (bit for bit).
"""
import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu

TILE = (58, 48)


def _storms(n, key, size=0, hours=(0.25, 0.35, 0.3, 0.4)):
    from his_gb300 import workloads as W
    return [W.uneven_member(f"{key}/{k}", size, hours[k % len(hours)] * 3600.0) for k in range(n)]


def _alone(storm):
    from his_gb300.engine import FloodEngine
    fe = FloodEngine([storm], precision="fp32", tile=TILE, track_peaks=True)
    reps = fe.run(chunk=128)
    return fe, reps[0]


def test_served_requests_equal_their_solo_runs():
    from his_gb300.serving import FloodServer
    storms = _storms(4, "serve-vs-solo")
    # staggered arrivals: members join and leave while others run (several rebuilds)
    arrivals = [0.0, 0.15, 0.3, 0.6]
    srv = FloodServer(precision="fp32", chunk_steps=24, tile=TILE, keep_state=True)
    st = srv.serve(list(zip(arrivals, storms)), max_wall_s=600)
    assert st.finished == 4 and st.statuses == {"done": 4}, st
    assert st.rebuilds >= 3
    assert st.max_mass_error < 1e-3
    by_key = {r.storm.key: r for r in srv.done}
    for s in storms:
        req = by_key[s.key]
        fe, rep = _alone(s)
        res = fe.results()[0]
        assert req.result.steps == rep.steps and req.result.t == rep.t, s.key
        assert np.array_equal(req.h, fe.h[0].cpu().numpy()), f"{s.key}: final depth differs from the solo run"
        assert np.array_equal(req.peak_h, fe.peak_h[0].cpu().numpy()), f"{s.key}: peak depth differs"
        assert np.array_equal(req.peak_speed, fe.peak_speed[0].cpu().numpy()), f"{s.key}: peak speed differs"
        assert req.result.sources == res.sources, f"{s.key}: accumulators differ"
        assert req.result.mass_error == res.mass_error


def test_admission_waits_for_hbm_budget():
    from his_gb300.serving import FloodServer, estimate_bytes
    storms = _storms(3, "serve-budget", hours=(0.2,))
    need = estimate_bytes(storms[0], torch.float32)
    srv = FloodServer(precision="fp32", chunk_steps=32, tile=TILE, hbm_budget=int(2.5 * need))
    st = srv.serve([(0.0, s) for s in storms], max_wall_s=600)
    assert st.finished == 3 and st.statuses == {"done": 3}
    assert st.max_members == 2                       # the third waited for a slot
    waited = sorted(r.admitted for r in srv.done)
    assert waited[0] == 0.0 or waited[0] < waited[2]
    assert max(r.admitted - r.arrival for r in srv.done) > 0.0


def test_a_request_larger_than_the_budget_is_refused():
    from his_gb300.serving import FloodServer
    storms = _storms(1, "serve-too-big", hours=(0.1,))
    srv = FloodServer(precision="fp32", tile=TILE, hbm_budget=1024)
    with pytest.raises(ValueError, match="HBM budget"):
        srv.serve([(0.0, storms[0])], max_wall_s=60)


def test_tuned_decomposition_gives_the_same_state():
    """The tuner only changes the order of the volume sums: any chosen tile yields the
    same state as the default decomposition, bit for bit."""
    from his_gb300.autotune import candidates, choose_tile
    from his_gb300.engine import FloodEngine
    storms = _storms(3, "tune", size=1)
    ref = FloodEngine(storms, precision="fp32", tile=TILE)
    members = ref.members
    import his_gb300._lib as L
    gdesc = (L.GridDesc * len(members))()
    for b, m in enumerate(members):
        m.fill_grid(gdesc[b])
    tile = choose_tile(ref.device, ref.prec, ref.cfg, gdesc, [m.state() for m in members], use_cache=False)
    assert tile in candidates([m.shape for m in members])
    other = (122, 16) if tuple(tile) == TILE else tuple(tile)
    alt = FloodEngine(storms, precision="fp32", tile=other)
    ref.advance(60)
    alt.advance(60)
    for a, b in zip(ref.members, alt.members):
        assert torch.equal(a.h, b.h) and torch.equal(a.hu, b.hu) and torch.equal(a.hv, b.hv)
        assert torch.equal(a.A, b.A) and torch.equal(a.Q, b.Q)
    ra, rb = ref.reports(), alt.reports()
    for x, y in zip(ra, rb):
        assert x.t == y.t and x.steps == y.steps
        # volume partials are float32 sums within a strip-chunk: the order changes them
        # at float32 rounding
        assert np.allclose(list(x.acc), list(y.acc), rtol=1e-6, atol=1e-6)
