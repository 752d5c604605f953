"""Output path of the device-resident engine: series at output times, written by the
kernels, against the drop-in CoupledEngine.run(out_times=...) of the same storm.

Both runs cut their steps at the output times the same way and store float32
snapshots of a float64 state that agrees to ~1e-12, so the series agree to float32
rounding: bound 2e-6 m on depth, 2e-5 m/s on velocity, 2e-5 m on channel level and
1e-3 m^3/s on channel discharge, times to 1e-9 s.
"""
import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu


def test_engine_outputs_match_dropin_run():
    from his_gb300 import workloads as W
    from his_gb300.assembly import build_engine
    from his_gb300.config import SolverConfig
    from his_gb300.engine import FloodEngine
    storm = W.plain_small()
    interval = 900.0
    snaps = []
    eng = build_engine(storm)
    eng.run(storm.t_end, out_times=np.arange(0.0, storm.t_end + 1.0, interval), on_snapshot=snaps.append,
            progress_s=0)
    fe = FloodEngine([storm], SolverConfig(slot_width_frac=storm.slot_width_frac), precision="fp64",
                     output_interval=interval, track_peaks=True)
    reps = fe.run(chunk=256)
    assert reps[0].status == 1
    res = fe.flood_results()[0]
    n = len(snaps)
    assert res.depth_series.shape[0] == n == int(reps[0].outputs)
    assert np.allclose(res.times.numpy(), [s.t for s in snaps], rtol=0, atol=1e-9)
    h_ref = np.stack([s.h for s in snaps])
    assert np.abs(res.depth_series.numpy() - h_ref.reshape(res.depth_series.shape)).max() <= 2e-6
    for name, key in (("u", "u"), ("v", "v")):
        ref = np.stack([getattr(s, key) for s in snaps]).reshape(res.u.shape)
        assert np.abs(getattr(res, name).numpy() - ref).max() <= 2e-5, name
    interior = fe.members[0].topo.kind <= 1
    eta_ref = np.stack([s.eta1.reshape(-1)[interior] for s in snaps])
    q_ref = np.stack([s.q1.reshape(-1)[interior] for s in snaps])
    assert np.abs(res.channel_eta.numpy() - eta_ref).max() <= 2e-5
    assert np.abs(res.channel_q.numpy() - q_ref).max() <= 1e-3
    assert torch.equal(res.depth_max, res.depth_series.amax(0))
    # running peaks over every step bound the peaks over the output times (up to the
    # float32 rounding of the snapshots)
    assert bool((res.extras["depth_max_every_step"] + 1e-6 >= res.depth_max.double()).all())
    assert res.mass_balance_error < 1e-3
    # the volume ledger at every output time equals the drop-in run's snapshot ledger
    for k, snap in enumerate(snaps):
        for key, want in snap.ledger.items():
            got = res.extras["ledger"][k][key]
            assert got == pytest.approx(float(want), rel=1e-9, abs=1e-6), f"output {k}: ledger {key}"
    src = eng.mb.sources()
    assert res.infiltrated_volume_m3 == pytest.approx(src["infiltration"], rel=1e-9, abs=1e-6)


def test_served_outputs_equal_solo_outputs(tmp_path):
    from his_gb300 import workloads as W
    from his_gb300.engine import FloodEngine
    from his_gb300.serving import FloodServer
    storms = [W.uneven_member(f"serve-out/{k}", 0, (0.3 + 0.1 * k) * 3600.0) for k in range(3)]
    srv = FloodServer(precision="fp32", chunk_steps=16, tile=(58, 48), output_interval=300.0,
                      record_dir=tmp_path / "records", store_factor=2)
    st = srv.serve([(0.1 * k, s) for k, s in enumerate(storms)], max_wall_s=600)
    assert st.finished == 3 and st.rebuilds >= 2
    by_key = {r.storm.key: r for r in srv.done}
    for s in storms:
        fl = by_key[s.key].flood
        fe = FloodEngine([s], precision="fp32", tile=(58, 48), track_peaks=True, output_interval=300.0)
        fe.run(chunk=64)
        solo = fe.flood_results()[0]
        assert fl.depth_series.shape[0] == int(s.t_end // 300.0) + 1
        assert torch.equal(fl.times, solo.times)
        assert torch.equal(fl.depth_series, solo.depth_series) and torch.equal(fl.u, solo.u)
        assert torch.equal(fl.channel_eta, solo.channel_eta) and torch.equal(fl.channel_q, solo.channel_q)
        assert fl.mass_balance_error == solo.mass_balance_error < 1e-3
        assert fl.extras["ledger"] == solo.extras["ledger"]
    # the finished requests' records, written by the server, read back
    from his_gb300.records import load_record
    import json
    index = json.loads((srv.record_dir / "index.json").read_text())
    assert len(index) == 3
    for rid, entry in index.items():
        rec = load_record(srv.record_dir / entry["record"])
        req = next(r for r in srv.done if str(r.rid) == rid)
        assert rec["meta"]["key"] == req.storm.key
        assert rec["h"].shape == (req.flood.depth_series.shape[0], 81 // 2, 100 // 2)
        assert torch.equal(rec["depth_max_full"], req.flood.depth_series.amax(0))
