"""Dataset records (no GPU): coarsening, the record built from a FloodResult, and the
gzip round trip with its index."""
import json

import numpy as np
import torch

from his_gb300 import workloads as W
from his_gb300.engine import FloodResult
from his_gb300.records import coarsen_mean, flood_record, load_record, write_records


def _result(storm, nt=4, seed=0):
    rng = np.random.default_rng(seed)
    ny, nx = storm.terrain.ny, storm.terrain.nx
    h = torch.as_tensor(np.clip(rng.normal(0.1, 0.2, (nt, ny, nx)), 0, None), dtype=torch.float32)
    u = torch.as_tensor(rng.normal(0, 0.5, (nt, ny, nx)), dtype=torch.float32)
    v = torch.as_tensor(rng.normal(0, 0.5, (nt, ny, nx)), dtype=torch.float32)
    ledger = [{"v2d": 1.0 + k, "v1d": 2.0, "storage": 0.5, "rain": 0.1 * k, "infiltration": 0.0, "bnd2d_in": 0.0,
               "bnd2d_out": 0.0, "bnd1d_in": 0.0, "bnd1d_out": 0.0, "clip": 0.0} for k in range(nt)]
    return FloodResult(depth_max=h.amax(0), depth_series=h, u=u, v=v, channel_eta=torch.zeros(nt, 5),
                       channel_q=torch.zeros(nt, 5), times=torch.arange(nt, dtype=torch.float64) * 600.0,
                       infiltrated_volume_m3=1.0, stored_volume_m3=2.0, mass_balance_error=1e-7,
                       extras={"sources": {"rain": 1.0}, "ledger": ledger})


def test_coarsen_mean_keeps_block_totals():
    a = np.arange(2 * 7 * 9, dtype=float).reshape(2, 7, 9)
    c = coarsen_mean(a, 3)
    assert c.shape == (2, 2, 3)
    assert np.allclose(c.sum(axis=(1, 2)) * 9, a[:, :6, :9].sum(axis=(1, 2)))
    assert coarsen_mean(a, 1) is a


def test_record_fields_and_depth_weighted_velocity():
    storm = W.uneven_member("rec/0", 0, 1800.0)
    res = _result(storm)
    rec = flood_record(storm, res, store_factor=2)
    ny, nx = storm.terrain.ny // 2, storm.terrain.nx // 2
    assert rec["h"].shape == (4, ny, nx) and rec["u"].dtype == torch.float32
    h, u = res.depth_series.numpy(), res.u.numpy()
    hc = coarsen_mean(h, 2)
    want = np.where(hc > 0, coarsen_mean(h * u, 2) / np.where(hc > 0, hc, 1.0), 0.0)
    assert np.allclose(rec["u"].numpy(), want, atol=1e-6)
    assert torch.equal(rec["depth_max_full"], res.depth_series.amax(0))
    assert rec["forcing"]["rain_mmh"].shape == (64,) and rec["store_coarsen"] == 2
    assert rec["ledger"]["v2d"].shape == (4,) and "v2d_coarse" in rec["ledger"]
    assert set(rec["fields"]) >= {"manning", "storage", "horton_f0"}


def test_records_round_trip_with_index(tmp_path):
    storms = [W.uneven_member(f"rec/{k}", 0, 1800.0) for k in range(2)]
    idx = write_records([(s, _result(s, seed=k)) for k, s in enumerate(storms)], tmp_path, store_factor=1,
                        first_id=7)
    index = json.loads(idx.read_text())
    assert sorted(index) == ["7", "8"]
    rec = load_record(tmp_path / index["8"]["record"])
    assert rec["meta"]["key"] == "rec/1" and rec["h"].shape[0] == 4
    write_records([(storms[0], _result(storms[0]))], tmp_path, store_factor=1, compress=False, first_id=9)
    assert (tmp_path / "sim_00009.pt").exists() and len(json.loads(idx.read_text())) == 3


def test_record_path_default_resolves_to_the_existing_file(tmp_path):
    """compress=None: the plain .pt file unless only the gzip file exists (the reference's
    record lookup, hydrointel/data/generate.py:37-43); explicit True / False choose."""
    from his_gb300.records import record_path
    assert record_path(tmp_path, 3).name == "sim_00003.pt"
    (tmp_path / "sim_00003.pt.gz").write_bytes(b"")
    assert record_path(tmp_path, 3).name == "sim_00003.pt.gz"
    (tmp_path / "sim_00003.pt").write_bytes(b"")
    assert record_path(tmp_path, 3).name == "sim_00003.pt"
    assert record_path(tmp_path, 3, compress=True).name == "sim_00003.pt.gz"
    assert record_path(tmp_path, 3, compress=False).name == "sim_00003.pt"
