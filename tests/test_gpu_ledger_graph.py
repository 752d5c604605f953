"""The ledger form of the 2-D step against the plain step, on a batch of member parts.

his_grid_step_ledger_async launches the step's stage kernels (every member part,
forked onto the library's streams and joined) and its finalize as one CUDA graph,
captured on the first call; his_grid_step_async issues the same launches one by one.
Both must leave the same state bit for bit, and the ledger's rows must equal the
step volumes summed in the same order (finalize adds the volumes of
swe2d.py:330-360 and boundaries.py:130-160 into the ledger rows).
"""
import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu

B, NY, NX, TILE = 24, 200, 163, (58, 16)       # 3 x 13 strip-chunks a member: three member parts
FIELDS = ("h", "hu", "hv", "s_filled", "infil_cum")
LG_RAIN, LG_INFIL, LG_BND2_IN, LG_BND2_OUT, LG_CLIP2 = 0, 1, 2, 3, 6


def _batch(seed=7):
    from his_gb300.boundaries import EdgeBC
    from his_gb300.config import SolverConfig
    from his_gb300.infiltration import Horton
    from his_gb300.swe2d import SWE2D
    rng = np.random.default_rng(seed)
    y, x = np.mgrid[0:NY, 0:NX]
    z = 0.003 * x + 0.4 * np.sin(y / 11.0) * np.cos(x / 17.0)
    n = 0.03 + 0.02 * rng.random((B, NY, NX))
    S = 0.002 * rng.random((B, NY, NX))
    f0, fc, k = 2e-5 * np.ones((B, NY, NX)), 2e-6 * np.ones((B, NY, NX)), 1e-3 * np.ones((B, NY, NX))
    bcs = {"west": EdgeBC("discharge", 0.3), "east": EdgeBC("stage", lambda t: 0.35 + 0.05 * np.sin(t / 50.0)),
           "south": EdgeBC("transmissive"), "north": EdgeBC("closed")}
    sim = SWE2D(z, n, 10.0, SolverConfig(), bcs, dtype=torch.float32, storage=S, horton=Horton(f0, fc, k, 10.0),
                batch=B, tile=TILE)
    h0 = np.clip(0.4 + 0.1 * rng.random((B, 1, 1)) - z[None], 0.0, None)
    sim.set_state(h0, 0.03 * h0, -0.02 * h0)
    return sim


def test_graph_launched_ledger_step_equals_the_plain_step():
    from his_gb300.massbalance import MassBalance
    a, b = _batch(), _batch()
    tiles = B * -(-NX // TILE[0]) * -(-NY // TILE[1])
    assert int(a._lib.his_engine_default_chains(B, tiles)) >= 2      # the step forks member parts
    mb = MassBalance(a.device, np.zeros(B))
    ledger = mb.device_ledger(a.device)
    sums = torch.zeros((B, 5), dtype=torch.float64, device=a.device)
    rain = 2e-5 * (1.0 + np.arange(B) / B)
    dt = 0.4
    for k in range(12):
        t = k * dt
        a.step_ledger(dt, t, rain, None, ledger.data_ptr())
        v = b.step(dt, t, rain)
        sums += v.table
    torch.cuda.synchronize()
    for f in FIELDS:
        assert torch.equal(getattr(a, f), getattr(b, f)), f
    s = sums.t()
    assert torch.equal(ledger[LG_RAIN], s[2]) and torch.equal(ledger[LG_INFIL], s[3])
    assert torch.equal(ledger[LG_BND2_IN], s[0]) and torch.equal(ledger[LG_BND2_OUT], s[1])
    assert torch.equal(ledger[LG_CLIP2], s[4])
    assert float(ledger[LG_RAIN].min()) > 0.0 and float(ledger[LG_INFIL].min()) > 0.0
