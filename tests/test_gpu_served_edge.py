"""The served request that ends in "implausible state": the float64 engine against the
oracle on the same storm (tests/golden/served_edge.npz, made by
tests/golden/make_served_edge.py).  Both choose their own CFL steps from their own
states; every 100 steps the clock and the largest depth along the north row agree, and
the engine stops the member as implausible at the step where the oracle first passes
the 10 m bound (hydrointel/solver/coupling.py:39, :169-192).  So the rise at the
transmissive north edge is the reference method's, not a fault of the kernels."""
import numpy as np
import pytest

import harness as H

pytestmark = pytest.mark.gpu


def test_north_edge_rise_follows_the_oracle_to_the_plausibility_bound():
    import make_served_edge as M
    from his_gb300 import _lib
    from his_gb300.config import SolverConfig
    from his_gb300.engine import FloodEngine
    fx = H.load("served_edge")
    storm = M.storm()
    fe = FloodEngine([storm], SolverConfig(), precision="fp64", graph_steps=int(fx["every"]), tile=(58, 16))
    done = 0
    worst_t = worst_h = 0.0
    for k, t, top in zip(fx["steps"], fx["t"], fx["top_max"]):
        fe.advance(int(k) - done)
        done = int(k)
        r = fe.reports()[0]
        h = fe.h[0].cpu().numpy()
        worst_t = max(worst_t, abs(r.t - float(t)))
        worst_h = max(worst_h, abs(float(h[-1].max()) - float(top)))
        if r.status != 0:
            break
    r = fe.reports()[0]
    print(f"engine stopped at step {r.steps}, t = {r.t:.2f} s ({_lib.STATUS[r.status]}); oracle passed 10 m at step "
          f"{int(fx['crossed_step'])}, t = {float(fx['crossed_t']):.2f} s; worst |dt| {worst_t:.2e} s, worst |d north "
          f"max| {worst_h:.2e} m")
    assert worst_t <= 1e-6 and worst_h <= 1e-6
    assert _lib.STATUS[r.status] == "implausible state"
    assert int(r.steps) == int(fx["crossed_step"])
    assert H.max_abs(fe.h[0].cpu().numpy()[-3:], fx["top_rows"]) <= 1e-6
