"""Per-member failure isolation: one storm whose state goes bad stops alone.

The failure is made on the host: the initial depth a storm hands the engine has one
cell set to NaN (a non-finite state) or to 50 m (beyond the 10 m plausibility bound
of hydrointel/solver/coupling.py:39).  No kernel is made to fault.  The device
engine and the server retire exactly those members with the matching status (the
reference's generator records such a storm as failed and carries on,
data/generate.py:289-299), and every other member is bit-identical to its solo run.
The drop-in run loop raises NumericalInstabilityError naming the bad members
(coupling.py:169-192).
"""
import dataclasses

import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu

TILE = (58, 48)


def _poisoned(storm, value):
    """The same storm with one inland cell of its initial depth set to ``value``."""
    from his_gb300.workloads import Storm

    @dataclasses.dataclass
    class Poisoned(Storm):
        poison: float = 0.0

        def h0(self):
            h = super().h0().copy()
            ny, nx = h.shape
            h[(3 * ny) // 4, nx // 3] = self.poison
            return h

    return Poisoned(**{f.name: getattr(storm, f.name) for f in dataclasses.fields(storm)}, poison=value)


def _batch():
    from his_gb300 import workloads as W
    good = [W.uneven_member(f"isolate/{k}", 0, 0.25 * 3600.0) for k in range(4)]
    storms = [good[0], _poisoned(good[1], float("nan")), _poisoned(good[2], 50.0), good[3]]
    return storms, {1: "non-finite state", 2: "implausible state"}


def _solo(storm):
    from his_gb300.engine import FloodEngine
    fe = FloodEngine([storm], precision="fp32", tile=TILE, track_peaks=True)
    reps = fe.run(chunk=64)
    return fe, reps[0]


def _same(a, b):
    return torch.equal(a, b)


def test_engine_retires_only_the_bad_members():
    from his_gb300 import _lib
    from his_gb300.engine import FloodEngine
    storms, bad = _batch()
    fe = FloodEngine(storms, precision="fp32", tile=TILE, track_peaks=True, chains=2)
    reps = fe.run(chunk=64)
    status = [_lib.STATUS[r.status] for r in reps]
    assert status == ["done", bad[1], bad[2], "done"], status
    # the bad members stop at once: their first step shows the state
    assert reps[1].steps <= 1 and reps[2].steps <= 1, [r.steps for r in reps]
    for b in (0, 3):
        solo, rs = _solo(storms[b])
        r = reps[b]
        assert (r.steps, r.t, list(r.acc)) == (rs.steps, rs.t, list(rs.acc)), f"member {b}: clock or accumulators"
        for f in ("h", "hu", "hv", "peak_h", "A", "Q"):
            assert _same(getattr(fe, f)[b], getattr(solo, f)[0]), f"member {b}: {f} differs from the solo run"
        solo.close()
    fe.close()


def test_server_reports_bad_requests_and_serves_the_rest():
    from his_gb300.serving import FloodServer
    storms, bad = _batch()
    arrivals = [0.0, 0.05, 0.1, 0.3]
    srv = FloodServer(precision="fp32", chunk_steps=32, tile=TILE, keep_state=True)
    st = srv.serve(list(zip(arrivals, storms)), max_wall_s=600)
    assert st.finished == 4
    assert st.statuses == {"done": 2, "non-finite state": 1, "implausible state": 1}, st.statuses
    by_key = {r.storm.key: r for r in srv.done}
    assert by_key[storms[1].key].result.status == bad[1]
    assert by_key[storms[2].key].result.status == bad[2]
    for b in (0, 3):
        req = by_key[storms[b].key]
        solo, rs = _solo(storms[b])
        assert req.result.status == "done" and req.result.steps == rs.steps and req.result.t == rs.t
        assert np.array_equal(req.h, solo.h[0].cpu().numpy()), f"member {b}: final depth"
        assert np.array_equal(req.peak_h, solo.peak_h[0].cpu().numpy()), f"member {b}: peak depth"
        assert req.result.sources == solo.results()[0].sources, f"member {b}: accumulators"
        solo.close()


@pytest.mark.parametrize("value,member", [(float("nan"), 1), (50.0, 2)])
def test_dropin_run_names_the_bad_member(value, member):
    """The batched drop-in engine (shared dt, the reference's build_engine_batch) raises
    NumericalInstabilityError naming only the poisoned member."""
    from his_gb300 import workloads as W
    from his_gb300._lib import NumericalInstabilityError
    from his_gb300.assembly import build_engine_batch
    storms = W.batched_uniform(3)
    storms[member % 3] = _poisoned(storms[member % 3], value)
    eng = build_engine_batch(storms, dtype=torch.float32)
    with pytest.raises(NumericalInstabilityError) as ei:
        eng.check_plausible(0.0, "isolation")
    msg = str(ei.value)
    assert f"member {member % 3}:" in msg and "The run is invalid" in msg
    others = [m for m in range(3) if m != member % 3]
    assert all(f"member {m}:" not in msg for m in others), msg
