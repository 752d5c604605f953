"""Fixture for the north-edge rise of the served request "served/51": the oracle (the C
restatement of the reference's float64 step, oracle/swe_oracle.c) runs the storm from
its start, choosing its own CFL steps, until a cell passes the 10 m plausibility bound
(hydrointel/solver/coupling.py:39), recording every 100 steps the clock, the largest
depth of the northernmost row and where it lies.  The transmissive north edge copies
the inflowing velocity into its ghost cells, so a valley lying against the edge keeps
filling: the reference's boundary model, reproduced by the oracle.

    python tests/golden/make_served_edge.py          # about 4 minutes on 8 cores
"""
from __future__ import annotations

import os
import sys
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
ROOT = HERE.parents[1]
sys.path[:0] = [str(ROOT), str(ROOT / "tests"), str(HERE)]

KEY, INDEX = "served", 51
EVERY = 100


def storm():
    from his_gb300 import workloads as W
    _, size, dur = W.served_requests(2.0, 600.0, KEY)[INDEX]
    return W.uneven_member(f"{KEY}/{INDEX}", size, dur)


def main():
    import harness as H
    from oracle import oracle as O
    O.set_threads(os.cpu_count() or 1)
    s = storm()
    orc = H.oracle_from_storm(s)
    t, k = 0.0, 0
    rec = []
    while t < s.t_end:
        t = orc.step(t, s.t_end)
        k += 1
        h = orc.two.h[0]
        crossed = h.max() > 10.0
        if k % EVERY == 0 or crossed:
            top = h[-1]
            rec.append((k, t, float(top.max()), int(top.argmax()), float(h.max())))
        if crossed:
            break
    rec = np.array(rec)
    np.savez_compressed(HERE / "served_edge.npz", steps=rec[:, 0].astype(np.int64), t=rec[:, 1],
                        top_max=rec[:, 2], top_argmax=rec[:, 3].astype(np.int64), h_max=rec[:, 4],
                        top_rows=orc.two.h[0][-3:].copy(), every=EVERY, crossed_step=k, crossed_t=t)
    print(f"{KEY}/{INDEX}: {s.terrain.nx}x{s.terrain.ny}, passed 10 m at step {k}, t = {t:.1f} s; "
          f"north row max {rec[-1, 2]:.3f} m at column {int(rec[-1, 3])}")


if __name__ == "__main__":
    main()
