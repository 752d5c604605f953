"""Exact solutions of the verification suite (no GPU): conservation and jump
conditions they must satisfy, and the recorded-metrics fixture's shape."""
import json
from pathlib import Path

import numpy as np
import pytest

from his_gb300 import analytical as A

G = 9.81


def test_ritter_conserves_mass_and_is_self_similar():
    x = np.linspace(0.0, 100.0, 200001)
    for t in (1.0, 3.0, 6.0):
        h, u = A.ritter(x, t, 50.0, 1.0)
        assert np.trapezoid(h, x) == pytest.approx(50.0, rel=1e-6)
        front = x[np.nonzero(h > 0)[0][-1]]
        assert front == pytest.approx(50.0 + 2 * np.sqrt(G) * t, abs=1e-3)


def test_riemann_star_state_satisfies_both_wave_relations():
    for hL, uL, hR, uR in ((1.0, 0.0, 0.1, 0.0), (1.0, 0.5, 0.7, -0.2), (1.0, -1.0, 1.0, 1.0), (0.3, 2.0, 1.5, 0.0)):
        hs, us = A.star_state(hL, uL, hR, uR)
        for hk, uk, sgn in ((hL, uL, -1.0), (hR, uR, 1.0)):
            if hs > hk:      # shock: mass and momentum jump conditions with its speed
                s = uk + sgn * np.sqrt(G * hk) * np.sqrt(0.5 * hs * (hs + hk)) / hk
                assert s * (hs - hk) == pytest.approx(hs * us - hk * uk, rel=1e-10, abs=1e-12)
                mom = lambda h, u: h * u * u + 0.5 * G * h * h
                assert s * (hs * us - hk * uk) == pytest.approx(mom(hs, us) - mom(hk, uk), rel=1e-10, abs=1e-12)
            else:            # rarefaction: the Riemann invariant across it
                assert us - sgn * 2 * np.sqrt(G * hs) == pytest.approx(uk - sgn * 2 * np.sqrt(G * hk), abs=1e-12)


def test_riemann_solution_conserves_mass():
    x = np.linspace(0.0, 100.0, 400001)
    h, _ = A.riemann(x, 6.0, 50.0, 1.0, 0.0, 0.1, 0.0)
    assert np.trapezoid(h, x) == pytest.approx(50.0 * 1.0 + 50.0 * 0.1, rel=1e-6)


def test_thacker_volume_is_constant_and_periodic():
    n, L = 400, 4000.0
    c = (np.arange(n) + 0.5) * L / n
    X, Y = np.meshgrid(c, c)
    h0, *_, T = A.thacker_planar(X, Y, 0.0, 1000.0, 2.0, 500.0, L)
    for t in (0.3 * T, 0.77 * T, T):
        h = A.thacker_planar(X, Y, t, 1000.0, 2.0, 500.0, L)[0]
        assert h.sum() == pytest.approx(h0.sum(), rel=2e-3)
    assert np.allclose(A.thacker_planar(X, Y, T, 1000.0, 2.0, 500.0, L)[0], h0, atol=1e-9)


@pytest.mark.parametrize("case", ["subcritical", "transcritical", "shock"])
def test_bump_depth_keeps_energy_and_discharge(case):
    x = (np.arange(125) + 0.5) * 0.2
    h, q, info = A.bump_exact(x, case)
    z = A.bump_bed(x)
    E = q * q / (2 * G * h * h) + h + z
    if case == "shock":
        up, down = x < info["x_shock"], x >= info["x_shock"]
        assert np.ptp(E[up]) < 1e-10 and np.ptp(E[down]) < 1e-10
        xs = info["x_shock"]
        h1, h2 = A.bump_exact(np.array([xs - 1e-9, xs + 1e-9]), case)[0]
        # sequent (conjugate) depths on either side of the jump
        assert 0.5 * h1 * (np.sqrt(1 + 8 * q * q / (G * h1 ** 3)) - 1) == pytest.approx(h2, rel=1e-6)
    else:
        assert np.ptp(E) < 1e-10
    if case == "transcritical":
        crest = np.argmin(np.abs(x - 10.0))
        assert h[crest] == pytest.approx((q * q / G) ** (1 / 3), rel=0.05)


def test_kinematic_wave_reaches_rain_times_length():
    t = np.linspace(0.0, 1500.0, 1501)
    q, te = A.kinematic_plane(t, 200.0, 0.05, 0.03, 100 / 3.6e6, 1500.0)
    assert q[-1] == pytest.approx(100 / 3.6e6 * 200.0)
    assert np.all(np.diff(q[t < te]) > 0)


def test_recorded_metrics_fixture_covers_the_analytic_cases():
    rec = json.loads((Path(__file__).resolve().parent / "golden" / "suite_recorded.json").read_text())
    assert set(rec["results"]) == {"2", "2b", "3", "4", "5", "6", "7"}
    assert rec["provenance"]["precision"] == "fp64"
    assert len(rec["results"]["2"]["metrics"]["o1_L1"]) == 4
