"""Exact solutions of the verification cases (numpy, float64).

The classical solutions the reference's verification suite checks its solver
against (hydrointel/benchmarks/analytical.py:13-169), restated from the published
mathematics:

* Ritter (1892): dam break onto a dry bed, a centred rarefaction.
* The exact solution of the shallow-water Riemann problem with wet states (Stoker's
  wet-bed dam break): star depth from the shock / rarefaction wave curves, solved
  here by Newton's method, then sampled in the self-similar variable (x - x0)/t.
* Thacker (1981): planar free surface oscillating frictionlessly in a paraboloid.
* Steady frictionless flow over a parabolic bump (the sub-, transcritical and
  transcritical-with-shock cases of Goutal & Maurel, 1997): depths from the
  specific-energy (Bernoulli) cubic, the jump where the supercritical branch's
  sequent depth meets the downstream subcritical branch.
* Kinematic-wave runoff from a plane under uniform rain.
"""
from __future__ import annotations

import numpy as np

G = 9.81


# ------------------------------------------------------------------ dam breaks
def ritter(x, t, x0, h0, g=G):
    """Dry-bed dam break of depth h0 at x0, at time t > 0: (h, u)."""
    c0 = np.sqrt(g * h0)
    xi = (np.asarray(x, dtype=float) - x0) / t
    fan = (xi > -c0) & (xi < 2.0 * c0)
    h = np.where(xi <= -c0, h0, 0.0)
    u = np.zeros_like(xi)
    h = np.where(fan, (2.0 * c0 - xi) ** 2 / (9.0 * g), h)
    u = np.where(fan, (2.0 / 3.0) * (xi + c0), u)
    return h, u


def _wave_curve(h, hk, g):
    """Velocity jump across the wave joining depth hk to depth h, and its derivative:
    a rarefaction for h <= hk, a shock (Rankine-Hugoniot) otherwise."""
    if h <= hk:
        return 2.0 * (np.sqrt(g * h) - np.sqrt(g * hk)), np.sqrt(g / h)
    w = 0.5 * g * (1.0 / h + 1.0 / hk)
    sw = np.sqrt(w)
    return (h - hk) * sw, sw - (h - hk) * g / (4.0 * h * h * sw)


def star_state(hL, uL, hR, uR, g=G):
    """Depth and velocity between the two waves of a wet-wet Riemann problem."""
    if hL <= 0.0 or hR <= 0.0:
        raise ValueError("star_state needs wet states on both sides (use ritter for a dry bed)")
    cL, cR = np.sqrt(g * hL), np.sqrt(g * hR)
    if 2.0 * (cL + cR) <= uR - uL:
        raise ValueError("the states separate into a dry region")
    h = max((0.5 * (cL + cR) - 0.25 * (uR - uL)) ** 2 / g, 1e-12)   # two-rarefaction estimate
    for _ in range(100):
        fL, dL = _wave_curve(h, hL, g)
        fR, dR = _wave_curve(h, hR, g)
        step = (fL + fR + uR - uL) / (dL + dR)
        h_new = max(h - step, 0.5 * h)
        if abs(h_new - h) <= 1e-15 * h:
            h = h_new
            break
        h = h_new
    fL, _ = _wave_curve(h, hL, g)
    fR, _ = _wave_curve(h, hR, g)
    return h, 0.5 * (uL + uR) + 0.5 * (fR - fL)


def riemann(x, t, x0, hL, uL, hR, uR, g=G):
    """Exact wet-wet Riemann solution at time t > 0: (h, u)."""
    hs, us = star_state(hL, uL, hR, uR, g)
    cL, cR, cs = np.sqrt(g * hL), np.sqrt(g * hR), np.sqrt(g * hs)
    xi = (np.asarray(x, dtype=float) - x0) / t
    h = np.full_like(xi, hs)
    u = np.full_like(xi, us)
    left = xi <= us
    if hs > hL:                                    # left shock
        s = uL - cL * np.sqrt(0.5 * hs * (hs + hL)) / hL
        m = left & (xi <= s)
        h[m], u[m] = hL, uL
    else:                                          # left rarefaction
        head, tail = uL - cL, us - cs
        m = left & (xi <= head)
        h[m], u[m] = hL, uL
        m = left & (xi > head) & (xi < tail)
        c = (uL + 2.0 * cL - xi[m]) / 3.0
        h[m], u[m] = c * c / g, (uL + 2.0 * cL + 2.0 * xi[m]) / 3.0
    right = ~left
    if hs > hR:                                    # right shock
        s = uR + cR * np.sqrt(0.5 * hs * (hs + hR)) / hR
        m = right & (xi >= s)
        h[m], u[m] = hR, uR
    else:                                          # right rarefaction
        head, tail = uR + cR, us + cs
        m = right & (xi >= head)
        h[m], u[m] = hR, uR
        m = right & (xi > tail) & (xi < head)
        c = (-uR + 2.0 * cR + xi[m]) / 3.0
        h[m], u[m] = c * c / g, (uR - 2.0 * cR + 2.0 * xi[m]) / 3.0
    return h, u


# ------------------------------------------------------------------ Thacker
def thacker_planar(X, Y, t, a=1.0, h0=0.1, eta=0.5, L=4.0, g=G):
    """Planar surface in the paraboloid z = -h0 (1 - r^2 / a^2) centred in an L x L
    domain: (h, u, v, z, period)."""
    om = np.sqrt(2.0 * g * h0) / a
    xc, yc = X - 0.5 * L, Y - 0.5 * L
    z = -h0 * (1.0 - (xc * xc + yc * yc) / (a * a))
    surface = eta * h0 / (a * a) * (2.0 * xc * np.cos(om * t) + 2.0 * yc * np.sin(om * t) - eta)
    h = np.maximum(surface - z, 0.0)
    wet = h > 0.0
    u = np.where(wet, -eta * om * np.sin(om * t), 0.0)
    v = np.where(wet, eta * om * np.cos(om * t), 0.0)
    return h, u, v, z, 2.0 * np.pi / om


# ------------------------------------------------------------------ bump
BUMP_CASES = {"subcritical": {"q": 4.42, "h_out": 2.0}, "transcritical": {"q": 1.53},
              "shock": {"q": 0.18, "h_out": 0.33}}
BUMP_TOP = 0.2


def bump_bed(x):
    x = np.asarray(x, dtype=float)
    return np.where((x > 8.0) & (x < 12.0), 0.2 - 0.05 * (x - 10.0) ** 2, 0.0)


def _bernoulli_depth(q, E, z, branch, g=G):
    """Depth h with q^2 / (2 g h^2) + h + z = E on the subcritical ('sub', the largest
    positive root of h^3 + (z - E) h^2 + q^2/(2g) = 0) or supercritical ('super', the
    smallest positive root) branch, per cell."""
    z = np.atleast_1d(np.asarray(z, dtype=float))
    out = np.empty_like(z)
    k = q * q / (2.0 * g)
    for i, zi in enumerate(z):
        r = np.roots([1.0, zi - E, 0.0, k])
        r = np.real(r[(np.abs(np.imag(r)) < 1e-9) & (np.real(r) > 0.0)])
        if len(r) == 0:
            raise ValueError("no flow depth for this energy (choked section)")
        out[i] = r.max() if branch == "sub" else r.min()
    return out


def bump_exact(x, case, g=G):
    """Steady depth over the bump for case in BUMP_CASES: (h, q, info)."""
    x = np.asarray(x, dtype=float)
    z = bump_bed(x)
    spec = BUMP_CASES[case]
    q = spec["q"]
    info = {"q": q}
    if case == "subcritical":
        E = q * q / (2.0 * g * spec["h_out"] ** 2) + spec["h_out"]
        info["h_out"] = spec["h_out"]
        return _bernoulli_depth(q, E, z, "sub", g), q, info
    hc = (q * q / g) ** (1.0 / 3.0)
    E1 = 1.5 * hc + BUMP_TOP                       # critical at the crest
    h = np.where(x <= 10.0, _bernoulli_depth(q, E1, z, "sub", g), _bernoulli_depth(q, E1, z, "super", g))
    if case == "shock":
        hout = spec["h_out"]
        E2 = q * q / (2.0 * g * hout ** 2) + hout

        def mismatch(xs):
            zs = bump_bed(np.array([xs]))
            h1 = _bernoulli_depth(q, E1, zs, "super", g)[0]
            seq = 0.5 * h1 * (np.sqrt(1.0 + 8.0 * q * q / (g * h1 ** 3)) - 1.0)
            return seq - _bernoulli_depth(q, E2, zs, "sub", g)[0]

        # the downstream subcritical branch exists where E2 - z >= 1.5 hc (past the crest)
        z_ok = E2 - 1.5 * hc
        lo = 10.0 + (np.sqrt((BUMP_TOP - z_ok) / 0.05) if z_ok < BUMP_TOP else 0.0) + 1e-9
        hi = 25.0
        if mismatch(lo) * mismatch(hi) > 0.0:
            raise ValueError("no hydraulic jump in the channel for this outflow depth")
        for _ in range(80):
            mid = 0.5 * (lo + hi)
            if mismatch(lo) * mismatch(mid) <= 0.0:
                hi = mid
            else:
                lo = mid
        xs = 0.5 * (lo + hi)
        down = x >= xs
        h = h.copy()
        if down.any():
            h[down] = _bernoulli_depth(q, E2, z[down], "sub", g)
        info.update({"h_out": hout, "x_shock": float(xs)})
    return h, q, info


# ------------------------------------------------------------------ kinematic wave
def kinematic_plane(t, length, slope, n, rain_ms, duration):
    """Outlet discharge per unit width of a plane of the given length, slope and
    Manning n under uniform rain, for t <= duration: (q(t), time of equilibrium)."""
    alpha, m = np.sqrt(slope) / n, 5.0 / 3.0
    t = np.asarray(t, dtype=float)
    te = (length / (alpha * rain_ms ** (m - 1.0))) ** (1.0 / m)
    q = np.where(t < te, alpha * (rain_ms * t) ** m, rain_ms * length)
    return np.where(t <= duration, q, np.nan), te


__all__ = ["ritter", "riemann", "star_state", "thacker_planar", "bump_bed", "bump_exact", "kinematic_plane"]
