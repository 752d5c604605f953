"""Horton infiltration parameters (hydrointel/solver/infiltration.py:15-37).

f(t) = fc + (f0 - fc) exp(-k max(t - t0, 0))  [m/s], evaluated per cell and per
member at the start of each step inside the CUDA source kernel; this class only
holds the three fields and the decay origin t0.
"""
from __future__ import annotations

from dataclasses import dataclass

MMH_TO_MS = 1.0 / 3.6e6


@dataclass
class Horton:
    f0: object      # m/s, (ny, nx) or (B, ny, nx) array / tensor
    fc: object      # m/s
    k: object       # 1/s
    t0: float = 0.0

    @classmethod
    def constant(cls, rate_ms, shape, device=None, dtype=None) -> "Horton":
        import torch
        r = torch.full(shape, float(rate_ms), dtype=dtype or torch.float64, device=device)
        return cls(r, r.clone(), torch.zeros_like(r))

    @classmethod
    def from_rates_mmh(cls, f0_mmh, fc_mmh, k_per_h, t0: float = 0.0) -> "Horton":
        import numpy as np
        return cls(np.asarray(f0_mmh, float) * MMH_TO_MS, np.asarray(fc_mmh, float) * MMH_TO_MS,
                   np.asarray(k_per_h, float) / 3600.0, t0)

    def rate(self, t: float):
        """Host evaluation, for inspection only (the step evaluates it on the device)."""
        import torch
        f0, fc, k = (torch.as_tensor(a, dtype=torch.float64) for a in (self.f0, self.fc, self.k))
        tt = max(float(t) - self.t0, 0.0)
        return fc + (f0 - fc) * torch.exp(-k * tt)
