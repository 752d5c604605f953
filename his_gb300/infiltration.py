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

    # class parameters by land-use code: a mapping with arrays "f0_mmh", "fc_mmh" and
    # "k_per_h" (one entry per class), or a module with lookup(raster, name); None: the
    # land-use table of the installed hydrointel package that supplies the domain
    LANDUSE_TABLE = None

    @classmethod
    def use_landuse_table(cls, table) -> None:
        """Set the class-parameter table ``from_landuse`` reads (see LANDUSE_TABLE)."""
        cls.LANDUSE_TABLE = table

    @classmethod
    def _landuse_param(cls, landuse, name: str):
        import numpy as np
        table = cls.LANDUSE_TABLE
        if table is None:
            try:
                from hydrointel.domain import landuse as table      # the caller's own domain package
            except ImportError as e:
                raise ImportError("Horton.from_landuse needs the land-use class table: call "
                                  "Horton.use_landuse_table({...}) or install the package that defines "
                                  "the domain (hydrointel)") from e
        if hasattr(table, "lookup"):
            return np.asarray(table.lookup(landuse, name), dtype=np.float64)
        codes = np.asarray(landuse).astype(np.int64)
        values = np.asarray(table[name], dtype=np.float64)
        if codes.min() < 0 or codes.max() >= len(values):
            raise ValueError(f"land-use raster contains codes outside 0..{len(values) - 1}: "
                             f"min={codes.min()}, max={codes.max()}")
        return values[codes]

    @classmethod
    def from_landuse(cls, landuse, kappa, device=None, dtype=None, t0: float = 0.0) -> "Horton":
        """Fields from a land-use class raster (hydrointel/solver/infiltration.py:22-26):
        f0 and fc from the class table in mm/h times the intervention multiplier kappa
        (per cell or scalar), k from the table in 1/h; converted to m/s and 1/s."""
        import numpy as np
        import torch
        dtype = dtype or torch.float64
        kap = kappa.detach().to("cpu").double().numpy() if torch.is_tensor(kappa) else \
            np.asarray(kappa, dtype=np.float64)
        field = lambda a: torch.as_tensor(a, dtype=dtype, device=device)
        kap_t = field(kap)
        return cls(field(cls._landuse_param(landuse, "f0_mmh")) * MMH_TO_MS * kap_t,
                   field(cls._landuse_param(landuse, "fc_mmh")) * MMH_TO_MS * kap_t,
                   field(cls._landuse_param(landuse, "k_per_h")) / 3600.0, float(t0))

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
