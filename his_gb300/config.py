"""Solver constants, with the reference's field names and defaults
(hydrointel/config.py:96-131, ``SolverConfig``).

``precision`` selects the arithmetic of the CUDA step: ``"fp64"`` is the plain
method (everything in float64); ``"fp32"`` is the production form (float32 state,
fluxes and updates; float64 surface-elevation differences and volume
accumulators).  ``compile`` is accepted for signature compatibility and ignored:
the step is always the hand-written CUDA kernels.
"""
from __future__ import annotations

from dataclasses import asdict, dataclass


@dataclass
class SolverConfig:
    g: float = 9.81
    h_dry: float = 1e-3
    kp_eps: float = 1e-12
    cfl: float = 0.45
    dt_min: float = 1e-4
    dt_max: float = 5.0
    spatial_order: int = 2
    flux: str = "hllc"
    precision: str = "fp64"
    compile: bool = True
    mass_tol: float = 1e-3
    recession_h: float = 2.0
    output_interval_s: float = 900.0
    slot_width_frac: float = 1.0
    cfl_1d: float = 0.45
    weir_cw: float = 1.7
    exchange_limit: float = 0.5
    exchange_relax: float = 0.5

    def validate(self) -> "SolverConfig":
        if self.spatial_order not in (1, 2):
            raise ValueError(f"spatial_order must be 1 or 2 (got {self.spatial_order})")
        if self.flux not in ("hllc", "hll"):
            raise ValueError(f"flux must be 'hllc' or 'hll' (got {self.flux!r})")
        if self.precision not in ("fp64", "fp32"):
            raise ValueError(f"precision must be 'fp64' or 'fp32' (got {self.precision!r})")
        if not (0 < self.cfl <= 1.0 and 0 < self.cfl_1d <= 1.0):
            raise ValueError("cfl and cfl_1d must lie in (0, 1]")
        if not (0 < self.dt_min <= self.dt_max):
            raise ValueError("need 0 < dt_min <= dt_max")
        return self

    def to_dict(self) -> dict:
        return asdict(self)

    @classmethod
    def coerce(cls, cfg) -> "SolverConfig":
        """This class from any object carrying the solver fields (the reference's own
        SolverConfig, a RunConfig's ``solver``): every field found is copied, the
        rest keep their defaults."""
        if isinstance(cfg, cls):
            return cfg
        out = cls()
        for name in out.__dataclass_fields__:
            if hasattr(cfg, name):
                setattr(out, name, getattr(cfg, name))
        return out
