"""Per-member volume accounting, with the reference's terms, error measure and
messages (hydrointel/solver/massbalance.py:18-77).

relative_error = |dV - net| / max(gross, 1e-9 |V0| + 1), where dV counts 2-D
surface water, retained (stored) water and 1-D channel water, net = rain -
infiltration + boundary in - boundary out (2-D and 1-D), gross is the sum of their
magnitudes, and ``clip`` (volume created by clamping negative depths) is an error
term, not a source.

The accumulators live wherever the caller keeps them: the device-resident engine
accumulates on the GPU in float64 and hands this class host copies; the drop-in
classes ``add`` one step at a time, as the reference does.
"""
from __future__ import annotations

import numpy as np

TERMS = ("rain", "infiltration", "bnd2d_in", "bnd2d_out", "bnd1d_in", "bnd1d_out", "clip")


def _np(v):
    if hasattr(v, "detach"):
        return v.detach().to("cpu").double().numpy()
    return v


class MassBalance:
    def __init__(self, device, v0):
        self.device = device
        self.v0 = np.asarray(_np(v0), dtype=np.float64)
        self.batch = self.v0.shape[0] if self.v0.ndim else None
        self.acc: dict[tuple[str, str], object] = {}
        self.series: list[dict] = []

    def add(self, name: str, value) -> None:
        import torch
        if name not in TERMS:
            raise KeyError(name)
        if not torch.is_tensor(value):
            value = torch.tensor(np.asarray(value, dtype=np.float64), dtype=torch.float64)
        value = value.to(torch.float64)
        if self.batch is not None and value.dim() == 0:
            value = value.expand(self.batch)
        if tuple(value.shape) != self.v0.shape:
            raise ValueError(f"mass term '{name}' has shape {tuple(value.shape)}, expected {self.v0.shape}")
        key = (name, str(value.device))
        if key not in self.acc:
            self.acc[key] = torch.zeros_like(value)
        self.acc[key] += value

    def add_columns(self, names: tuple, values) -> None:
        """Add the columns of ``values`` (B x len(names) float64 device tensor) to the
        named terms in one device operation.  Each term receives the same float64 sums
        as ``add`` one column at a time (every index is distinct, so each accumulator
        element gets exactly one addition per call)."""
        import torch
        cache = self.__dict__.setdefault("_col_idx", {})
        idx = cache.get((names, values.device))
        if idx is None:
            for n in names:
                if n not in TERMS:
                    raise KeyError(n)
            if len(set(names)) != len(names):
                raise ValueError("a term may appear once per add_columns call")
            idx = cache[(names, values.device)] = torch.as_tensor([TERMS.index(n) for n in names],
                                                                   device=values.device)
        B = self.v0.size
        if tuple(values.shape) != (B, len(names)):
            raise ValueError(f"mass columns have shape {tuple(values.shape)}, expected ({B}, {len(names)})")
        key = ("_columns", str(values.device))
        acc = self.acc.get(key)
        if acc is None:
            acc = self.acc[key] = torch.zeros((len(TERMS), B), dtype=torch.float64, device=values.device)
        acc.index_add_(0, idx, values.t().to(torch.float64))

    def set_totals(self, totals: dict) -> None:
        """Replace the accumulators by totals computed elsewhere (e.g. on the device)."""
        import torch
        self.acc = {}
        for k, v in totals.items():
            if k not in TERMS:
                raise KeyError(k)
            t = torch.as_tensor(np.asarray(v, dtype=np.float64).reshape(self.v0.shape), dtype=torch.float64)
            self.acc[(k, "cpu")] = t

    def sources(self) -> dict:
        zero = np.zeros(self.v0.shape)
        out = {k: zero.copy() for k in TERMS}
        for (k, _), v in self.acc.items():
            if k == "_columns":
                cols = _np(v)
                for i, name in enumerate(TERMS):
                    out[name] = out[name] + cols[i].reshape(self.v0.shape)
                continue
            out[k] = out[k] + _np(v)
        return {k: (v if self.batch is not None else float(v)) for k, v in out.items()}

    def check(self, volume_now, t: float, record: bool = True):
        s = self.sources()
        net = s["rain"] - s["infiltration"] + s["bnd2d_in"] - s["bnd2d_out"] + s["bnd1d_in"] - s["bnd1d_out"]
        gross = s["rain"] + s["infiltration"] + s["bnd2d_in"] + s["bnd2d_out"] + s["bnd1d_in"] + s["bnd1d_out"]
        dv = np.asarray(_np(volume_now), dtype=np.float64) - self.v0
        err = np.abs(dv - net) / np.maximum(gross, 1e-9 * np.abs(self.v0) + 1.0)
        if record:
            f = (lambda x: x) if self.batch is not None else float
            self.series.append({"t": t, "volume": f(_np(volume_now)), "net_sources": f(net), "gross": f(gross),
                                "clip": f(s["clip"]), "rel_error": f(err)})
        return err if self.batch is not None else float(err)

    def assert_ok(self, volume_now, t: float, tol: float, label: str = ""):
        err = self.check(volume_now, t)
        if self.batch is not None:
            bad = np.nonzero(~(np.asarray(err) < tol))[0]
        else:
            bad = [] if err < tol else [0]
        if len(bad):
            where = f" in {label}" if label else ""
            if self.batch is not None:
                detail = ", ".join(f"member {int(i)}: {np.asarray(err)[int(i)]:.3e}" for i in bad[:8])
                raise AssertionError(f"mass balance violated{where} for {len(bad)}/{self.batch} batch members "
                                     f"(tolerance {tol:.1e}) -- {detail}")
            raise AssertionError(f"mass balance violated{where}: relative error {float(err):.3e} >= {tol:.1e} "
                                 f"(sources {self.sources()})")
        return err
