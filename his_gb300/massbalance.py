"""Per-member volume accounting of the coupled engine.

Contract kept from the reference (hydrointel/solver/massbalance.py:18-77): the class
name and constructor ``MassBalance(device, v0)``, the seven term names, ``add``,
``sources``, ``check`` and ``assert_ok``, the error measure

    relative_error = |dV - net| / max(gross, 1e-9 |V0| + 1)

(dV: change of 2-D surface + retained + 1-D channel water; net: the signed sources;
gross: their magnitudes; ``clip``, the volume created by clamping negative depths,
is an error term and enters neither), the ``mass_series`` record keys that
hydrointel/api.py reads, and ``AssertionError("mass balance violated ...")`` naming
the failing members.

Design: every term lives in one float64 ledger of shape (7, n) per device (n = batch
size, 1 unbatched), so adding a step's terms is one device operation and nothing is
copied to the host until ``sources`` or ``check`` is called.  Net and gross are a dot
product of the ledger with fixed sign and weight vectors.  The device-resident engine
keeps its own float64 ledger on the GPU and hands totals in through ``set_totals``.
"""
from __future__ import annotations

import numpy as np

TERMS = ("rain", "infiltration", "bnd2d_in", "bnd2d_out", "bnd1d_in", "bnd1d_out", "clip")
_ROW = {name: i for i, name in enumerate(TERMS)}
# contribution of each term to the net source (+ into the water body, - out of it) and
# to the gross turnover; clip counts in neither
NET_SIGN = np.array([1.0, -1.0, 1.0, -1.0, 1.0, -1.0, 0.0])
GROSS_WEIGHT = np.abs(NET_SIGN)


def _host(v) -> np.ndarray:
    if hasattr(v, "detach"):
        v = v.detach().to("cpu").double().numpy()
    return np.asarray(v, dtype=np.float64)


def relative_error(ledger: np.ndarray, volume_now, v0) -> tuple[np.ndarray, np.ndarray, np.ndarray]:
    """(error, net, gross) per member from a (7, n) ledger, the current and the initial
    volume (arrays of n)."""
    net = NET_SIGN @ ledger
    gross = GROSS_WEIGHT @ ledger
    floor = 1e-9 * np.abs(v0) + 1.0
    return np.abs((volume_now - v0) - net) / np.maximum(gross, floor), net, gross


class MassBalance:
    def __init__(self, device, v0):
        self.device = device
        v0 = _host(v0)
        self.batch = int(v0.shape[0]) if v0.ndim else None
        self.v0 = v0
        self._n = self.batch or 1
        self._ledgers: dict[str, object] = {}     # device name -> (7, n) float64 tensor
        self._device_ledgers: dict[str, object] = {}   # device name -> (8, n), filled by the library
        self._index_cache: dict = {}
        self.series: list[dict] = []

    # ------------------------------------------------------------------ adding
    def _ledger(self, device):
        import torch
        key = str(device)
        led = self._ledgers.get(key)
        if led is None:
            led = self._ledgers[key] = torch.zeros((len(TERMS), self._n), dtype=torch.float64, device=device)
        return led

    def add(self, name: str, value) -> None:
        """Accumulate one term for this step: a float64 scalar (every member) or one
        value per member, on any device."""
        import torch
        row = _ROW.get(name)
        if row is None:
            raise KeyError(name)
        v = value if torch.is_tensor(value) else torch.as_tensor(np.asarray(value, dtype=np.float64))
        v = v.to(torch.float64)
        want = (self.batch,) if self.batch is not None else ()
        if v.dim() and tuple(v.shape) != want:
            raise ValueError(f"mass term '{name}' has shape {tuple(v.shape)}, expected {want}")
        led = self._ledger(v.device)
        led[row] += v.reshape(-1) if v.dim() else v

    def add_columns(self, names: tuple, values) -> None:
        """Accumulate several terms at once from the columns of ``values`` (n x
        len(names), float64, on the device that produced them): one index_add into
        the ledger, the same float64 sums as adding the columns one by one (each
        ledger element receives one addition per call)."""
        import torch
        idx = self._index_cache.get((names, values.device))
        if idx is None:
            unknown = [n for n in names if n not in _ROW]
            if unknown:
                raise KeyError(unknown[0])
            if len(set(names)) != len(names):
                raise ValueError("a term may appear once per add_columns call")
            idx = torch.as_tensor([_ROW[n] for n in names], device=values.device)
            self._index_cache[(names, values.device)] = idx
        if tuple(values.shape) != (self._n, len(names)):
            raise ValueError(f"mass columns have shape {tuple(values.shape)}, expected ({self._n}, {len(names)})")
        self._ledger(values.device).index_add_(0, idx, values.t().to(torch.float64))

    def device_ledger(self, device):
        """An 8 x n float64 ledger on ``device`` that the library's step kernels add a
        coupled step's volumes into (his_grid_step_ledger_async, his_net_step_ledger_async):
        rows rain, infiltration, 2-D boundary in and out, 1-D boundary in and out, then
        the 2-D and the 1-D clip.  It is read with the other accumulators."""
        import torch
        key = str(device)
        led = self._device_ledgers.get(key)
        if led is None:
            led = self._device_ledgers[key] = torch.zeros((8, self._n), dtype=torch.float64, device=device)
        return led

    def set_totals(self, totals: dict) -> None:
        """Replace the ledger by totals accumulated elsewhere (e.g. on the device)."""
        import torch
        led = np.zeros((len(TERMS), self._n))
        for name, v in totals.items():
            if name not in _ROW:
                raise KeyError(name)
            led[_ROW[name]] = _host(v).reshape(self._n)
        self._ledgers = {"cpu": torch.as_tensor(led)}
        for dev in self._device_ledgers.values():     # kept: the library holds their addresses
            dev.zero_()

    # ---------------------------------------------------------------- reading
    def ledger(self) -> np.ndarray:
        """All terms as a host (7, n) float64 array (ledgers of several devices summed)."""
        total = np.zeros((len(TERMS), self._n))
        for led in self._ledgers.values():
            total += _host(led)
        clip = _ROW["clip"]
        for dev in self._device_ledgers.values():
            d = _host(dev)
            total[:clip] += d[:clip]
            total[clip] += d[clip] + d[clip + 1]
        return total

    def sources(self) -> dict:
        """Accumulated volume per term: floats unbatched, arrays of the members batched."""
        led = self.ledger()
        if self.batch is None:
            return {name: float(led[i, 0]) for i, name in enumerate(TERMS)}
        return {name: led[i].copy() for i, name in enumerate(TERMS)}

    def check(self, volume_now, t: float, record: bool = True):
        """Relative error per member now; ``record`` appends a mass-series entry."""
        led = self.ledger()
        vol = _host(volume_now).reshape(self._n)
        err, net, gross = relative_error(led, vol, self.v0.reshape(self._n))
        scalar = self.batch is None
        out = (lambda a: float(a[0])) if scalar else (lambda a: a)
        if record:
            self.series.append({"t": t, "volume": out(vol), "net_sources": out(net), "gross": out(gross),
                                "clip": out(led[_ROW["clip"]]), "rel_error": out(err)})
        return out(err)

    def assert_ok(self, volume_now, t: float, tol: float, label: str = ""):
        """``check`` and raise AssertionError naming the members at or above ``tol``."""
        err = self.check(volume_now, t)
        failing = np.flatnonzero(~(np.atleast_1d(err) < tol))
        if failing.size == 0:
            return err
        where = f" in {label}" if label else ""
        if self.batch is None:
            raise AssertionError(f"mass balance violated{where}: relative error {float(err):.3e} >= {tol:.1e} "
                                 f"(sources {self.sources()})")
        named = ", ".join(f"member {int(m)}: {err[int(m)]:.3e}" for m in failing[:8])
        raise AssertionError(f"mass balance violated{where} for {failing.size}/{self.batch} batch members "
                             f"(tolerance {tol:.1e}) -- {named}")


__all__ = ["MassBalance", "TERMS", "relative_error"]
