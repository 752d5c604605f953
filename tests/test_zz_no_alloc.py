"""The allocation-free 2-D step (his_grid_step_noalloc) against his_grid_step.

Both entry points run the same strip kernels on the same decomposition (58-column
strips, 48-row chunks) and sum the volume partials in the same fixed order, so a grid
stepped through the scratch compiled into the library must equal a one-member grid set
stepped through its own allocated scratch bit for bit, call after call, in both
precisions.
This file sorts last so that the shared scratch has been through every other test's
process state first; it passes alone as well.
"""
import ctypes as C

import numpy as np
import pytest
import torch

from his_gb300 import _lib
from his_gb300.boundaries import EdgeBC
from his_gb300.config import SolverConfig
from his_gb300.infiltration import Horton

FIELDS = ("h", "hu", "hv", "s_filled", "infil_cum")


def _fields(ny, nx, seed):
    rng = np.random.default_rng(seed)
    y, x = np.mgrid[0:ny, 0:nx]
    z = 0.004 * x + 0.3 * np.sin(y / 9.0) * np.cos(x / 13.0) + 0.05 * rng.standard_normal((ny, nx))
    n = 0.03 + 0.02 * rng.random((ny, nx))
    S = 0.002 * rng.random((ny, nx))
    f0, fc = 2e-5 + 1e-5 * rng.random((ny, nx)), 2e-6 * np.ones((ny, nx))
    k = 1e-3 * np.ones((ny, nx))
    rw = 0.5 + rng.random((ny, nx))
    eta = 0.35 + 0.02 * np.sin(x / 5.0)
    h0 = np.clip(eta - z, 0.0, None)
    return z, n, S, (f0, fc, k), rw, h0


def _grid_set(ny, nx, dtype, order, seed):
    from his_gb300.swe2d import SWE2D
    z, n, S, (f0, fc, k), rw, h0 = _fields(ny, nx, seed)
    bcs = {"west": EdgeBC("discharge", 0.4), "east": EdgeBC("stage", lambda t: 0.3 + 0.05 * np.sin(t / 60.0)),
           "south": EdgeBC("transmissive"), "north": EdgeBC("closed")}
    cfg = SolverConfig(spatial_order=order)
    sim = SWE2D(z, n, 12.5, cfg, bcs, dtype=dtype, storage=S, horton=Horton(f0, fc, k, 15.0), rain_weight=rw)
    sim.set_state(h0, 0.02 * h0, -0.01 * h0)
    return sim


class Twin:
    """A one-member grid set and a copy of its state stepped by the allocation-free entry point."""

    def __init__(self, ny, nx, dtype, order, seed):
        self.sim = _grid_set(ny, nx, dtype, order, seed)
        self.state = {f: getattr(self.sim, f).clone() for f in FIELDS}
        d = _lib.GridDesc.from_buffer_copy(self.sim._descs[0])
        d.h, d.hu, d.hv = (self.state[f].data_ptr() for f in ("h", "hu", "hv"))
        d.s_filled, d.infil_cum = self.state["s_filled"].data_ptr(), self.state["infil_cum"].data_ptr()
        self.desc = d
        self.cfg = _lib.solver_cfg(self.sim.cfg)
        self.lib = _lib.load()

    def step(self, t, rain):
        dt = self.sim.max_dt()
        want = self.sim.step(dt, t, rain)
        params = self.sim.step_params(dt, t, rain)
        got = np.zeros(5)
        with torch.cuda.device(self.sim.device):
            _lib.check(self.lib.his_grid_step_noalloc(self.sim.prec, C.byref(self.cfg), C.byref(self.desc),
                                                      params, _lib.as_p(got), _lib.stream_handle()),
                       "his_grid_step_noalloc")
        return dt, want, got

    def compare(self, want, got, k):
        ref = np.array([float(getattr(want, f)) for f in ("bnd_in", "bnd_out", "rain", "infil", "clip")])
        assert np.array_equal(got, ref), f"call {k}: volumes {got} vs {ref}"
        for f in FIELDS:
            a = self.state[f]
            b = getattr(self.sim, f)
            assert torch.isfinite(a).all(), f"call {k}: {f} not finite"
            assert torch.equal(a, b), f"call {k}: {f} differs by {float((a.double() - b.double()).abs().max())}"


@pytest.mark.gpu
@pytest.mark.parametrize("order", [2, 1])
@pytest.mark.parametrize("dtype", [torch.float64, torch.float32], ids=["f64", "f32"])
def test_noalloc_step_matches_grid_step_two_calls_in_a_row(dtype, order):
    # a small grid first, so that the large one starts from scratch left over by another size
    small = Twin(23, 37, dtype, order, seed=11)
    large = Twin(140, 150, dtype, order, seed=12)      # 3 x 3 strips and chunks
    rain = 40.0 / 3.6e6
    t_small = t_large = 0.0
    for k in range(2):
        dt, want, got = small.step(t_small, rain)
        small.compare(want, got, k)
        t_small += dt
        dt, want, got = large.step(t_large, rain)
        large.compare(want, got, k)
        t_large += dt
    assert float(large.state["h"].double().sum()) > 0.0


NPART = 16                       # float64 partial sums per strip-chunk
STRIP_REF_BYTES = 24             # one strip-chunk record


def _plan_bytes(ny, nx, elem):
    """Scratch a grid needs: three stage planes, the partial sums and strip records of
    its 58-column x 48-row strip-chunks, and three 256-byte record slots, each region
    rounded up to 256 bytes."""
    a = lambda x: (x + 255) // 256 * 256
    n = -(-nx // 58) * -(-ny // 48)
    return 3 * a(ny * nx * elem) + a(8 * NPART * n) + a(STRIP_REF_BYTES * n) + 3 * 256


def _call_noalloc(prec, ny, nx, dt):
    """his_grid_step_noalloc on a grid of fake addresses: every argument check runs, and
    the call is rejected before any device work (dt = NaN fails the last check)."""
    lib = _lib.load()
    cfg = _lib.solver_cfg(SolverConfig())
    d = _lib.GridDesc()
    d.ny, d.nx = ny, nx
    d.dx = d.dy = 10.0
    for name in ("h", "hu", "hv", "s_filled", "infil_cum", "z", "manning"):
        setattr(d, name, 0x1000)                       # never dereferenced: rejected before any device work
    params = _lib.StepParams()
    params.dt = dt
    rc = lib.his_grid_step_noalloc(prec, C.byref(cfg), C.byref(d), C.byref(params), None, None)
    return rc, _lib.last_error()


@pytest.mark.parametrize("prec,elem", [(_lib.PREC_F64, 8), (_lib.PREC_F32, 4)], ids=["f64", "f32"])
def test_noalloc_accepts_up_to_its_scratch_size_exactly(prec, elem):
    """At the largest accepted grid (for a 600-row and a 1-row shape) the size checks pass
    and the NaN dt is what is rejected; one column more and the size is rejected."""
    for ny in (600, 1):
        lo, hi = 1, _lib.NOALLOC_SCRATCH_BYTES          # fits at lo, not at hi
        while hi - lo > 1:
            mid = (lo + hi) // 2
            lo, hi = (mid, hi) if _plan_bytes(ny, mid, elem) <= _lib.NOALLOC_SCRATCH_BYTES else (lo, mid)
        nx = lo
        assert _plan_bytes(ny, nx, elem) <= _lib.NOALLOC_SCRATCH_BYTES < _plan_bytes(ny, nx + 1, elem)
        rc, msg = _call_noalloc(prec, ny, nx, float("nan"))
        assert rc == _lib.HIS_ERR_BAD_ARG and "finite" in msg, (ny, nx, msg)
        rc, msg = _call_noalloc(prec, ny, nx + 1, float("nan"))
        assert rc == _lib.HIS_ERR_BAD_ARG and "scratch" in msg, (ny, nx + 1, msg)


def test_noalloc_rejects_a_grid_beyond_its_scratch_without_a_gpu():
    lib = _lib.load()
    cfg = _lib.solver_cfg(SolverConfig())
    d = _lib.GridDesc()
    d.ny, d.nx = 1000, 1000                            # 24 MB of float64 stage planes
    d.dx = d.dy = 10.0
    for name in ("h", "hu", "hv", "s_filled", "infil_cum", "z", "manning"):
        setattr(d, name, 0x1000)                       # never dereferenced: rejected before any device work
    params = _lib.StepParams()
    rc = lib.his_grid_step_noalloc(_lib.PREC_F64, C.byref(cfg), C.byref(d), C.byref(params), None, None)
    assert rc == _lib.HIS_ERR_BAD_ARG
    with pytest.raises(ValueError, match="scratch"):
        _lib.check(rc, "his_grid_step_noalloc")
