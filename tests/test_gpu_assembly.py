"""The engine assembled from the reference's own argument lists
(his_gb300.assembly.build_engine(cfg, domain, forcing, storage, kappa, manning, gamma,
landuse) and build_engine_batch(...)) against the reference's build_engine and
build_engine_batch on the same generated domain and scenarios
(tests/golden/assembly_run.npz, made by tests/golden/make_golden.py): the initial 2-D
and 1-D states, then 800 coupled steps on the reference's dt and substep sequence, in
float64.  This is the drop-in use: a caller keeps its configuration, domain and
scenario forcing and swaps the solver imports."""
import numpy as np
import pytest
import torch

import harness as H

pytestmark = pytest.mark.gpu

TERMS = ("rain", "infiltration", "bnd2d_in", "bnd2d_out", "bnd1d_in", "bnd1d_out", "clip")


def _np(t):
    return t.detach().double().cpu().numpy()


@pytest.fixture(scope="module")
def fx():
    return H.load("assembly_run")


@pytest.fixture(autouse=True)
def landuse_table(fx):
    from his_gb300.infiltration import Horton
    saved = Horton.LANDUSE_TABLE
    Horton.use_landuse_table(H.assembly_inputs(fx)[3])
    yield
    Horton.use_landuse_table(saved)


def _replay(eng, fx, tag):
    t = 0.0
    t_end = float(fx["m0_t_end"])
    for dt, n_sub in zip(fx[f"{tag}dt"], fx[f"{tag}n_sub"]):
        t = eng.step(t, t_end, dt=float(dt), n_sub=int(n_sub))
    return t


def _compare(eng, fx, tag, what):
    for f in ("h", "hu", "hv", "s_filled", "infil_cum"):
        d = H.max_abs(_np(getattr(eng.two, f)), fx[f"{tag}{f}_end"])
        assert d <= 1e-9, f"{what}: {f} differs by {d}"
    for f in ("A", "Q"):
        d = H.max_abs(_np(getattr(eng.one, f)), fx[f"{tag}{f}_end"])
        assert d <= 1e-8, f"{what}: {f} differs by {d}"
    src = eng.mb.sources()
    for k in TERMS:
        want = fx[f"{tag}src_{k}"]
        assert np.allclose(src[k], want, rtol=1e-9, atol=1e-6), f"{what}: {k} {src[k]} vs {want}"


def test_build_engine_with_the_reference_arguments(fx):
    from his_gb300.assembly import build_engine
    cfg, domain, members, _ = H.assembly_inputs(fx)
    m = members[0]
    eng = build_engine(cfg, domain, m.forcing, m.storage, m.kappa, m.manning, m.gamma, landuse=m.landuse,
                       device=torch.device("cpu"))
    assert np.array_equal(_np(eng.two.h), fx["single_h0"])
    assert H.max_abs(_np(eng.one.A), fx["single_A0"]) <= 1e-9
    t = _replay(eng, fx, "single_")
    print(f"single: t = {t:.1f} s, sources {eng.mb.sources()}")
    _compare(eng, fx, "single_", "build_engine")


def test_build_engine_batch_with_the_reference_arguments(fx):
    from his_gb300.assembly import build_engine_batch
    cfg, domain, members, _ = H.assembly_inputs(fx)
    cols = lambda k: [getattr(m, k) for m in members]
    eng, forcing = build_engine_batch(cfg, domain, cols("forcing"), cols("storage"), cols("kappa"), cols("manning"),
                                      cols("gamma"), cols("landuse"))
    assert forcing.B == len(members)
    assert np.array_equal(_np(eng.two.h), fx["batch_h0"])
    assert H.max_abs(_np(eng.one.A), fx["batch_A0"]) <= 1e-9
    t = _replay(eng, fx, "batch_")
    print(f"batch: t = {t:.1f} s, sources {eng.mb.sources()}")
    _compare(eng, fx, "batch_", "build_engine_batch")
