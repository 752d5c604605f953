"""The reference-signature engine assembly, host parts (hydrointel/engine.py:169-238),
against the reference's own build_engine recorded in tests/golden/assembly_run.npz:
scenario forcing tables, Horton fields from the land-use raster, the channel's initial
level, and the solver-configuration coercion."""
import numpy as np
import pytest

import harness as H


@pytest.fixture(scope="module")
def fx():
    return H.load("assembly_run")


def test_forcing_tables_reproduce_the_scenario_forcing(fx):
    from his_gb300.assembly import forcing_tables
    _, _, members, _ = H.assembly_inputs(fx)
    for m, mem in enumerate(members):
        f = forcing_tables(mem.forcing)
        ts = fx[f"m{m}_sample_t"]
        rain = np.array([f.rain_rate(t) for t in ts])
        tide = np.array([f.tide(t) for t in ts])
        inflow = np.array([f.inflow(t) for t in ts])
        assert np.array_equal(rain, fx[f"m{m}_sample_rain"])
        assert np.array_equal(inflow, fx[f"m{m}_sample_inflow"])
        assert np.max(np.abs(tide - fx[f"m{m}_sample_tide"])) <= 1e-12
        assert rain.max() > 0


def test_horton_from_landuse_matches_the_reference_fields(fx):
    import torch
    from his_gb300.infiltration import Horton
    _, domain, members, table = H.assembly_inputs(fx)
    saved = Horton.LANDUSE_TABLE
    Horton.use_landuse_table(table)
    try:
        h = Horton.from_landuse(domain.landuse, members[0].kappa, None, torch.float64,
                                t0=members[0].forcing.storm_start)
        for f in ("f0", "fc", "k"):
            assert np.array_equal(getattr(h, f).numpy(), fx[f"single_{f}"]), f
        assert h.t0 == members[0].forcing.storm_start
        with pytest.raises(ValueError, match="codes outside"):
            Horton.from_landuse(np.full((2, 2), len(table["f0_mmh"])), 1.0)
    finally:
        Horton.use_landuse_table(saved)


def test_initial_channel_level_matches_the_reference(fx):
    from his_gb300.assembly import _effective_gamma, forcing_tables, initial_channel_level
    from his_gb300.channels import apply_gamma
    from his_gb300.config import SolverConfig
    _, domain, members, _ = H.assembly_inputs(fx)
    mem = members[0]
    net = apply_gamma(domain.network, _effective_gamma(mem.gamma, mem.forcing))
    f = forcing_tables(mem.forcing)
    level = initial_channel_level(net, SolverConfig(), f.inflow(0.0), f.tide(0.0))
    want = fx["single_level0"].reshape(-1)
    assert level.shape == want.shape
    assert np.max(np.abs(level - want)) <= 1e-9


def test_solver_config_coerce_copies_known_fields():
    from types import SimpleNamespace
    from his_gb300.config import SolverConfig
    src = SimpleNamespace(cfl=0.3, flux="hll", spatial_order=1, precision="fp32", unknown_field=5)
    c = SolverConfig.coerce(src)
    assert (c.cfl, c.flux, c.spatial_order, c.precision) == (0.3, "hll", 1, "fp32")
    assert c.g == SolverConfig().g and not hasattr(c, "unknown_field")
    same = SolverConfig()
    assert SolverConfig.coerce(same) is same
