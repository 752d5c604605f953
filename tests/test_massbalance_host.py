"""Mass accounting host logic (hydrointel/solver/massbalance.py:18-77): the column
form used by the coupled step gives the same float64 totals as adding term by term,
and the error measure and messages follow the reference's."""
import numpy as np
import pytest
import torch

from his_gb300.massbalance import TERMS, MassBalance

COLS_2D = ("bnd2d_in", "bnd2d_out", "rain", "infiltration", "clip")
COLS_1D = ("bnd1d_in", "bnd1d_out", "clip")


def test_add_columns_equals_add_per_term():
    rng = np.random.default_rng(0)
    B = 5
    a, b = MassBalance("cpu", np.full(B, 1e6)), MassBalance("cpu", np.full(B, 1e6))
    for _ in range(300):
        v2 = torch.as_tensor(rng.lognormal(0, 3, (B, 5)))
        v1 = torch.as_tensor(rng.lognormal(0, 3, (B, 3)))
        for j, n in enumerate(COLS_2D):
            a.add(n, v2[:, j])
        for j, n in enumerate(COLS_1D):
            a.add(n, v1[:, j])
        b.add_columns(COLS_2D, v2)
        b.add_columns(COLS_1D, v1)
    sa, sb = a.sources(), b.sources()
    for k in TERMS:
        assert np.array_equal(sa[k], sb[k]), k


def test_add_columns_checks_names_and_shape():
    mb = MassBalance("cpu", np.zeros(3))
    with pytest.raises(KeyError):
        mb.add_columns(("rain", "snow"), torch.zeros(3, 2, dtype=torch.float64))
    with pytest.raises(ValueError):
        mb.add_columns(("rain", "rain"), torch.zeros(3, 2, dtype=torch.float64))
    with pytest.raises(ValueError):
        mb.add_columns(("rain", "clip"), torch.zeros(4, 2, dtype=torch.float64))


def test_error_measure_and_failure_names_the_member():
    mb = MassBalance("cpu", np.array([100.0, 100.0]))
    mb.add_columns(("rain",), torch.tensor([[10.0], [10.0]], dtype=torch.float64))
    err = mb.check(np.array([110.0, 120.0]), 0.0)
    assert err[0] == 0.0 and err[1] == pytest.approx(10.0 / 10.0)
    with pytest.raises(AssertionError, match="member 1"):
        mb.assert_ok(np.array([110.0, 120.0]), 0.0, 1e-3)
    single = MassBalance("cpu", 50.0)
    single.add("rain", 5.0)
    assert single.check(55.0, 0.0) == 0.0


def test_device_ledger_rows_read_as_the_reference_terms():
    """The 8-row ledger the library's step kernels add into reads back as the seven
    terms, the two models' clips summed, together with terms added from the host."""
    mb = MassBalance("cpu", np.array([0.0, 0.0]))
    led = mb.device_ledger("cpu")
    assert tuple(led.shape) == (8, 2)
    led += torch.arange(16, dtype=torch.float64).reshape(8, 2)
    mb.add("rain", torch.tensor([1.0, 1.0], dtype=torch.float64))
    s = mb.sources()
    assert list(s["rain"]) == [1.0, 2.0] and list(s["bnd1d_out"]) == [10.0, 11.0]
    assert list(s["clip"]) == [12.0 + 14.0, 13.0 + 15.0]
    mb.set_totals({k: np.zeros(2) for k in TERMS})
    assert mb.device_ledger("cpu") is led and float(led.abs().sum()) == 0.0
