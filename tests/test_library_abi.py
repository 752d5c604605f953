"""The C-ABI library builds for sm_103a, loads, and exports every entry point its header
declares (no compute calls: this runs without a GPU)."""
import ctypes
import re
from pathlib import Path

from his_gb300 import _lib

ROOT = Path(__file__).resolve().parents[1]


def declared_symbols():
    text = (ROOT / "include" / "his_gb300.h").read_text()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(his_[a-z0-9_]+)\s*\(", text)))


def test_header_declares_the_bound_signatures():
    assert set(declared_symbols()) == set(_lib.SIGNATURES), "ctypes signatures and header disagree"


def test_library_exports_every_declared_symbol():
    lib = _lib.load()
    for name in declared_symbols():
        assert hasattr(lib, name), f"{name} not exported"
    assert lib.his_version() >= 100


def test_bad_arguments_map_to_value_error_without_a_gpu():
    lib = _lib.load()
    out = ctypes.c_void_p()
    cfg = _lib.SolverCfg(9.81, 1e-3, 1e-12, 0.45, 1e-4, 5.0, 0.45, 1.0, 1.7, 0.5, 0.5, 3, 1)   # order 3: invalid
    rc = lib.his_grid_create(0, ctypes.byref(cfg), 1, None, 0, 0, ctypes.byref(out))
    assert rc == _lib.HIS_ERR_BAD_ARG
    try:
        _lib.check(rc, "his_grid_create")
    except ValueError as e:
        assert "order" in str(e)
    else:
        raise AssertionError("expected ValueError")


def test_asynchronous_entry_points_refuse_missing_arguments_without_a_gpu():
    """Null handles and outputs are refused before any device call (HIS_ERR_BAD_ARG,
    with a message naming what is missing)."""
    lib = _lib.load()
    for name, args in (("his_grid_step_rate_async", (None, None, None)),
                       ("his_grid_max_rate_async", (None, None, None)),
                       ("his_grid_step_ledger_async", (None, None, None, None)),
                       ("his_net_step_ledger_async", (None, 0.5, 1, None, None, None))):
        rc = getattr(lib, name)(*args)
        assert rc == _lib.HIS_ERR_BAD_ARG, name
        assert "required" in _lib.last_error(), (name, _lib.last_error())
