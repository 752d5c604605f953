"""Host logic of the float32-against-float64 error report: arrival times from an
output series and the peak-depth, arrival and volume comparison."""
from types import SimpleNamespace

import numpy as np
import pytest

from his_gb300.accuracy import arrival_times, compare


def _result(series, times, infil=10.0, stored=5.0):
    h = np.asarray(series, dtype=np.float32)
    return SimpleNamespace(depth_series=h, times=np.asarray(times, dtype=np.float64), depth_max=h.max(axis=0),
                           infiltrated_volume_m3=infil, stored_volume_m3=stored)


def test_arrival_is_the_first_output_at_the_threshold():
    t = [0.0, 60.0, 120.0, 180.0]
    h = np.zeros((4, 1, 3))
    h[2:, 0, 0] = 0.2            # reaches 0.1 m at 120 s
    h[1:, 0, 1] = 0.1            # exactly the threshold at 60 s
    h[:, 0, 2] = 0.05            # never
    a = arrival_times(h, t, 0.1)
    assert a[0, 0] == 120.0 and a[0, 1] == 60.0 and np.isnan(a[0, 2])
    with pytest.raises(ValueError):
        arrival_times(h, t[:3])


def test_compare_reports_peak_arrival_and_volume_errors():
    t = [0.0, 60.0, 120.0]
    ref = np.zeros((3, 2, 2))
    ref[1:, 0, 0] = 0.5          # arrives at 60 s
    ref[2:, 0, 1] = 0.3          # arrives at 120 s
    test = ref.copy()
    test[1, 0, 1] = 0.15         # arrives one output earlier
    test[2, 0, 0] = 0.52         # peak 2 cm higher
    test[2, 1, 1] = 0.2          # floods where the reference does not
    m = compare(_result(test, t, infil=10.1), _result(ref, t))
    assert m["peak_depth_max_m"] == pytest.approx(0.2, abs=1e-6)
    assert m["wet_cells"] == 3
    assert m["arrival_cells"] == 2 and m["arrival_cells_in_one_run_only"] == 1
    assert m["arrival_max_s"] == 60.0 and m["arrival_rmse_s"] == pytest.approx(np.sqrt(60.0 ** 2 / 2))
    assert m["output_interval_s"] == 60.0
    assert m["infiltrated_volume_rel"] == pytest.approx(0.01)
    assert m["stored_volume_rel"] == 0.0
    same = compare(_result(ref, t), _result(ref, t))
    assert same["peak_depth_rmse_m"] == 0.0 and same["arrival_rmse_s"] == 0.0
    assert same["final_surface_volume_rel"] == 0.0


def test_series_metrics_in_the_reference_terms():
    """Depth RMSE / p99 / max over wet samples, flooded-area change and per-reach peak
    discharge, on hand-made series with known answers."""
    from types import SimpleNamespace
    import numpy as np
    import torch
    from his_gb300.accuracy import reference_criteria, series_metrics
    h_a = np.zeros((3, 4, 5))
    h_a[1:, 1:3, 1:4] = 0.4
    h_b = h_a.copy()
    h_b[2, 1, 1] += 0.01
    h_b[1:, 2, 3] = 0.1                    # this cell never reaches 0.15 m in run b
    q_a = np.array([[0.0, 0.0, 0.0], [2.0, -4.0, 1.0], [1.0, 3.0, 0.5]])
    q_b = q_a.copy()
    q_b[1, 1] = -4.2
    mk = lambda h, q: SimpleNamespace(depth_series=torch.as_tensor(h), channel_q=torch.as_tensor(q))
    m = series_metrics(mk(h_b, q_b), mk(h_a, q_a), reach_of=np.array([0, 1, 1]))
    wet = np.maximum(h_a, h_b) > 1e-3
    d = (h_b - h_a)[wet]
    assert abs(m["depth_rmse_wet_m"] - np.sqrt(np.mean(d ** 2))) < 1e-15
    assert abs(m["depth_max_abs_m"] - 0.3) < 1e-12
    assert abs(m["flooded_area_rel"] - 1.0 / 6.0) < 1e-12       # 6 cells >= 0.15 m in a, 5 in b
    assert abs(m["reach_peak_discharge_rel"] - 0.05) < 1e-12    # reach 1: 4.2 against 4.0
    crit = reference_criteria(dict(m, peak_depth_max_m=0.0, mass_error_fp32=1e-6))
    assert crit["reach_peak_discharge_rel"]["pass"] is False and crit["mass_balance_error"]["pass"] is True
