"""Vectorised batch forcing against the per-member forcing it replaces on the host
path of the batched drop-in engine (rain blocks, inflow table, harmonic tide)."""
import numpy as np

from his_gb300 import workloads as W


def _members():
    rng = np.random.default_rng(3)
    fs = [W.Forcing(), W.Forcing(rain=np.array([1e-6, 2e-6]), q=np.array([5.0]), tide_on=False, tide_base=0.3)]
    for i in range(6):
        n_h = int(rng.integers(0, 4))
        fs.append(W.Forcing(rain_t0=float(rng.uniform(-600, 600)), rain_step=float(rng.choice([60.0, 600.0])),
                            rain=rng.uniform(0, 3e-5, int(rng.integers(1, 40))),
                            tide_base=float(rng.uniform(-1, 1)), tide_shift=float(rng.uniform(0, 4e4)),
                            tide_amp=tuple(rng.uniform(0, 1.5, n_h)), tide_w=tuple(rng.uniform(1e-5, 2e-4, n_h)),
                            tide_phase=tuple(rng.uniform(0, 6.3, n_h)), q_t0=float(rng.uniform(-100, 100)),
                            q_step=60.0, q=rng.uniform(0, 400, int(rng.integers(1, 30)))))
    return fs


def test_batch_forcing_equals_per_member():
    fs = _members()
    bf = W.BatchForcing(fs)
    ts = np.concatenate([np.random.default_rng(4).uniform(-2000, 60000, 500), [0.0, 60.0, 600.0, -1e-9, 1e12]])
    for t in ts:
        assert np.array_equal(bf.rain_rate(t), [f.rain_rate(t) for f in fs]), t
        assert np.array_equal(bf.inflow(t), [f.inflow(t) for f in fs]), t
        want = np.array([f.tide(t) for f in fs])
        assert np.allclose(bf.tide(t), want, rtol=1e-15, atol=1e-14), t     # numpy vs math cosine: an ulp
