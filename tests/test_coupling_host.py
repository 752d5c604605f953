"""Host logic of the drop-in coupled step, without a GPU: where each step's CFL rates
come from (coupling.py:205-211 reads them at the start of every step).

The 2-D rates are the ones the engine's own last step formed while the 2-D state
version is what that step left; any write in between (through torch or by the
library's exchange) changes the version and the rates are reduced afresh.  The 1-D
rates reduced ahead at the end of a step serve the next step once, if the 1-D state
is unchanged.  The models are stand-ins that record which call the step makes.
"""
import contextlib

import torch


class _Two:
    B = 2
    device = None

    def __init__(self, calls):
        self.calls, self.version = calls, 0

    def state_version(self):
        return (self.version,)

    def rates_async(self, out, stream=None):
        self.calls.append("reduce 2-D")

    def step_rate_async(self, out, stream=None):
        self.calls.append("last step's 2-D")


class _One:
    def __init__(self, calls):
        self.calls, self.version = calls, 0

    def state_version(self):
        return (self.version,)

    def rates_async(self, out, stream=None):
        self.calls.append("reduce 1-D")


def _engine(monkeypatch):
    from his_gb300 import _lib
    from his_gb300.coupling import CoupledEngine
    monkeypatch.setattr(_lib, "on_device", lambda device: contextlib.nullcontext())
    calls = []
    eng = CoupledEngine.__new__(CoupledEngine)
    eng.two, eng.one = _Two(calls), _One(calls)
    eng._rates = torch.zeros(6, dtype=torch.float64)
    eng._rates1_at = eng._rates2_at = None
    return eng, calls


def test_2d_rates_come_from_the_last_step_only_while_the_state_is_unwritten(monkeypatch):
    eng, calls = _engine(monkeypatch)
    eng._enqueue_rates(True, False, 0)
    assert calls[-1] == "reduce 2-D"                      # no step of this engine yet
    eng._rates2_at = eng.two.state_version()              # what a step records after the 2-D launch
    eng._enqueue_rates(True, False, 0)
    assert calls[-1] == "last step's 2-D"
    eng._enqueue_rates(True, False, 0)
    assert calls[-1] == "last step's 2-D"                 # still the same state
    eng.two.version += 1                                  # written in between
    eng._enqueue_rates(True, False, 0)
    assert calls[-1] == "reduce 2-D"


def test_1d_rates_reduced_ahead_serve_one_step_of_an_unchanged_state(monkeypatch):
    eng, calls = _engine(monkeypatch)
    eng._rates1_at = eng.one.state_version()              # reduced ahead at the end of a step
    eng._enqueue_rates(False, True, 0)
    assert calls == []                                    # used as they are
    eng._enqueue_rates(False, True, 0)
    assert calls == ["reduce 1-D"]                        # used once: then reduced again
    eng._rates1_at = eng.one.state_version()
    eng.one.version += 1                                  # written after they were reduced
    eng._enqueue_rates(False, True, 0)
    assert calls == ["reduce 1-D", "reduce 1-D"]


def test_a_step_given_its_dt_reads_no_rates(monkeypatch):
    eng, calls = _engine(monkeypatch)
    eng._enqueue_rates(False, False, 0)
    assert calls == []
