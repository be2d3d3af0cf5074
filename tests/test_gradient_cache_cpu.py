"""Host logic of the gradient call's problem cache (no GPU): the first call of
a shape runs eagerly, the second captures the CUDA graph, later calls reload
their inputs and replay it; a shape mismatch at reload builds a new problem;
at most two problems are kept."""
import types

import numpy as np
import pytest

from discoeb_gb300 import gradient


class FakeProblem:
    made = []

    def __init__(self, plist, backgrounds, pert, kmodes, aexp_out, **opts):
        self.log = []
        self.graph = None
        self.n = len(plist)
        self.d_P, self.d_dl = "P", "dl"
        FakeProblem.made.append(self)

    def load(self, plist, backgrounds, pert):
        if len(plist) != self.n:
            raise ValueError("shape")
        self.log.append("load")

    def run(self):
        self.log.append("run")
        return "P", "dl"

    def capture(self):
        self.log.append("capture")
        self.graph = object()

    def replay(self):
        self.log.append("replay")
        return "P", "dl"


@pytest.fixture
def fake(monkeypatch):
    fake_torch = types.SimpleNamespace(cuda=types.SimpleNamespace(current_device=lambda: 0))
    monkeypatch.setitem(__import__("sys").modules, "torch", fake_torch)
    monkeypatch.setattr(gradient, "GradientProblem", FakeProblem)
    monkeypatch.setattr(gradient, "_problems", {})
    FakeProblem.made = []
    return FakeProblem


def _call(nc=1, num_k=4, kind="native"):
    plist = [dict(A_s=2e-9)] * nc
    pert = [[("Omegam", 1e-5, {}, {})]] * nc
    return gradient._run_cached(plist, kind, pert, np.geomspace(1e-3, 1.0, num_k), [1.0], dict(rtol=1e-5))


def test_run_then_capture_then_replay(fake):
    for _ in range(4):
        _call()
    assert len(fake.made) == 1
    assert fake.made[0].log == ["run", "load", "capture", "load", "replay", "load", "replay"]


def test_other_shapes_get_their_own_problem_and_the_cache_is_bounded(fake):
    _call(num_k=4)
    _call(num_k=8)
    _call(num_k=4, kind="gpu")
    assert len(fake.made) == 3 and len(gradient._problems) == 2
    _call(num_k=4)          # evicted earlier: built again
    assert len(fake.made) == 4
