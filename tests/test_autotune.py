"""Autotuner logic on the CPU: signatures, candidate sets, choice and cache
(the GPU timing call is replaced by a fake engine)."""
from beguidedoff_gb300 import autotune as A


class FakePlan:
    def __init__(self):
        self.tunings = []

    def set_tuning(self, *t):
        self.tunings.append(tuple(t))

    def families(self):
        import numpy as np
        return np.zeros(0, dtype=np.int32)


class FakeEngine:
    def __init__(self, times):
        self.times = times
        self.calls = []

    def scan_time(self, plan, strands, ne, k, mode, reps, stream=None):
        tune = plan.tunings[-1]
        self.calls.append((mode, tune))
        return self.times[(mode, tune)]


def test_signature_rounds_counts_and_ignores_order():
    a = A.signature(["NGG"] * 100 + ["nrn"] * 3, 5)
    b = A.signature(["NRN"] * 4 + ["NGG"] * 120, 5)
    assert a == b == (5, ("NGG", 128), ("NRN", 4))
    assert A.signature(["NGG"], 4) != A.signature(["NGG"], 5)


def test_candidates_respect_limits():
    names = [c[0] for c in A.candidates_for(4, 1)]
    assert "all-guides" in names and not any("per-family" in n for n in names)
    assert [c[1] for c in A.candidates_for(9, 3)] == [1]
    assert any(c[2][3] == 1 for c in A.candidates_for(5, 3))


def test_choose_picks_fastest_and_caches():
    times = {(m, t): 10.0 + i for i, (_, m, t) in enumerate(A.CANDIDATES)}
    fast = A.CANDIDATES[2]
    times[(fast[1], fast[2])] = 1.0
    eng = FakeEngine(times)
    tuner = A.Autotuner(eng, [], [], 1000)
    tuner._strands = [object(), object()]
    plan = FakePlan()
    ch = tuner.choose(plan, ["NGG", "NRN"], 5)
    assert (ch.mode, ch.tuning, ch.name) == (fast[1], fast[2], fast[0])
    assert plan.tunings[-1] == fast[2]
    assert len(ch.times_ms) == len(A.candidates_for(5, 2))
    n = len(eng.calls)
    plan2 = FakePlan()
    ch2 = tuner.choose(plan2, ["NRN", "NGG"], 5)
    assert ch2 is ch and len(eng.calls) == n and plan2.tunings == [fast[2]]
    assert ch.as_dict()["tuning"]["split_families"] == fast[2][3]


def test_coarse_signature_classes():
    assert A.coarse_signature(1, 4) == (4, 0)
    assert A.coarse_signature(16, 4) == (4, 0)
    assert A.coarse_signature(17, 4) == (4, 1)
    assert A.coarse_signature(300, 5) == (5, 3)
    assert A.coarse_signature(5000, 3) == (3, 4)
