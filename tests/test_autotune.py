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


def test_candidate_tunings_are_valid_and_distinct():
    """Every candidate passes the C ABI's tuning rules (bgo_plan_set_tuning)
    and names a distinct form, for single launches and per family."""
    seen = set()
    for name, mode, tune in A.CANDIDATES:
        t = dict(zip(A.TUNING_FIELDS, tuple(tune) + (0,) * (len(A.TUNING_FIELDS) - len(tune))))
        assert mode in (1, 2, 3), name
        assert t["chunk_sites"] in (0, 1024, 2048) or (
            t["chunk_sites"] == 4096 and t["prefilter"] == 1), name
        assert t["prefilter"] in (0, 1), name
        assert not (t["prefilter"] and (t["tolerance"] != 1 or t["chunk_sites"] == 1024)), name
        assert t["group_guides"] in (0, 32, 64, 128), name
        assert t["split_families"] in (0, 1) and t["tolerance"] in (0, 1), name
        assert t["min_blocks"] in (0, 1, 2, 3, 4), name
        assert t["inline_entries"] in (0, 1, 2) and t["range_walk"] in (0, 1), name
        key = (mode, tuple(t.values()))
        assert key not in seen, name
        seen.add(key)
    fam_seen = set()
    for cand in A.FAMILY_CANDIDATES:
        name, form, chunk, minb, tol, inl, walk = cand[:7]
        pf = cand[7] if len(cand) > 7 else 0
        assert form in (0, 1) and minb in (0, 1, 2, 3, 4), name
        assert chunk in (0, 1024, 2048) or (chunk == 4096 and pf == 1), name
        assert tol in (0, 1) and inl in (0, 1, 2) and walk in (0, 1) and pf in (0, 1), name
        assert not (pf and (tol != 1 or chunk == 1024)), name
        assert (form, chunk, minb, tol, inl, walk, pf) not in fam_seen, name
        fam_seen.add((form, chunk, minb, tol, inl, walk, pf))


def test_per_family_choice_applies_each_familys_form():
    """A per-family choice sets split launches on the plan and each PAM
    family's own form; a family the choice does not know keeps the plan's
    defaults."""
    import numpy as np

    class Plan(FakePlan):
        def __init__(self):
            super().__init__()
            self.fam_calls = {}

        def families(self):
            return np.array([0, 1, 0, 2, -1], dtype=np.int32)

        def set_family_tuning(self, f, **kw):
            self.fam_calls[f] = kw

    fam = {"NGG": ("index/t1/cta768", 0, 0, 1, 1, 0, 0, 0.2),
           "NRN": ("every-guide", 1, 0, 0, 0, 0, 0, 0.5)}
    ch = A.Choice("per-family", 2, A.PER_FAMILY_TUNING, {}, 0, fam)
    plan = Plan()
    ch.apply(plan, ["NGG", "NRN", "ngg", "NNGRRT", "NG"])
    assert plan.tunings[-1] == A.PER_FAMILY_TUNING
    assert plan.fam_calls[0] == dict(chunk_sites=0, min_blocks=1, tolerance=1, form=0,
                                     inline_entries=0, range_walk=0, prefilter=0)
    assert plan.fam_calls[1]["form"] == 1
    assert 2 not in plan.fam_calls
