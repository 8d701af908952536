"""Serving loop on the GPU: every request's table is the one search() gives
it alone, while requests arrive during other batches and share launches."""
import threading
import time

import numpy as np
import pytest

from _golden import rows_equal
from _keys import table_rows
from beguidedoff_gb300 import _native, build
from beguidedoff_gb300.finder import beguidedoff
from beguidedoff_gb300.serving import SearchServer
from beguidedoff_gb300.types import GuideInput

pytestmark = pytest.mark.gpu

PAMS = ["NGG", "NG", "NNGRRT", "NNNRRT", "NRN"]
EDITORS = [("ABE", 4, 8), ("CBE", 3, 9), ("CGE", 5, 8)]


@pytest.fixture(scope="module", autouse=True)
def _lib():
    build.build()
    assert _native.device_count() >= 1


def _genome():
    lens = [1_500_000, 700_001, 900_000]
    g = _native.synth_genome(23, lens, [(100_000, 104_000)], thresholds=(76, 128, 180),
                             repeats={"n_families": 3, "family_len": 300, "n_copies": 300,
                                      "divergence": 0.1, "seed": 4})
    return g


def _requests(g, rng, n):
    fams = g["repeat_families"]
    reqs = []
    for i in range(n):
        k = int(rng.integers(3, 6))
        m = int(np.exp(rng.uniform(0, np.log(40))))
        guides = []
        for j in range(m):
            if rng.random() < 0.4:
                fam = fams[int(rng.integers(0, len(fams)))]
                p = int(rng.integers(0, len(fam) - 26))
                seq = fam[p:p + 20]
            else:
                seq = "".join(rng.choice(list("ACGT"), 20))
            ed, a, b = EDITORS[int(rng.integers(0, 3))]
            guides.append(GuideInput(f"q{i}_{j % 7}", seq, PAMS[int(rng.integers(0, 5))],
                                     "3prime", a, b, ed, base_editor=ed))
        kw = {}
        if rng.random() < 0.3:
            kw["return_all"] = True
        if rng.random() < 0.5:
            kw["count_score_threshold"] = float(rng.choice([1.0, 4.0, 15.0]))
        reqs.append((guides, k, kw))
    return reqs


def test_requests_equal_alone_and_in_the_mix():
    g = _genome()
    rng = np.random.default_rng(8)
    reqs = _requests(g, rng, 24)
    # an unknown editor fails only its own request
    bad = [GuideInput("bad", "ACGT" * 5, "NGG", "3prime", 4, 8, "XBE")]
    with SearchServer(genome_data=g, n_slots=2, memory_bytes=64 << 20,
                      max_batch_guides=60) as srv:
        futs = []

        def client(part):
            for guides, k, kw in part:
                futs.append((guides, k, kw, srv.submit(guides, k, **kw)))
                time.sleep(0.004)

        threads = [threading.Thread(target=client, args=(reqs[i::3],)) for i in range(3)]
        for t in threads:
            t.start()
        bad_fut = srv.submit(bad, 4)
        for t in threads:
            t.join()
        results = [(guides, k, kw, f.result(timeout=300)) for guides, k, kw, f in futs]
        with pytest.raises(ValueError):
            bad_fut.result(timeout=300)
        batches = list(srv.batches)
    assert any(b["requests"] > 1 for b in batches), batches
    alone = {k: beguidedoff(None, max_mismatches=k, genome_data=g) for k in (3, 4, 5)}
    try:
        n_rows = 0
        for guides, k, kw, got in results:
            exp = alone[k].search(guides=guides, verbose=False, **kw)
            ok, why = rows_equal(table_rows(got), table_rows(exp))
            assert ok, (k, kw, why)
            n_rows += len(table_rows(exp))
        assert n_rows > 50
    finally:
        for f in alone.values():
            f.close()


def test_plans_created_and_destroyed_on_two_streams_at_once():
    """Two threads, each with its own engine and stream, create, scan and
    destroy plans in a loop while the other's scans run (plan memory comes
    from the library's pool; destroy waits for the plan's own last use only):
    every scan returns the keys of the same plan scanned alone."""
    g = _genome()
    f = beguidedoff(None, max_mismatches=4, genome_data=g)
    try:
        rng = np.random.default_rng(5)
        sets = []
        for t in range(2):
            seqs = ["".join(rng.choice(list("ACGT"), 20)) for _ in range(24 + 8 * t)]
            pams = [PAMS[i % len(PAMS)] for i in range(len(seqs))]
            sets.append((seqs, pams))
        expected = []
        for seqs, pams in sets:
            plan = f._plan(seqs, pams)
            expected.append(f._engine.scan(plan, f._strands, [0, 3], 4, 2))
            plan.close()
        errors = []

        def worker(t):
            eng = _native.Engine(0)
            st = _native.Stream(0)
            try:
                seqs, pams = sets[t]
                for it in range(12):
                    plan = f._plan(seqs, pams, eng, st.handle)
                    plan.set_tuning(1024 if it % 2 else 0, 0, 0, 0, 1 if it % 3 else 3,
                                    it % 2)
                    keys = eng.scan(plan, f._strands, [0, 3], 4, 2, st.handle)
                    plan.close()
                    if not np.array_equal(keys, expected[t]):
                        errors.append((t, it))
            except Exception as exc:  # reported by the main thread
                errors.append((t, repr(exc)))
            finally:
                st.close()
                eng.close()

        threads = [threading.Thread(target=worker, args=(t,)) for t in range(2)]
        for th in threads:
            th.start()
        for th in threads:
            th.join()
        assert not errors, errors
    finally:
        f.close()
