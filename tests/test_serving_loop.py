"""Host logic of the continuous-batching serving loop (no GPU): Poisson
arrivals, admission into a fixed number of slots, slots freed on completion
and reused, batched steps against one call per proposal, and each chain's
trace being the same in the mix as alone."""
import threading
import time

import numpy as np

from mctomo_gb300 import serving


class FakeBackend:
    """-log L is a fixed function of the model; a call takes `delay` s."""

    def __init__(self, nslots, delay=0.002):
        self.nslots, self.delay = nslots, delay
        self.calls = []
        self.lock = threading.Lock()

    def new_model(self, rng):
        return rng.random(3)

    def propose(self, rng, model):
        return model + rng.normal(0.0, 0.1, 3)

    def forward(self, slots, models):
        assert len(set(slots)) == len(slots)
        assert all(0 <= s < self.nslots for s in slots)
        with self.lock:
            self.calls.append(list(slots))
        time.sleep(self.delay)
        return np.array([float(np.sum((m - 0.5) ** 2) * 50.0) for m in models])

    def commit(self, slots, accept):
        assert len(slots) == len(accept)


def test_poisson_arrivals_rate_and_kinds():
    rng = np.random.default_rng(0)
    arr = serving.poisson_arrivals(rng, 40.0, 200.0, ["a", "b", "c"])
    assert abs(len(arr) / 200.0 - 40.0) < 2.0
    ts = [t for t, _ in arr]
    assert ts == sorted(ts) and ts[-1] < 200.0
    kinds = [k for _, k in arr]
    for k in "abc":
        assert abs(kinds.count(k) / len(kinds) - 1 / 3) < 0.03


def run(kinds_slots, arrivals, proposals, plain=False, duration=2.0):
    workers = [serving.Worker(k, FakeBackend(n), proposals, plain=plain) for k, n in kinds_slots]
    stats, chains = serving.run_stream(workers, arrivals, duration, (0.0, duration), seed=5, until_done=True)
    return stats, chains, workers


def test_slots_admission_completion_and_reuse():
    rng = np.random.default_rng(1)
    arrivals = serving.poisson_arrivals(rng, 60.0, 0.5, ["a", "b"])
    stats, chains, workers = run([("a", 3), ("b", 2)], arrivals, proposals=6)
    assert len(chains) == len(arrivals) > 10
    for w in workers:
        # never more chains in a step than slots, and slots were reused
        assert max(len(c) for c in w.backend.calls) <= w.backend.nslots
        assert len(w.done) == stats["kinds"][w.kind]["arrived"] > w.backend.nslots
    for ch in chains:
        assert ch.t_done is not None and ch.t_admit >= ch.t_arrive and ch.nprop == 6
        assert len(ch.trace) == 7                      # starting model + 6 proposals
    assert stats["evals"] == sum(len(c) for w in workers for c in w.backend.calls)
    assert stats["latency_p99_ms"] >= stats["latency_p50_ms"] > 0


def test_each_chain_is_the_same_alone_in_the_mix_and_plain():
    rng = np.random.default_rng(2)
    arrivals = serving.poisson_arrivals(rng, 80.0, 0.3, ["a", "b"])
    _, mix, _ = run([("a", 4), ("b", 3)], arrivals, proposals=8)
    _, plain, _ = run([("a", 4), ("b", 3)], arrivals, proposals=8, plain=True)
    for ch, pc in zip(mix, plain):
        assert ch.trace == pc.trace
    # alone: one chain with the same id (hence seed) in an empty system
    for ch in mix[:5]:
        w = serving.Worker(ch.kind, FakeBackend(1), 8)
        w.start()
        alone = serving.Chain(ch.cid, ch.kind, time.perf_counter(), 5 * 1000003 + ch.cid)
        w.submit(alone)
        t0 = time.time()
        while alone.t_done is None and time.time() - t0 < 10:
            time.sleep(0.001)
        w.stop.set(); w.join()
        assert alone.trace == ch.trace
