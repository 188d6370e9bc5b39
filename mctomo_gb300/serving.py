"""Continuous-batching serving loop over likelihood contexts (host side).

The reference's sampler evaluates one proposal per likelihood call and has
no serving layer; this module is the request loop around the batched
contexts for a stream of independent chains of mixed problem shapes:

* chains arrive as a Poisson stream (`poisson_arrivals`); each has a kind
  (its problem shape) and its own random stream for proposals and the
  Metropolis decisions, so its trace depends only on its likelihoods;
* each kind has a `Worker` thread owning a backend (one or more device
  contexts) with a fixed number of chain slots, which is the kind's share of
  the device memory: a chain waits in its kind's queue until a slot is
  free, is admitted between two steps, and leaves after its proposals,
  freeing the slot for the next arrival;
* a batched worker evaluates the current proposal of every chain it holds
  in one forward per step (chains admitted meanwhile join the next step);
  a plain worker makes one call per proposal, as the reference's sampler
  does;
* workers run concurrently on their own CUDA streams, so the kinds'
  kernels overlap on the device.

A backend provides `nslots`, `new_model(rng)`, `propose(rng, model)`,
`forward(slots, models) -> -log L per chain` and `commit(slots, accept)`.
The per-proposal latency is the time from a proposal's submission to its
result; the admission wait is the time from a chain's arrival to its first
step.
"""
import collections
import heapq
import math
import threading
import time

import numpy as np


def poisson_arrivals(rng, rate, duration, kinds):
    """Arrival times (s, from 0) of a Poisson stream of the given rate over
    duration, each with a kind drawn uniformly from kinds."""
    t, out = 0.0, []
    while True:
        t += rng.exponential(1.0 / rate)
        if t >= duration:
            return out
        out.append((t, kinds[int(rng.integers(len(kinds)))]))


class Chain:
    __slots__ = ("cid", "kind", "rng", "t_arrive", "t_admit", "t_done", "slot", "model", "like", "nprop",
                 "trace")

    def __init__(self, cid, kind, t_arrive, seed):
        self.cid, self.kind, self.t_arrive = cid, kind, t_arrive
        self.rng = np.random.default_rng(seed)
        self.t_admit = self.t_done = None
        self.slot = -1
        self.model = None
        self.like = math.inf
        self.nprop = 0
        self.trace = []


class Worker(threading.Thread):
    """One kind's request loop. proposals: proposals per chain before it
    leaves; plain: one forward call per proposal instead of one per step."""

    def __init__(self, kind, backend, proposals, plain=False, clock=time.perf_counter):
        super().__init__(daemon=True, name="serve-" + kind)
        self.kind, self.backend, self.proposals, self.plain = kind, backend, proposals, plain
        self.clock = clock
        self.queue = collections.deque()
        self.lock = threading.Lock()
        self.stop = threading.Event()
        self.free = list(range(backend.nslots))      # a min-heap: the lowest free slot first
        self.active = []
        self.done = []
        self.latency = []      # (t_result, seconds) per evaluated proposal
        self.evals = []        # (t_result, count) per forward call
        self.error = None

    def submit(self, chain):
        with self.lock:
            self.queue.append(chain)

    def _admit(self):
        with self.lock:
            while self.free and self.queue:
                ch = self.queue.popleft()
                ch.slot = heapq.heappop(self.free)
                ch.t_admit = self.clock()
                ch.model = self.backend.new_model(ch.rng)
                self.active.append(ch)

    def _step(self, chains):
        """One forward of the chains' current proposals (a new chain's first
        step evaluates its starting model, which becomes its state)."""
        models = [ch.model if ch.nprop == 0 and not ch.trace else self.backend.propose(ch.rng, ch.model)
                  for ch in chains]
        t0 = self.clock()
        like = self.backend.forward([ch.slot for ch in chains], models)
        t1 = self.clock()
        accept = np.zeros(len(chains), np.int32)
        for i, ch in enumerate(chains):
            first = ch.nprop == 0 and not ch.trace
            u = ch.rng.random()
            if first or math.log(u) < ch.like - like[i]:
                accept[i] = 1
                ch.model = models[i]
                ch.like = float(like[i])
            ch.trace.append(ch.like)
            if not first:
                ch.nprop += 1
            self.latency.append((t1, t1 - t0))
        self.evals.append((t1, len(chains)))
        self.backend.commit([ch.slot for ch in chains], accept)
        for ch in chains:
            if ch.nprop >= self.proposals:
                ch.t_done = t1
                self.active.remove(ch)
                self.done.append(ch)
                with self.lock:
                    heapq.heappush(self.free, ch.slot)

    def run(self):
        try:
            while not self.stop.is_set():
                self._admit()
                if not self.active:
                    time.sleep(0.0005)
                    continue
                if self.plain:
                    for ch in list(self.active):
                        if self.stop.is_set():
                            break
                        self._step([ch])
                else:
                    self._step(list(self.active))
        except Exception as e:   # reported by the driver
            self.error = e


def run_stream(workers, arrivals, duration, window, seed=0, clock=time.perf_counter, until_done=False):
    """Feeds the arrivals (time, kind) to the workers in real time for
    duration seconds (or, with until_done, until every chain has finished,
    at most duration) and stops them. Statistics are taken over [window[0],
    window[1]] seconds after the start. Returns (stats, chains)."""
    by_kind = {w.kind: w for w in workers}
    for w in workers:
        w.start()
    t_start = clock()
    chains = []
    for i, (t, kind) in enumerate(arrivals):
        now = clock() - t_start
        if t > now:
            time.sleep(t - now)
        ch = Chain(i, kind, t_start + t, seed * 1000003 + i)
        chains.append(ch)
        by_kind[kind].submit(ch)
        if any(w.error for w in workers):
            break
    while clock() - t_start < duration:
        if until_done and all(ch.t_done is not None for ch in chains):
            break
        if any(w.error for w in workers):
            break
        time.sleep(min(0.01, max(0.0, duration - (clock() - t_start))))
    for w in workers:
        w.stop.set()
    for w in workers:
        w.join()
    for w in workers:
        if w.error:
            raise w.error
    a, b = t_start + window[0], t_start + window[1]
    stats = {"window_s": window[1] - window[0], "kinds": {}}
    all_lat, all_ev = [], 0
    for w in workers:
        lat = [s for (t, s) in w.latency if a <= t <= b]
        ev = sum(n for (t, n) in w.evals if a <= t <= b)
        adm = [ch.t_admit - ch.t_arrive for ch in chains if ch.kind == w.kind and ch.t_admit and a <= ch.t_admit <= b]
        stats["kinds"][w.kind] = {
            "slots": w.backend.nslots, "evals": ev, "evals_per_s": ev / (b - a),
            "latency_p50_ms": _pct(lat, 50), "latency_p99_ms": _pct(lat, 99),
            "arrived": sum(1 for ch in chains if ch.kind == w.kind),
            "admitted": sum(1 for ch in chains if ch.kind == w.kind and ch.t_admit is not None),
            "completed": len(w.done),
            "admission_wait_p50_ms": _pct(adm, 50), "admission_wait_p99_ms": _pct(adm, 99)}
        all_lat += lat
        all_ev += ev
    stats["evals"] = all_ev
    stats["evals_per_s"] = all_ev / (b - a)
    stats["latency_p50_ms"] = _pct(all_lat, 50)
    stats["latency_p99_ms"] = _pct(all_lat, 99)
    return stats, chains


def _pct(x, q):
    return round(float(np.percentile(np.asarray(x) * 1e3, q)), 3) if len(x) else None


# ---------------------------------------------------------------------------
# Backends over the likelihood contexts. A model is (ncells, points, params)
# of one chain, padded to the context's ncell_max. single = True maps every
# chain onto the context's slot 0 (one chain per call: the plain drop-in).
# ---------------------------------------------------------------------------
class _SlotBackend:
    def __init__(self, nslots, new_model, propose, single):
        self.nslots, self._new, self._propose, self.single = nslots, new_model, propose, single

    def new_model(self, rng):
        return self._new(rng)

    def propose(self, rng, model):
        return self._propose(rng, model)

    def _pack(self, slots, models):
        """Arrays over the context's chains 0..m-1 (the body and 2D contexts
        evaluate a leading range of slots): a slot outside this call keeps
        the last model it was given, whose result is not used."""
        m = 1 if self.single else max(slots) + 1
        if not hasattr(self, "_last"):
            nc, p, q = models[0]
            self._last = [(nc, p, q)] * (1 if self.single else self.nslots)
        idx = [0 if self.single else s for s in slots]
        for i, mdl in zip(idx, models):
            self._last[i] = mdl
        nc = np.array([self._last[i][0] for i in range(m)], np.int32)
        pts = np.stack([self._last[i][1] for i in range(m)])
        par = np.stack([self._last[i][2] for i in range(m)])
        return m, idx, nc, pts, par


class TT2DBackend(_SlotBackend):
    """The 2D travel-time context; n1 is the noise level of every chain."""

    def __init__(self, ctx, nslots, new_model, propose, n1=0.05, single=False):
        super().__init__(nslots, new_model, propose, single)
        self.ctx, self.n1 = ctx, n1

    def set_priority(self, high):
        self.ctx.set_priority(high)

    def set_sm_share(self, share):
        self.ctx.set_sm_share(share)

    def forward(self, slots, models):
        assert not self.single or len(models) == 1
        m, idx, nc, pts, par = self._pack(slots, models)
        o = self.ctx.forward(nc, pts, par, np.zeros((m, 2)), np.full((m, 2), self.n1))
        return o[idx, 0]

    def commit(self, slots, accept):
        m = 1 if self.single else max(slots) + 1
        acc = np.zeros(m, np.int32)
        for s, a in zip(slots, accept):
            acc[0 if self.single else s] = a
        self.ctx.commit(acc)


class BodyBackend(TT2DBackend):
    """The 3D body-wave context; locations: (nsrc, 4) events of every chain."""

    def __init__(self, ctx, nslots, new_model, propose, locations, n1=0.05, single=False):
        super().__init__(ctx, nslots, new_model, propose, n1, single)
        self.loc = np.asarray(locations, np.float64)

    def forward(self, slots, models):
        assert not self.single or len(models) == 1
        npd = self.ctx.np
        m, idx, nc, pts, par = self._pack(slots, models)
        o = self.ctx.forward(nc, pts, par, np.repeat(self.loc[None], m, 0), np.zeros((m, npd)),
                             np.full((m, npd), self.n1))
        return o[idx, 0]


class SurfaceBackend(_SlotBackend):
    """The surface-wave context (explicit slots); sigma = n0 * time."""

    def __init__(self, ctx, nslots, new_model, propose, nperiods, n0=0.02, single=False):
        super().__init__(nslots, new_model, propose, single)
        self.ctx, self.npd, self.n0 = ctx, nperiods, n0

    def _args(self, slots, models):
        k = len(models)
        sl = np.zeros(k, np.int32) if self.single else np.asarray(slots, np.int32)
        nc = np.array([m[0] for m in models], np.int32)
        pts = np.stack([m[1] for m in models]); par = np.stack([m[2] for m in models])
        return sl, nc, pts, par, np.full((k, self.npd), self.n0), np.zeros((k, self.npd))

    def forward(self, slots, models):
        assert not self.single or len(models) == 1
        return self.ctx.forward(*self._args(slots, models))[:, 0]

    def set_priority(self, high):
        self.ctx.set_priority(high)

    def set_sm_share(self, share):
        self.ctx.set_sm_share(share)

    def submit(self, slots, models):
        self.ctx.submit(*self._args(slots, models))

    def poll_wait(self):
        done, out = self.ctx.poll()
        while not done:
            time.sleep(0.0002)
            done, out = self.ctx.poll()
        return out[:, 0]

    def commit(self, slots, accept):
        # accept / reject each proposal of the last forward, in its order
        self.ctx.commit(np.asarray(accept, np.int32))


class JointBackend:
    """Joint surface + body chains: one model on both contexts, -log L the
    sum; the surface forward runs asynchronously beside the body forward."""

    def __init__(self, surface, body):
        self.s, self.b = surface, body
        self.nslots = min(surface.nslots, body.nslots)

    def set_priority(self, high):
        self.s.set_priority(high)
        self.b.set_priority(high)

    def new_model(self, rng):
        return self.b.new_model(rng)

    def propose(self, rng, model):
        return self.b.propose(rng, model)

    def forward(self, slots, models):
        self.s.submit(slots, models)
        lb = self.b.forward(slots, models)
        return self.s.poll_wait() + lb

    def commit(self, slots, accept):
        self.s.commit(slots, accept)
        self.b.commit(slots, accept)
