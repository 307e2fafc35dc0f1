"""The serving loop's host logic against a host-only backend: every request
completes once, compatible requests share launches within the set cap,
launches never exceed the memory budget, latency is completion - arrival,
and the plain mode serves one request per launch."""
import numpy as np

from tskit_gb300.serve import Request, Server, poisson_requests


class FakeTS:
    def __init__(self, n, L=1e6):
        self._s = np.arange(n)
        self.sequence_length = L
        self.num_samples = n

    def samples(self):
        return self._s


class FakeClock:
    def __init__(self):
        self.t = 0.0

    def __call__(self):
        self.t += 1e-5
        return self.t


class FakeBackend:
    """Completes a launch 2 ms (virtual) after it starts; workspace bytes
    proportional to the number of sets and windows."""

    def __init__(self, clock, resident):
        self.clock = clock
        self.resident = resident
        self.launched = []
        self.inflight_bytes = []
        self.live = {}

    def max_sets(self, key):
        return 8 if self.resident[key].num_samples <= 65535 else 4

    def output_bytes(self, r):
        nwin = 1 if r.windows is None else len(r.windows) - 1
        if r.kind == "rv":
            return nwin * self.resident[r.ts].num_samples * r.weights.shape[1] * 8
        return nwin * 8

    def workspace_bytes(self, groups):
        return 1000 * sum(1 + len(r.sample_sets) for g in groups for r in g)

    def discard(self, groups):
        pass

    def launch(self, groups, slot):
        reqs = [r for g in groups for r in g]
        w = {"reqs": reqs, "groups": groups, "t": self.clock.t, "slot": slot,
             "bytes": self.workspace_bytes(groups)}
        self.live[slot] = w["bytes"]
        self.inflight_bytes.append(sum(self.live.values()))
        self.launched.append(w)
        return w

    def ready(self, w):
        ok = self.clock.t >= w["t"] + 2e-3
        if ok:
            self.live.pop(w["slot"], None)
        return ok

    def wait(self, w):
        self.clock.t = max(self.clock.t, w["t"] + 2e-3)

    def results(self, w):
        return {r.rid: ("done", r.rid) for r in w["reqs"]}


def _stream(num=300, rate=20000.0, seed=1):
    resident = {"a": FakeTS(1000), "b": FakeTS(100000)}
    return resident, poisson_requests(resident, num, rate, seed, window_choices=(1, 10))


def test_all_requests_complete_once_and_batch():
    resident, reqs = _stream()
    clock = FakeClock()
    be = FakeBackend(clock, resident)
    st = Server(be, num_slots=4, hbm_budget=10 ** 9).run(reqs, clock=clock)
    assert st.num == len(reqs)
    assert sorted(st.results) == sorted(r.rid for r in reqs)
    assert all(st.results[r.rid] == ("done", r.rid) for r in reqs)
    assert np.all(st.latencies_s > 0)
    assert st.launches < len(reqs)  # batching happened
    assert st.fused_queries == sum(len(w["groups"]) for w in be.launched)
    assert any(len({g[0].ts for g in w["groups"]}) > 1 for w in be.launched)  # across sequences
    for w in be.launched:
        assert 1 <= len(w["groups"]) <= 8
        for rs in w["groups"]:
            keys = {r.batch_key() for r in rs}
            assert len(keys) == 1
            if rs[0].kind == "counts":
                assert sum(len(r.sample_sets) for r in rs) <= be.max_sets(rs[0].ts)
            if rs[0].kind == "afs":
                assert len(rs) == 1


def test_memory_budget_respected():
    resident, reqs = _stream(num=200, seed=2)
    clock = FakeClock()
    be = FakeBackend(clock, resident)
    budget = 12000
    Server(be, num_slots=8, hbm_budget=budget).run(reqs, clock=clock)
    # a single launch may exceed the budget only when it runs alone
    for b, w in zip(be.inflight_bytes, be.launched):
        assert b <= budget or b == w["bytes"]


def test_plain_mode_one_request_per_launch():
    resident, reqs = _stream(num=50, seed=3)
    clock = FakeClock()
    be = FakeBackend(clock, resident)
    st = Server(be, num_slots=4).run(reqs, mode="plain", clock=clock)
    assert st.launches == len(reqs)
    assert all(len(w["reqs"]) == 1 and len(w["groups"]) == 1 for w in be.launched)


def test_oversized_requests_rejected_and_counted():
    resident = {"a": FakeTS(1000), "b": FakeTS(100000)}
    reqs = poisson_requests(resident, 300, 20000.0, 6, window_choices=(1, 10, 100, 1000))
    clock = FakeClock()
    be = FakeBackend(clock, resident)
    cap = 64 << 20
    st = Server(be, num_slots=4, max_output_bytes=cap).run(reqs, clock=clock)
    over = {r.rid for r in reqs if be.output_bytes(r) > cap}
    assert over and all(r.kind == "rv" for r in reqs if r.rid in over)
    assert set(st.rejected) == over
    assert st.num == len(reqs) - len(over) == len(st.results) == len(st.latencies_s)
    assert not over & set(st.results)
    # the requests keep the windows they were drawn with
    assert any(r.kind == "rv" and r.windows is not None and len(r.windows) == 1001
               for r in reqs)


def test_request_mix_shapes():
    resident, reqs = _stream(num=400, seed=4)
    for r in reqs:
        if r.stat in ("divergence", "Fst"):
            assert len(r.sample_sets) == 2
            assert not set(r.sample_sets[0]) & set(r.sample_sets[1])
        elif r.stat == "relatedness_vector":
            assert r.mode == "branch" and r.weights.shape[1] == 8
        else:
            assert len(r.sample_sets) == 1
        for s in r.sample_sets:
            assert 10 <= len(s) <= 10000
    arr = np.array([r.arrival for r in reqs])
    assert np.all(np.diff(arr) > 0)
