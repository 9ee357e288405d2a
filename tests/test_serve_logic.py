"""Server scheduling on the CPU with a fake device backend (no GPU).

Covers continuous batching (requests of several classes in flight at once,
later arrivals admitted as lanes free up), the HBM budget (lanes created only
while they fit, idle lanes of other classes evicted), refusals (too many
particles, a class that cannot fit), failures that are reported and not
retried, drain deadlines, and latency accounting.
"""
import numpy as np
import pytest

from gbpowspec.serve import Request, Result, Server, percentiles


class FakeClock:
    def __init__(self):
        self.t = 0.0

    def __call__(self):
        return self.t


class FakeLane:
    def __init__(self, key):
        self.key = key
        self.req = None
        self.polls_left = 0
        self.closed = False


class FakeBackend:
    """Each request finishes after `work` polls; lane bytes depend on the mesh."""

    def __init__(self, work=2, fail_start=()):
        self.work = work
        self.fail_start = set(fail_start)
        self.created = []
        self.started = []
        self.max_concurrent = 0

    def lane_bytes(self, req, capacity):
        return req.n_mesh ** 3 * 10

    def create(self, req, capacity):
        lane = FakeLane(req.key())
        self.created.append(lane)
        return lane

    def destroy(self, lane):
        lane.closed = True

    def start(self, lane, req):
        if req.ticket in self.fail_start:
            raise RuntimeError("injected launch failure")
        lane.req = req
        lane.polls_left = self.work
        self.started.append(req.ticket)
        busy = sum(1 for l in self.created if l.req is not None and not l.closed)
        self.max_concurrent = max(self.max_concurrent, busy)

    def finished(self, lane):
        lane.polls_left -= 1
        return lane.polls_left <= 0

    def result(self, lane, req):
        lane.req = None
        return Result(req.ticket, pk=np.full((3, 3), float(req.ticket)), n_kept=req.n)


def _req(n_mesh, n=100, mas="cic"):
    a = np.zeros(n, np.float32)
    return Request(a, a, a, box=100.0, n_mesh=n_mesh, mas=mas)


def test_continuous_batching_mixes_classes_and_admits_late_arrivals():
    be = FakeBackend(work=3)
    srv = Server(budget_bytes=1e12, lanes_per_class=2, capacity=1000, backend=be, clock=FakeClock())
    tickets = [srv.submit(_req(16 if i % 2 else 32)) for i in range(6)]
    assert srv.in_flight() == 4                       # 2 lanes x 2 classes; 2 requests wait
    late = srv.submit(_req(8))                        # a third class starts at once
    assert srv.in_flight() == 5
    res = srv.drain(timeout=1e9)
    assert sorted(r.ticket for r in res) == sorted(tickets + [late])
    assert all(r.error is None for r in res)
    assert all(r.pk[0, 0] == r.ticket for r in res)
    assert be.max_concurrent == 5
    assert len(be.created) == 5                       # lanes are reused, not re-created


def test_budget_limits_lanes_and_evicts_idle_lanes_of_other_classes():
    be = FakeBackend(work=1)
    # one 32^3 lane = 327,680 bytes; the budget holds one such lane, or a 16^3 lane (40,960) next to nothing else
    srv = Server(budget_bytes=330_000, lanes_per_class=4, capacity=1000, backend=be, clock=FakeClock())
    a = [srv.submit(_req(32)) for _ in range(3)]
    assert srv.in_flight() == 1 and srv.used == 327_680    # a second 32^3 lane does not fit
    res = srv.drain(timeout=1e9)
    assert sorted(r.ticket for r in res) == a and all(r.error is None for r in res)
    b = srv.submit(_req(16))                           # needs memory: the idle 32^3 lane is evicted
    assert be.created[0].closed and srv.used == 40_960
    res = srv.drain(timeout=1e9)
    assert [r.ticket for r in res] == [b] and res[0].error is None


def test_refusals_are_results_not_exceptions():
    be = FakeBackend()
    srv = Server(budget_bytes=1e5, lanes_per_class=1, capacity=50, backend=be, clock=FakeClock())
    big = srv.submit(_req(8, n=51))                    # more particles than any lane holds
    huge = srv.submit(_req(32, n=10))                  # one lane of 32^3 exceeds the budget
    res = {r.ticket: r for r in srv.drain(timeout=1e9)}
    assert "capacity" in res[big].error
    assert "budget" in res[huge].error
    again = srv.submit(_req(32, n=10))                 # the class stays refused
    assert "budget" in srv.drain(timeout=1e9)[0].error
    assert be.created == []


def test_launch_failure_is_reported_once_and_the_lane_is_reused():
    be = FakeBackend(work=1, fail_start={1})
    srv = Server(budget_bytes=1e12, lanes_per_class=1, capacity=1000, backend=be, clock=FakeClock())
    t = [srv.submit(_req(8)) for _ in range(3)]
    res = {r.ticket: r for r in srv.drain(timeout=1e9)}
    assert "injected" in res[1].error
    assert res[0].error is None and res[2].error is None
    assert be.started.count(1) == 0 and len(be.created) == 1


def test_drain_deadline_reports_timeouts():
    clk = FakeClock()
    be = FakeBackend(work=10 ** 9)
    srv = Server(budget_bytes=1e12, lanes_per_class=1, capacity=1000, backend=be, clock=clk)
    a, b = srv.submit(_req(8)), srv.submit(_req(8))

    def tick():
        clk.t += 1.0
        return clk.t
    srv.clock = tick
    res = srv.drain(timeout=5.0)
    assert sorted(r.ticket for r in res) == [a, b]
    assert all(r.error == "timed out" for r in res)


def test_latency_is_arrival_to_result():
    clk = FakeClock()
    be = FakeBackend(work=1)
    srv = Server(budget_bytes=1e12, lanes_per_class=1, capacity=1000, backend=be, clock=clk)
    srv.submit(_req(8))
    clk.t = 2.5
    srv.submit(_req(8))                                # waits for the lane
    clk.t = 4.0
    r1 = srv.poll()                                    # first finishes, second starts
    clk.t = 7.0
    r2 = srv.poll()
    assert [r.latency for r in r1] == [4.0]
    assert [r.latency for r in r2] == [4.5]
    p = percentiles([1.0, 2.0, 3.0, 4.0])
    assert p["p50"] == pytest.approx(2.5) and p["p99"] == pytest.approx(3.97)
