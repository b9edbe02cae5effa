"""Host-side logic without a GPU: the request stream, the continuous-batching
scheduler on a fake device backend, and the multi-rank (replica) reductions
of bench.py over two gloo ranks."""
import os
import socket
import sys

import numpy as np
import pytest

from conftest import REPO
from mhd_gb300 import serve
from mhd_gb300.serve import Request, Server, device_bytes_estimate, poisson_requests


def test_poisson_requests_are_reproducible_and_in_range():
    a = poisson_requests(50, rate=20.0, seed=3)
    b = poisson_requests(50, rate=20.0, seed=3)
    assert [(r.case.nPx, r.case.nPz, r.steps, r.precision, r.arrival) for r in a] == \
           [(r.case.nPx, r.case.nPz, r.steps, r.precision, r.arrival) for r in b]
    arr = np.array([r.arrival for r in a])
    assert np.all(np.diff(arr) > 0)
    assert all(32 <= r.case.nPx <= 256 and r.case.nPx == r.case.nPy and 32 <= r.case.nPz <= 128 for r in a)
    assert all(50 <= r.steps <= 2000 for r in a)
    assert all(1 / 3e-2 - 1e-9 <= r.case.RE <= 1 / 3e-3 + 1e-9 for r in a)
    assert {r.precision for r in a} == {"fp32", "fp64"}


class FakeSim:
    live = 0

    def __init__(self, case, precision="fp64", **kw):
        self.case, self.precision, self.steps_done, self.timt = case, precision, 0, 0.0
        FakeSim.live += 1

    def upload_state(self, st):
        pass

    def init_on_device(self):
        pass

    def communicate(self):
        pass

    def steps(self, n, dt=None):
        self.steps_done += n

    def sync(self):
        pass

    def download_state(self):
        return {"steps": self.steps_done}

    def close(self):
        FakeSim.live -= 1


class FakeBatch:
    def __init__(self, sims):
        self.sims = sims

    def autotune(self, report=True):
        return 1, [1.0, 0.5, 0.7]

    def set_tile(self, t):
        self.t = t

    def steps(self, n):
        for s in self.sims:
            s.steps_done += n

    def steps_limited(self, n, limits):
        for s, m in zip(self.sims, limits):
            s.steps_done += min(n, m)

    def autotune_bytes(self):
        return 0

    def zrange(self):
        return 32

    def set_zrange(self, z):
        self.z = z

    def sync(self):
        pass

    def close(self):
        pass


@pytest.fixture
def fake_backend(monkeypatch):
    monkeypatch.setattr(serve, "Simulation", FakeSim)
    monkeypatch.setattr(serve, "Batch", FakeBatch)
    monkeypatch.setattr(serve, "initial_state", lambda case: {})
    FakeSim.live = 0
    yield


def test_scheduler_admits_under_budget_and_completes_every_request(fake_backend):
    reqs = poisson_requests(40, rate=100.0, seed=1, grid_min=(16, 16, 8), grid_max=(64, 64, 32), steps=(3, 40))
    sizes = [device_bytes_estimate(r.case, r.precision) for r in reqs]
    budget = sum(sorted(sizes)[-3:])
    srv = Server(budget, quantum=5, keep_results=True)
    used_peak = [0]
    orig = srv._admit

    def spy(req, now):
        ok = orig(req, now)
        used_peak[0] = max(used_peak[0], srv.used)
        return ok
    srv._admit = spy
    st = srv.run(reqs, realtime=False)
    assert used_peak[0] <= budget
    assert FakeSim.live == 0 and srv.used == 0
    assert all(r.result["steps"] == r.steps for r in reqs)          # each ran exactly its step count
    assert all(r.t_done >= r.t_admit >= r.arrival for r in reqs)
    # no batch reached a quarter of the 64 M-cell target: the default tile, never tuned
    assert st["max_resident"] >= 2 and st["tile"] == serve.DEFAULT_TILE
    assert st["tts_p99_s"] >= st["tts_p50_s"] > 0


def test_server_tunes_the_tile_once_on_a_representative_batch(fake_backend, monkeypatch):
    tuned, tiles = [], []

    class CountingBatch(FakeBatch):
        def autotune(self, report=True):
            tuned.append(len(self.sims))
            tiles.append((len(self.sims), "tuned"))
            return super().autotune(report)

        def set_tile(self, t):
            tiles.append((len(self.sims), t))
            super().set_tile(t)
    monkeypatch.setattr(serve, "Batch", CountingBatch)
    reqs = poisson_requests(24, rate=1000.0, seed=5, grid_min=(32, 32, 16), grid_max=(32, 32, 16), steps=(20, 40),
                            fp32_fraction=0.0)
    cells = reqs[0].case.cells
    srv = Server(1 << 40, quantum=5, target_cells=16 * cells)        # tuned from 4 instances on
    st = srv.run(reqs, realtime=False)
    assert len(tuned) == 1 and tuned[0] >= 4
    k = tiles.index((tuned[0], "tuned"))
    assert k > 0 and all(t == serve.DEFAULT_TILE and n < 4 for n, t in tiles[:k])   # small batches first
    assert all(t == 1 for n, t in tiles[k + 1:]) and st["tile"] == 1                # the tuned shape from then on


def test_srpt_admits_least_work_first_and_caps_resident_cells(fake_backend):
    """With "srpt" the waiting request with the least work is admitted first
    and resident work stays near target_cells; every request still runs
    exactly its step count."""
    reqs = poisson_requests(30, rate=1e6, seed=3, grid_min=(16, 16, 8), grid_max=(64, 64, 32), steps=(3, 40))
    for r in reqs:
        r.arrival = 0.0
    target = 3 * max(r.case.cells for r in reqs)
    srv = Server(1 << 40, quantum=5, keep_results=True, policy="srpt", target_cells=target)
    order = []
    orig = srv._admit

    def spy(req, now):
        ok = orig(req, now)
        if ok:
            order.append(req)
            assert srv.resident_cells <= target + req.case.cells
        return ok
    srv._admit = spy
    st = srv.run(reqs, realtime=False)
    assert st["policy"] == "srpt" and FakeSim.live == 0 and srv.resident_cells == 0
    assert all(r.result["steps"] == r.steps for r in reqs)
    # all arrived at once: the first admissions are the least-work requests
    work = sorted(r.case.cells * r.steps for r in reqs)
    first = [r.case.cells * r.steps for r in order[:3]]
    assert first == work[:3]
    fifo = Server(1 << 40, quantum=5, policy="fifo").run(
        poisson_requests(30, rate=1e6, seed=3, grid_min=(16, 16, 8), grid_max=(64, 64, 32), steps=(3, 40)),
        realtime=False)
    assert fifo["policy"] == "fifo" and fifo["max_resident"] >= st["max_resident"]


def test_server_skips_a_tuning_whose_scratch_does_not_fit(fake_backend, monkeypatch):
    """The autotuner's scratch copy (24 doubles per cell here) counts against
    the budget: one resident simulation fits, it and the copy do not."""
    class SizedBatch(FakeBatch):
        def autotune_bytes(self):
            return sum(s.case.nx * s.case.ny * s.case.nz * 24 * 8 for s in self.sims)
    monkeypatch.setattr(serve, "Batch", SizedBatch)

    def stream():
        reqs = poisson_requests(4, rate=50.0, seed=13, grid_min=(32, 32, 16), grid_max=(32, 32, 16), steps=(3, 8),
                                fp32_fraction=0.0)
        for r in reqs:
            r.arrival = 0.0
        return reqs
    need = max(device_bytes_estimate(r.case, r.precision) for r in stream())
    st = Server(need + (1 << 20), quantum=4, target_cells=1).run(stream(), realtime=False)
    assert st["tune_skipped"] >= 1 and st["tile"] == serve.DEFAULT_TILE and st["zrange"]["fp64"] is None
    st2 = Server(3 * need, quantum=4, target_cells=1).run(stream(), realtime=False)
    assert st2["tune_skipped"] == 0 and st2["tile"] == 1 and st2["zrange"]["fp64"] == 32


def test_scheduler_rejects_a_request_larger_than_the_budget(fake_backend):
    big = Request(rid=0, case=poisson_requests(1, 1.0, seed=2)[0].case, steps=3)
    with pytest.raises(RuntimeError):
        Server(10, quantum=5).run([big], realtime=False)


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def _rank_main(rank, world, port, q):
    os.environ.update(RANK=str(rank), WORLD_SIZE=str(world), LOCAL_RANK=str(rank),
                      MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    sys.path.insert(0, str(REPO))
    import bench
    d = bench.Dist()
    d.barrier()
    m = d.max(float(rank + 1) * 1.5)
    d.close()
    q.put((rank, m))


def test_bench_replica_reductions_two_gloo_ranks():
    import multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    ps = [ctx.Process(target=_rank_main, args=(r, 2, port, q)) for r in range(2)]
    for p in ps:
        p.start()
    out = [q.get(timeout=120) for _ in ps]
    for p in ps:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert sorted(out) == [(0, 3.0), (1, 3.0)]


def test_device_initial_state_mirror_is_a_seeded_gaussian():
    from mhd_gb300.case import device_initial_state, small_cases, z_coordinate
    c = small_cases()["mhd_fixedT"].replace(nPx=32, nPy=32, nPz=16, seed=5)
    a, b = device_initial_state(c), device_initial_state(c)
    assert all(np.array_equal(a[k], b[k]) for k in a)
    t1 = 1 + c.THETA * z_coordinate(c)
    g = (a["TT"][1:-1, 1:-1, 1:-1] / t1[1:-1, None, None] - 1) / c.noise
    assert abs(g.mean()) < 0.02 and abs(g.std() - 1) < 0.02
    d = device_initial_state(c.replace(seed=6))
    assert not np.array_equal(a["TT"], d["TT"])
    # periodic ghosts
    assert np.array_equal(a["TT"][:, 0, :], a["TT"][:, -2, :]) and np.array_equal(a["TT"][:, :, -1], a["TT"][:, :, 1])


def test_quantum_does_not_shrink_to_the_shortest_request(fake_backend, monkeypatch):
    """A request with one step left takes that step and drops out of the
    quantum; the others still get the full quantum."""
    calls = []

    class RecordingBatch(FakeBatch):
        def steps_limited(self, n, limits):
            calls.append((n, list(limits)))
            super().steps_limited(n, limits)
    monkeypatch.setattr(serve, "Batch", RecordingBatch)
    reqs = poisson_requests(2, rate=1e6, seed=2, grid_min=(16, 16, 8), grid_max=(16, 16, 8), steps=(3, 3),
                            fp32_fraction=0.0)
    reqs[0].steps, reqs[1].steps = 1, 50
    for r in reqs:
        r.arrival = 0.0
    srv = Server(1 << 40, quantum=25, keep_results=True)
    srv.run(reqs, realtime=False)
    assert calls[0] == (25, [1, 50])
    assert [n for n, _ in calls] == [25, 25]
    assert [r.result["steps"] for r in reqs] == [1, 50]


def test_quanta_balance_the_precisions(fake_backend, monkeypatch):
    """With balance on, a batch whose steps are estimated to take a quarter
    of the time takes four times the steps per quantum (capped at 8 x
    quantum); without it every batch takes the quantum."""
    calls = []

    class RecordingBatch(FakeBatch):
        def steps_limited(self, n, limits):
            calls.append((self.sims[0].precision, n))
            super().steps_limited(n, limits)
    monkeypatch.setattr(serve, "Batch", RecordingBatch)

    def stream():
        reqs = poisson_requests(2, rate=1e6, seed=2, grid_min=(16, 16, 8), grid_max=(16, 16, 8), steps=(3, 3))
        reqs[0].precision, reqs[1].precision = "fp64", "fp32"
        for r in reqs:
            r.steps, r.arrival = 400, 0.0
        return reqs
    srv = Server(1 << 40, quantum=10, rates={"fp64": 1.0, "fp32": 4.0}, keep_results=True)
    reqs = stream()
    srv.run(reqs, realtime=False)
    first = dict(calls[:2])
    assert first == {"fp64": 10, "fp32": 40}
    assert [r.result["steps"] for r in reqs] == [400, 400]
    calls.clear()
    Server(1 << 40, quantum=10, balance=False).run(stream(), realtime=False)
    assert dict(calls[:2]) == {"fp64": 10, "fp32": 10}
