"""Continuous-batching server: requests admitted under an HBM budget while
others run, results identical alone and in the mix."""
import numpy as np
import pytest

from mhd_gb300.case import STATE_FIELDS
from mhd_gb300.serve import Request, Server, device_bytes_estimate, poisson_requests

pytestmark = pytest.mark.gpu


def small_stream(n=10, seed=5):
    return poisson_requests(n, rate=50.0, seed=seed, grid_min=(16, 16, 8), grid_max=(48, 48, 16),
                            steps=(3, 20), fp32_fraction=0.4)


def test_results_same_alone_and_in_mix():
    reqs = small_stream()
    budget = sum(device_bytes_estimate(r.case, r.precision) for r in reqs) // 2
    srv = Server(budget, quantum=4, tile=0, keep_results=True)
    stats = srv.run(reqs, realtime=False)
    assert stats["requests"] == len(reqs)
    assert stats["max_resident"] >= 2          # work overlapped on the device
    assert srv.admissions == len(reqs)
    for r in reqs:
        alone = Request(rid=r.rid, case=r.case, steps=r.steps, precision=r.precision, arrival=0.0)
        s1 = Server(device_bytes_estimate(r.case, r.precision) + 1, quantum=4, tile=0, keep_results=True)
        s1.run([alone], realtime=False)
        for k in STATE_FIELDS[:r.case.nfields]:
            assert np.array_equal(r.result[k], alone.result[k]), (r.rid, r.precision, k)


def test_budget_is_respected_and_oversize_rejected():
    reqs = small_stream(n=6, seed=9)
    sizes = [device_bytes_estimate(r.case, r.precision) for r in reqs]
    budget = max(sizes) + min(sizes)
    srv = Server(budget, quantum=5, tile=0)
    peak = {"v": 0}
    orig = srv._admit

    def spy(req, now):
        ok = orig(req, now)
        peak["v"] = max(peak["v"], srv.used)
        return ok
    srv._admit = spy
    srv.run(reqs, realtime=False)
    assert peak["v"] <= budget
    big = Request(rid=99, case=reqs[0].case.replace(nPx=64, nPy=64, nPz=32), steps=2)
    with pytest.raises(RuntimeError):
        Server(1024, tile=0).run([big], realtime=False)


def test_realtime_poisson_run_reports_latency():
    reqs = small_stream(n=8, seed=11)
    srv = Server(8 << 30, quantum=5)
    st = srv.run(reqs, realtime=True)
    assert st["tts_p50_s"] > 0 and st["tts_p99_s"] >= st["tts_p50_s"]
    assert st["value"] > 0 and st["tile"] in (0, 1, 2)


def test_autotuner_scratch_counts_against_the_budget():
    """A budget that holds the simulations but not the autotuner's scratch
    copy of their batch: the server skips the tuning and runs the default."""
    reqs = poisson_requests(4, rate=50.0, seed=13, grid_min=(32, 32, 16), grid_max=(32, 32, 16), steps=(3, 8),
                            fp32_fraction=0.0)
    # target_cells=1: one simulation resident at a time, each fits alone but
    # not beside the tuner's copy of it
    need = max(device_bytes_estimate(r.case, r.precision) for r in reqs)
    srv = Server(need + (1 << 20), quantum=4, target_cells=1, keep_results=False)
    for r in reqs:
        r.arrival = 0.0
    st = srv.run(reqs, realtime=False)
    assert st["tune_skipped"] >= 1 and st["tile"] == 2 and st["zrange"]["fp64"] is None
    roomy = poisson_requests(4, rate=50.0, seed=13, grid_min=(32, 32, 16), grid_max=(32, 32, 16), steps=(3, 8),
                             fp32_fraction=0.0)
    for r in roomy:
        r.arrival = 0.0
    st2 = Server(3 * need, quantum=4, target_cells=1).run(roomy, realtime=False)
    assert st2["tune_skipped"] == 0 and st2["zrange"]["fp64"] in (64, 32, 16)


def test_realtime_mixed_stream_with_tuning_overlaps_and_matches_alone():
    """Both precisions' batches running at once while requests are admitted,
    both autotuned (tile shape and z range), step limits and balanced quanta
    on: every request completes, no work item fails its check, and the
    results of a few requests equal the same requests served alone."""
    reqs = poisson_requests(24, rate=200.0, seed=17, grid_min=(32, 32, 32), grid_max=(64, 64, 64),
                            steps=(10, 40), fp32_fraction=0.5)
    cells = sum(r.case.cells for r in reqs)
    srv = Server(64 << 30, quantum=6, keep_results=True, target_cells=cells // 3)
    st = srv.run(reqs, realtime=True)
    assert st["requests"] == len(reqs) and srv.completed == len(reqs)
    assert st["max_resident"] >= 4
    assert st["zrange"]["fp64"] is not None and st["zrange"]["fp32"] is not None
    for r in reqs[:4]:
        alone = Request(rid=r.rid, case=r.case, steps=r.steps, precision=r.precision, arrival=0.0)
        s1 = Server(8 << 30, quantum=6, tile=st["tile"], keep_results=True)
        s1.zrange = dict(st["zrange"])           # the same tuned work-item shapes as in the mix
        s1.tuned = {"fp64": True, "fp32": True}
        s1.run([alone], realtime=False)
        for k in STATE_FIELDS[:r.case.nfields]:
            assert np.array_equal(r.result[k], alone.result[k]), (r.rid, r.precision, k)
