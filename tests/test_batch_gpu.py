"""Ragged batches: one persistent launch per substage over the tiles of all
instances, CUDA-graph steps, autotuned tile shape."""
import numpy as np
import pytest

from gpu_util import rel_err
from mhd_gb300.case import STATE_FIELDS, initial_state, small_cases
from mhd_gb300.sim import Batch, Simulation

pytestmark = pytest.mark.gpu

SIZES = [(32, 32, 8), (48, 48, 16), (20, 12, 10), (64, 64, 8), (33, 5, 6), (16, 40, 12)]


def make_cases(seed0=3):
    base = small_cases()["mhd_fixedT"]
    return [base.replace(nPx=x, nPy=y, nPz=z, seed=seed0 + i, RE=50.0 + 10 * i, bz0=1e-3 * (i + 1))
            for i, (x, y, z) in enumerate(SIZES)]


def fresh(case):
    sim = Simulation(case, path="fused")
    sim.upload_state(initial_state(case))
    sim.communicate()
    return sim


@pytest.mark.parametrize("tile", [0, 1, 2])
def test_batch_equals_instances_alone(tile):
    cases = make_cases()
    sims = [fresh(c) for c in cases]
    b = Batch(sims)
    b.set_tile(tile)
    b.steps(3)
    b.sync()
    got = [s.download_state() for s in sims]
    b.close()
    for s in sims:
        s.close()
    # each instance alone, in a batch of one with the same tile shape: bit-exact
    for i, c in enumerate(cases):
        solo = fresh(c)
        bs = Batch([solo])
        bs.set_tile(tile)
        bs.steps(3)
        bs.sync()
        ref = solo.download_state()
        bs.close()
        # and the single-instance fused path: equal to rounding
        plain = fresh(c)
        plain.steps(3, c.dt)
        pl = plain.download_state()
        plain.close()
        solo.close()
        for k in STATE_FIELDS:
            assert np.array_equal(got[i][k], ref[k]), (i, k)
            assert rel_err(got[i][k], pl[k]) <= 1e-12, (i, k)


def test_autotune_picks_and_caches_a_tile():
    cases = make_cases(seed0=20)
    sims = [fresh(c) for c in cases]
    b = Batch(sims)
    chosen, ms = b.autotune()
    assert chosen in (0, 1, 2) and all(m > 0 for m in ms)
    before = [s.download_state()["TT"] for s in sims]
    b.steps(2)
    b.sync()
    assert b.tile() == chosen
    # the autotuner ran on scratch copies: the instances only advanced by the 2 real steps
    after = [s.download_state()["TT"] for s in sims]
    assert any(not np.array_equal(x, y) for x, y in zip(before, after))
    b.close()
    for s in sims:
        s.close()


def test_batch_then_single_steps_interleave():
    """Batched steps and single steps on the same instances stay consistent."""
    cases = make_cases(seed0=40)[:3]
    sims = [fresh(c) for c in cases]
    b = Batch(sims)
    b.set_tile(0)
    b.steps(1)
    for s in sims:
        s.step(s.case.dt)
    b.steps(2)
    b.sync()
    got = [s.download_state() for s in sims]
    b.close()
    for i, c in enumerate(cases):
        ref = fresh(c)
        ref.steps(4, c.dt)
        r = ref.download_state()
        ref.close()
        for k in STATE_FIELDS:
            assert rel_err(got[i][k], r[k]) <= 1e-12, (i, k)
    for s in sims:
        s.close()


def test_mixed_switch_sets_rejected():
    a = fresh(small_cases()["mhd_fixedT"])
    c = fresh(small_cases()["hydro_default_bc"])
    from mhd_gb300.abi import MhdError
    with pytest.raises(MhdError):
        Batch([a, c])
    a.close()
    c.close()


def test_fp32_batch_equals_instances_alone():
    cases = make_cases(seed0=60)[:4]

    def fresh32(c):
        s = Simulation(c, precision="fp32")
        s.upload_state(initial_state(c))
        s.communicate()
        return s
    sims = [fresh32(c) for c in cases]
    b = Batch(sims)
    b.steps(3)
    b.sync()
    got = [s.download_state() for s in sims]
    b.close()
    for s in sims:
        s.close()
    for i, c in enumerate(cases):
        solo = fresh32(c)
        bs = Batch([solo])
        bs.steps(3)
        bs.sync()
        ref = solo.download_state()
        bs.close()
        solo.close()
        plain = fresh32(c)
        plain.steps(3, c.dt)
        pl = plain.download_state()
        plain.close()
        for k in STATE_FIELDS:
            assert np.array_equal(got[i][k], ref[k]), (i, k)
            assert rel_err(got[i][k], pl[k]) <= 1e-6, (i, k)


def config2_subset():
    """Instances of the 64-instance ragged batch (nx = ny from
    {32,48,64,96,128}, nz from {32,64}, per-instance seed, 1/Re and Bz0), one
    of each distinct shape, so the tallest and widest ones (128x128x64) are in."""
    from mhd_gb300.case import config2_batch
    seen, out = set(), []
    for c in config2_batch():
        key = (c.nPx, c.nPz)
        if key not in seen:
            seen.add(key)
            out.append(c)
    return out


@pytest.mark.parametrize("tile,zmax", [(0, 64), (2, 16)])
def test_batch_config2_shapes_against_the_oracle(tile, zmax):
    """One batched step of config 2's real instance shapes, every instance
    compared with the oracle directly: 1e-12 of each field's max-norm.  With
    zmax 16 every instance is split into 2 or 4 z ranges of one work list."""
    from gpu_util import oracle_for
    cases = config2_subset()
    assert any(c.nPz == 64 for c in cases) and any(c.nPx == 128 for c in cases)
    states = [initial_state(c) for c in cases]
    sims = []
    for c, st in zip(cases, states):
        s = Simulation(c, path="fused")
        s.upload_state(st)
        s.communicate()
        sims.append(s)
    b = Batch(sims)
    b.set_tile(tile)
    b.set_zrange(zmax)
    assert b.zrange() == zmax
    b.steps(1)
    b.sync()
    got = [s.download_state() for s in sims]
    b.close()
    for s in sims:
        s.close()
    for c, st, g in zip(cases, states, got):
        o = oracle_for(c, st, nthreads=16)
        o.steps(1)
        for k in STATE_FIELDS:
            assert rel_err(g[k], o.arr[k]) <= 1e-12, (c.nPx, c.nPz, k, rel_err(g[k], o.arr[k]))


@pytest.mark.parametrize("prec", ["fp64", "fp32"])
def test_limited_steps_equal_instances_alone(prec):
    """mhd_batch_steps_limited: instance i takes min(n, limit[i]) of n batched
    steps; each result equals the instance stepped alone that many times in a
    batch of one (bit for bit), and a later unlimited call continues from it."""
    cases = make_cases(seed0=80)[:4]
    limits = [5, 0, 2, 7]

    def fresh_p(c):
        s = Simulation(c, path="fused", precision=prec)
        s.upload_state(initial_state(c))
        s.communicate()
        return s
    sims = [fresh_p(c) for c in cases]
    b = Batch(sims)
    b.set_tile(0)
    b.steps_limited(5, limits)
    b.steps(1)
    b.sync()
    got = [s.download_state() for s in sims]
    b.close()
    for s in sims:
        s.close()
    for i, c in enumerate(cases):
        solo = fresh_p(c)
        bs = Batch([solo])
        bs.set_tile(0)
        bs.steps(min(5, limits[i]) + 1)
        bs.sync()
        ref = solo.download_state()
        bs.close()
        solo.close()
        for k in STATE_FIELDS:
            assert np.array_equal(got[i][k], ref[k]), (prec, i, k)


def test_fp32_autotune_picks_a_zrange():
    cases = make_cases(seed0=100)

    def fresh32(c):
        s = Simulation(c, precision="fp32")
        s.upload_state(initial_state(c))
        s.communicate()
        return s
    sims = [fresh32(c) for c in cases]
    b = Batch(sims)
    assert b.autotune_bytes() > 0
    chosen, ms = b.autotune()
    assert chosen == 0 and ms[0] > 0 and b.zrange() in (64, 32, 16)
    b.steps(1)
    b.sync()
    b.close()
    for s in sims:
        s.close()
