"""The serving loop's admission and chunk policy, run without a device
(sbg_serve_simulate drives the same scheduler sbg_server_tick uses)."""
import numpy as np
import pytest

from simbody_gb300 import _native as N
from simbody_gb300.serve import simulate

BIG = [10**9] * 5


def chunks(h, c):
    return max(1, -(-h // c))


def test_every_request_runs_its_chunks_in_consecutive_ticks():
    rng = np.random.default_rng(3)
    n, chunk = 200, 16
    units = rng.integers(1, 50, size=(n, 5))
    hz = rng.integers(0, 300, size=n)
    arr = np.sort(rng.integers(0, 40, size=n))
    adm, done, peak = simulate(units, hz, arr, BIG, max_slots=10**6, chunk_steps=chunk)
    assert (adm == arr).all()  # unlimited memory and slots: admitted on arrival
    assert (done == adm + np.array([chunks(int(h), chunk) for h in hz]) - 1).all()
    assert peak <= n


def test_slots_bound_residency_and_admission_is_fifo():
    rng = np.random.default_rng(4)
    n, chunk, slots = 120, 8, 7
    units = np.ones((n, 5), dtype=np.int64)
    hz = rng.integers(1, 100, size=n)
    arr = np.zeros(n, dtype=np.int64)
    adm, done, peak = simulate(units, hz, arr, BIG, max_slots=slots, chunk_steps=chunk)
    assert peak <= slots
    assert (np.diff(adm) >= 0).all()  # strict arrival order
    assert (done >= adm).all()
    # at every tick at most `slots` requests are resident
    T = int(done.max()) + 1
    occ = np.zeros(T, dtype=int)
    for a, d in zip(adm, done):
        occ[a:d + 1] += 1
    assert occ.max() <= slots


def test_memory_budget_bounds_residency():
    # each request needs 30 state units; the pool holds 100: three at a time
    n = 40
    units = np.zeros((n, 5), dtype=np.int64)
    units[:, 2] = 30
    cap = [10**9, 10**9, 100, 10**9, 10**9]
    hz = np.full(n, 64)
    adm, done, peak = simulate(units, hz, np.zeros(n, dtype=np.int64), cap, max_slots=1000, chunk_steps=16)
    T = int(done.max()) + 1
    occ = np.zeros(T, dtype=int)
    for a, d in zip(adm, done):
        occ[a:d + 1] += 1
    assert occ.max() == 3 and peak == 3
    # memory freed by a finished request is reused at the next tick
    assert adm[3] == done[0] + 1


def test_request_that_never_fits_is_rejected():
    units = np.array([[1, 1, 1000, 1, 1]], dtype=np.int64)
    with pytest.raises(N.EngineError) as e:
        simulate(units, [10], [0], [10, 10, 100, 10, 10], max_slots=4, chunk_steps=8)
    assert e.value.code == 4  # SBG_ERR_BUDGET


@pytest.mark.parametrize("seed", [5, 6, 7])
def test_mixed_sizes_never_overcommit_a_pool_and_all_finish(seed):
    """Requests of very different footprints against small pools: at every
    tick the resident requests' units fit every pool, admission stays in
    arrival order, and every request finishes with its own number of chunks."""
    rng = np.random.default_rng(seed)
    n, chunk = 150, 8
    cap = np.array([400, 300, 500, 2000, 700], dtype=np.int64)
    units = np.stack([rng.integers(1, c // 3, size=n) for c in cap], axis=1).astype(np.int64)
    hz = rng.integers(1, 120, size=n)
    arr = np.sort(rng.integers(0, 60, size=n))
    adm, done, peak = simulate(units, hz, arr, cap, max_slots=32, chunk_steps=chunk)
    assert (adm >= arr).all() and (np.diff(adm) >= 0).all()
    assert (done - adm + 1 >= np.array([chunks(int(h), chunk) for h in hz])).all()
    T = int(done.max()) + 1
    use = np.zeros((T, 5), dtype=np.int64)
    occ = np.zeros(T, dtype=int)
    for k in range(n):
        use[adm[k]:done[k] + 1] += units[k]
        occ[adm[k]:done[k] + 1] += 1
    assert (use <= cap).all()
    assert occ.max() <= 32 and peak <= 32
