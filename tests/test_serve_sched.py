"""Serving form, host logic (no GPU): admission under the device-memory budget and
continuous-batching selection of the Scheduler."""
import numpy as np
import pytest

from st_spix_gb300.serve import Scheduler, poisson_arrivals


def test_admission_waits_for_memory():
    s = Scheduler(budget=100, reserve=20, max_batch=4)
    assert s.offer(1, 30, [0.0, 0.1])
    assert s.offer(2, 30, [0.0])
    assert not s.offer(3, 30, [0.0, 0.5])          # 20 + 30 + 30 + 30 > 100
    assert s.queue == [3] and s.used == 80
    items = s.next_batch(0.0)
    assert sorted(i[0] for i in items) == [1, 2]
    fin = s.complete(items, 0.2)
    assert fin == [2]                                # stream 2 had one frame
    # stream 3 admitted when stream 2 released its memory, arrivals from then on
    assert s.streams[3].admitted_at == 0.2
    np.testing.assert_allclose(s.streams[3].arrivals, [0.2, 0.7])
    assert s.used == 80 and s.peak_used <= 100


def test_stream_larger_than_budget_rejected():
    s = Scheduler(budget=100, reserve=50, max_batch=2)
    with pytest.raises(ValueError):
        s.offer(1, 60, [0.0])
    with pytest.raises(ValueError):
        Scheduler(budget=10, reserve=20, max_batch=1)


def test_batch_selection_oldest_first_one_per_stream():
    s = Scheduler(budget=1000, reserve=0, max_batch=2)
    s.offer(1, 1, [0.3, 0.4])
    s.offer(2, 1, [0.1, 0.2])
    s.offer(3, 1, [0.2])
    s.offer(4, 1, [5.0])
    assert s.next_batch(0.05) == []                 # nothing has arrived
    items = s.next_batch(1.0)
    assert items == [(2, 0, 0.1), (3, 0, 0.2)]      # oldest two, max_batch = 2
    items2 = s.next_batch(1.0)                       # 2 and 3 are in flight
    assert items2 == [(1, 0, 0.3)]
    assert s.next_batch(1.0) == []
    s.complete(items, 1.1)
    assert s.next_batch(1.2) == [(2, 1, 0.2)]       # stream 2's next frame
    assert s.next_arrival() == 5.0


def test_out_of_order_completion_is_an_error():
    s = Scheduler(budget=10, reserve=0, max_batch=1)
    s.offer(1, 1, [0.0, 0.0])
    s.next_batch(0.0)
    with pytest.raises(RuntimeError):
        s.complete([(1, 1, 0.0)], 0.1)


def test_simulated_serving_serves_every_frame_in_order():
    rng = np.random.Generator(np.random.PCG64(0))
    s = Scheduler(budget=200, reserve=40, max_batch=3)
    for sid in range(8):
        s.offer(sid, 50, poisson_arrivals(6, 30.0, rng))
    now = 0.0
    steps = 0
    while not s.done():
        items = s.next_batch(now)
        if not items:
            now = max(now, s.next_arrival() or now)
            continue
        now += 0.004 * len(items)                    # a batch's service time
        s.complete(items, now)
        assert s.used <= s.budget
        steps += 1
    assert len(s.latency) == 8 * 6 and steps < 48
    for sid in range(8):
        frames = [f for (q, f, a, d) in s.latency if q == sid]
        assert frames == list(range(6))
    assert all(d >= a for (_, _, a, d) in s.latency)
    assert s.peak_used <= 200


def test_finished_state_is_reused_or_evicted():
    s = Scheduler(budget=100, reserve=0, max_batch=4)
    s.offer(1, 60, [0.0], kind="a")
    assert not s.offer(2, 50, [0.0], kind="b")      # 60 + 50 > 100
    s.complete(s.next_batch(0.0), 0.1)              # stream 1's state becomes a spare
    # stream 2 (kind b) needs fresh bytes: the spare of kind a is evicted for it
    assert s.streams[2].admitted_at == 0.1 and s.evicted == ["a"]
    assert s.used == 50
    s.offer(3, 50, [0.0], kind="b")                 # fits next to stream 2
    s.complete(s.next_batch(1.0), 1.0)              # 2 and 3 finish: two spares of kind b
    assert s.used == 100
    s.offer(4, 50, [0.0], kind="b")                 # takes over a spare: no fresh bytes
    assert s.reused == 1 and s.used == 100 and s.peak_used <= 100


def test_pixel_cap_bounds_batches_oldest_first():
    s = Scheduler(budget=1000, reserve=0, max_batch=8, max_pixels=1000)
    s.offer(1, 1, [0.1], npix=600)
    s.offer(2, 1, [0.2], npix=600)
    s.offer(3, 1, [0.3], npix=300)
    s.offer(4, 1, [0.4], npix=2000)        # larger than the cap: still served alone
    items = s.next_batch(1.0)
    assert [i[0] for i in items] == [1]     # 1 + 2 would exceed the cap; 3 may not jump 2
    items = s.next_batch(1.0)
    assert [i[0] for i in items] == [2, 3]
    assert [i[0] for i in s.next_batch(1.0)] == [4]
    # no cap: one batch of everything that arrived
    s = Scheduler(budget=1000, reserve=0, max_batch=8)
    for sid in range(3):
        s.offer(sid, 1, [0.0], npix=10 ** 6)
    assert len(s.next_batch(0.0)) == 3


def test_batches_group_frames_of_the_oldest_frames_size():
    s = Scheduler(budget=1000, reserve=0, max_batch=3)
    s.offer(1, 1, [0.1], npix=100)
    s.offer(2, 1, [0.2], npix=400)
    s.offer(3, 1, [0.3], npix=100)
    s.offer(4, 1, [0.4], npix=400)
    s.offer(5, 1, [0.5], npix=100)
    # the oldest frame (100 px) first, then the other 100-px frames, oldest first
    assert [i[0] for i in s.next_batch(1.0)] == [1, 3, 5]
    assert [i[0] for i in s.next_batch(1.0)] == [2, 4]
    # without grouping: oldest first across sizes
    s = Scheduler(budget=1000, reserve=0, max_batch=3, group_sizes=False)
    for sid, n in zip(range(1, 6), [100, 400, 100, 400, 100]):
        s.offer(sid, 1, [0.1 * sid], npix=n)
    assert [i[0] for i in s.next_batch(1.0)] == [1, 2, 3]
