"""Host-side pieces of the benchmark's request streams: the batched configuration (64
jobs at once, soup and stadium alternately, 4 spp, 128^2..1080p) and the served one
(Poisson arrivals, three scenes, spp in {1, 4, 16, 64}, 64^2..1080p), and the
autotuner's batch of uneven requests."""
import numpy as np

import bench
from mambatracer_gb300 import tune


def _check_sizes(reqs, lo):
    for _, _, w, h, _, _ in reqs:
        assert 8 <= w <= 1920 and 8 <= h <= 1080
        assert 0.5 * lo <= w * h <= 1920 * 1080


def test_batched_requests():
    reqs = bench.request_list("batched", np.random.default_rng(3), 0, 0)
    assert len(reqs) == 64 and all(t == 0.0 for t, *_ in reqs)
    assert [k for _, k, *_ in reqs] == ["soup", "stadium"] * 32
    assert all(spp == 4 for *_, spp, _ in reqs)
    _check_sizes(reqs, 128 * 128)
    again = bench.request_list("batched", np.random.default_rng(3), 0, 0)
    assert again == reqs  # seeded: the same stream every run


def test_served_requests_are_a_poisson_stream():
    rate, duration = 200.0, 10.0
    reqs = bench.request_list("served", np.random.default_rng(4), duration, rate)
    times = np.array([t for t, *_ in reqs])
    assert np.all(np.diff(times) >= 0) and times[-1] < duration
    assert abs(len(reqs) - rate * duration) < 4 * np.sqrt(rate * duration)
    assert {k for _, k, *_ in reqs} == {"room", "soup", "stadium"}
    assert {spp for *_, spp, _ in reqs} == {1, 4, 16, 64}
    _check_sizes(reqs, 64 * 64)
    px = np.array([w * h for _, _, w, h, _, _ in reqs], float)
    # log-uniform pixel counts: the median sits near the geometric mean of the bounds
    assert 0.5 < np.median(px) / np.sqrt(64 * 64 * 1920 * 1080) < 2.0


def test_tuner_request_batch():
    reqs = tune.served_requests()
    assert len(reqs) == 64 and [k for k, *_ in reqs] == list(range(64))
    for _, cam, w, h, spp in reqs:
        assert spp == 4 and 8 <= w <= 1920 and 8 <= h <= 1080 and cam.nbytes == 64
