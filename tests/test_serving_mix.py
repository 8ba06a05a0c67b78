"""Host side of the serving loop: the seeded request stream and its
time-step rule (no GPU)."""
import numpy as np

from advection_miniapp_gb300.serving import DEGREES, SIZES, request_mix


def test_requests_depend_only_on_seed_and_index():
    a = request_mix(40, seed=7, rate=100.0)
    b = request_mix(80, seed=7, rate=100.0)
    for x, y in zip(a, b):
        assert (x.n, x.degree, x.velocity, x.phase, x.t_end, x.precision) == \
               (y.n, y.degree, y.velocity, y.phase, y.t_end, y.precision)
    c = request_mix(40, seed=8)
    assert any(x.n != y.n or x.velocity != y.velocity for x, y in zip(a, c))


def test_distribution_of_the_mix():
    reqs = request_mix(2000, seed=1, rate=500.0)
    assert {r.n for r in reqs} == set(SIZES)
    assert {r.degree for r in reqs} == set(DEGREES)
    assert {r.precision for r in reqs} == {0, 1}
    for r in reqs:
        assert abs(np.linalg.norm(r.velocity) - 1.0) < 1e-14
        assert all(0.0 <= p < 1.0 for p in r.phase)
        assert 0.1 <= r.t_end <= 1.0
    arr = np.array([r.arrival for r in reqs])
    assert arr[0] == 0.0 and np.all(np.diff(arr) >= 0)
    # Poisson process: mean inter-arrival 1/rate
    assert abs(np.diff(arr).mean() * 500.0 - 1.0) < 0.1


def test_step_rule():
    """dt = Courant h / |a| / k^1.5 rounded down to t_end / ceil(t_end / dt)."""
    for r in request_mix(50, seed=3):
        dt0 = 0.5 / r.n / r.degree ** 1.5
        s = r.steps()
        assert r.t_end / s <= dt0 * (1 + 1e-12)
        assert s == 1 or r.t_end / (s - 1) > dt0 * (1 - 1e-12)


def test_device_bytes_of_a_request():
    from advection_miniapp_gb300.serving import Request
    r64 = Request(0, 4, 3, (1.0, 0.0, 0.0), (0.0, 0.0, 0.0), 0.1, 0)
    r32 = Request(1, 4, 3, (1.0, 0.0, 0.0), (0.0, 0.0, 0.0), 0.1, 1)
    assert r32.device_bytes() == 3 * 8 * 64 * 64
    assert r64.device_bytes() == 3 * 8 * 64 * 64 + 2 * 6 * 16 * 8 * 64
