"""CPU: the serving engine's admission policy (HBM budget, slots, anti-starvation)."""
from fast_tensor_leverage_gb300.serving import admission_order


def test_admits_in_order_within_budget_and_slots():
    assert admission_order([10, 20, 30], [0, 0, 0], 0, 100, 8, 4) == [0, 1, 2]
    assert admission_order([10, 20, 30], [0, 0, 0], 50, 100, 8, 4) == [0, 1]
    assert admission_order([10, 20, 30], [0, 0, 0], 0, 100, 2, 4) == [0, 1]


def test_small_requests_bypass_a_large_one():
    # the head does not fit; the ones behind it that fit are admitted
    assert admission_order([90, 10, 20], [0, 0, 0], 20, 100, 8, 4) == [1, 2]


def test_starved_request_blocks_the_queue():
    # the head has been bypassed max_bypass times: nothing behind it starts
    assert admission_order([90, 10, 20], [4, 0, 0], 20, 100, 8, 4) == []
    # and once it fits it goes first
    assert admission_order([90, 10, 20], [4, 0, 0], 0, 100, 8, 4) == [0, 1]


def test_never_exceeds_budget():
    import random
    rng = random.Random(0)
    for _ in range(200):
        sizes = [rng.randint(1, 50) for _ in range(rng.randint(0, 12))]
        used = rng.randint(0, 60)
        take = admission_order(sizes, [0] * len(sizes), used, 100, rng.randint(0, 8), 3)
        assert used + sum(sizes[i] for i in take) <= max(100, used)


def test_poisson_stream_is_seeded_and_within_ranges():
    import numpy as np
    from fast_tensor_leverage_gb300 import serving as S
    a = S.poisson_request_stream(5, 200.0, 2.0)
    b = S.poisson_request_stream(5, 200.0, 2.0)
    assert [t for t, _ in a] == [t for t, _ in b]
    assert [repr(r) for _, r in a] == [repr(r) for _, r in b]
    ts = np.array([t for t, _ in a])
    assert np.all(np.diff(ts) > 0) and ts[-1] < 2.0
    assert 250 < len(a) < 550                      # mean 400 arrivals
    for _, r in a:
        if isinstance(r, S.SampleRequest):
            dims, R = r.factors.dims, r.factors.R
            assert 3 <= len(dims) <= 6 and 0 <= r.j <= len(dims)
            assert all(1e4 - 1 <= I <= 1e7 + 1 for I in dims)
        else:
            dims, R = r.dims, r.R
            assert r.idx.dims == dims and r.sweeps == 5
            # fiber keys of every mode stay below 2^62
            for j in range(len(dims)):
                assert np.prod([float(d) for k, d in enumerate(dims) if k != j]) < 2.0 ** 62
        assert R in (8, 16, 32, 64, 128)
        assert 2 ** 10 - 1 <= r.J <= 2 ** 17 + 1
        assert 0 < S.estimate_bytes(r) < 100e9
