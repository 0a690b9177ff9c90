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
