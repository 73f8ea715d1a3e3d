"""The oracle's CPython float primitives against the running interpreter (CPU only)."""
import math
import random

import pytest

import oracle


def _values(n, seed):
    rng = random.Random(seed)
    out = []
    for _ in range(n):
        scale = 10.0 ** rng.randint(-20, 20)
        out.append(rng.uniform(-1.0, 1.0) * scale)
    return out


def test_sum_uses_neumaier_compensation_like_cpython():
    values = _values(3000, 1)
    for i in range(0, len(values) - 3, 3):
        triple = values[i:i + 3]
        assert oracle.py_sum(triple) == sum(triple)
        squares = [v * v for v in triple]
        assert oracle.py_sum(squares) == sum(squares)
    assert oracle.py_sum([1e16, 1.0, -1e16]) == sum([1e16, 1.0, -1e16]) == 1.0


def test_mod_and_divmod_follow_python():
    values = _values(2000, 2) + [-1e-17, -0.0, 0.0, 1.0, -1.0, 2.5, -2.5]
    for x in values:
        for y in (1.0, 3.7, 10.857):
            assert oracle.py_mod(x, y) == x % y
            assert oracle.py_divmod(x, y) == divmod(x, y)


def test_time_add_matches_reference_time_class():
    rng = random.Random(3)
    for _ in range(2000):
        q, r = float(rng.randint(0, 10 ** 6)), rng.random()
        dt = rng.expovariate(1.0) * 10.0 ** rng.randint(-6, 2)
        add_q, new_r = divmod(r + dt, 1.0)
        assert oracle.time_add(q, r, dt) == (q + add_q, new_r)
    assert oracle.time_add(3.0, 0.5, math.inf) == (math.inf, math.inf)


def test_own_log_is_accurate():
    rng = random.Random(4)
    for _ in range(20000):
        x = rng.random() or 0.5
        exact = math.log(x)
        assert abs(oracle.log(x) - exact) <= 2.5 * math.ulp(exact) + 1e-300
    assert oracle.log(1.0) == 0.0


def test_keyed_draws_are_uniform_and_distinct():
    key = oracle.chain_key(7, 3)
    draws = [oracle.draw(key, e, k, t) for e in range(20) for k in range(3) for t in range(50)]
    assert len(set(draws)) == len(draws)
    u = [oracle.uniform(d) for d in draws]
    assert 0.45 < sum(u) / len(u) < 0.55
    assert all(0.0 <= x < 1.0 for x in u)
    counts = [0] * 7
    for d in draws:
        counts[oracle.randbelow(d, 7)] += 1
    assert min(counts) > 0.8 * len(draws) / 7
