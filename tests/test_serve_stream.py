"""Request stream of the served workload (host logic only, no GPU)."""
import numpy as np

from curvib_old_gb300 import serve as S


def test_stream_is_seeded_and_rate_independent():
    a = S.make_stream(300, 5.0, seed=4)
    b = S.make_stream(300, 50.0, seed=4)
    assert [(r.n, r.spheres, r.seed, r.base) for r in a] == [(r.n, r.spheres, r.seed, r.base) for r in b]
    assert np.allclose([r.arrival * 5.0 for r in a], [r.arrival * 50.0 for r in b])
    assert all(x.arrival < y.arrival for x, y in zip(a, a[1:]))


def test_stream_mix():
    st = S.make_stream(2000, 10.0, seed=4)
    follow = [r for r in st if r.base >= 0]
    assert 0.25 < len(follow) / len(st) < 0.35
    for r in follow:
        base = st[r.base]
        assert base.base < 0 and base.rid < r.rid and base.n == r.n and base.spheres == r.spheres
    news = [r for r in st if r.base < 0]
    assert {r.n for r in news} <= set(S.SIZE_LADDER)
    assert all(0 <= len(r.spheres) <= 3 for r in news)
    # log-uniform in unknowns: the median size is near the geometric middle (~90^3)
    med = np.median([r.n for r in news])
    assert 64 <= med <= 128
