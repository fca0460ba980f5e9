"""The launch-shape autotuner's host logic (elsim_gb300/autotune.py) with a
stand-in context, no GPU: every point of the search space is tried, the
first solve of each point (graph capture) is not timed, the fastest point is
kept and left active, and the result is cached per grid shape."""
import itertools

import pytest

from elsim_gb300 import autotune


class FakeCtx:
    """Solve time is a function of the active tuning; the first solve after
    each set_tuning is slow (it would capture a graph)."""

    def __init__(self, shape, cost):
        self.shape = shape
        self.cost = cost
        self.tuning = None
        self.fresh = False
        self.solves = 0
        self.loads = 0

    def set_tuning(self, zc32=0, chunk=0, no_tma=False, **_):
        self.tuning = (zc32, chunk, no_tma)
        self.fresh = True

    def cg_solve(self, **kw):
        assert kw["precision"] == autotune.sbm.PREC_MIXED
        self.solves += 1
        ms = self.cost(*self.tuning) + (1000.0 if self.fresh else 0.0)
        self.fresh = False
        return {"ms": ms, "iters": 42}


@pytest.fixture(autouse=True)
def _empty_cache():
    autotune._cache.clear()
    yield
    autotune._cache.clear()


def test_picks_the_fastest_point_and_leaves_it_active():
    def cost(zc, chunk, no_tma):
        return 10.0 + abs(zc - 16) + (0.5 if chunk == 8 else 0.0) + (3.0 if no_tma else 0.0)

    ctx = FakeCtx((64, 64, 64), cost)
    res = autotune.tune(ctx, lambda: setattr(ctx, "loads", ctx.loads + 1), reps=2)
    space = autotune.DEFAULT_SPACE
    n_points = len(list(itertools.product(*space.values())))
    assert len(res["trials"]) == n_points
    assert {(t["zc32"], t["chunk"], t["no_tma"]) for t in res["trials"]} == set(
        itertools.product(*space.values()))
    # one untimed and `reps` timed solves per point, each after a reload
    assert ctx.solves == ctx.loads == n_points * 3
    assert all(t["ms"] < 1000.0 for t in res["trials"])
    assert res["best"] == {"zc32": 16, "chunk": 16, "no_tma": False, "ms": 10.0, "iters": 42}
    assert ctx.tuning == (16, 16, False)


def test_result_is_cached_per_shape():
    ctx = FakeCtx((32, 32, 32), lambda zc, ch, nt: float(zc))
    first = autotune.tune(ctx, lambda: None)
    n = ctx.solves
    other = FakeCtx((32, 32, 32), lambda zc, ch, nt: 100.0 - zc)
    again = autotune.tune(other, lambda: None)
    assert again is first and other.solves == 0
    assert other.tuning == (8, first["best"]["chunk"], first["best"]["no_tma"])
    assert ctx.solves == n
    third = FakeCtx((32, 32, 32), lambda *a: 0.0)
    assert autotune.apply_cached(third) and third.tuning == other.tuning
    assert not autotune.apply_cached(FakeCtx((48, 48, 48), lambda *a: 0.0))


def test_custom_space():
    ctx = FakeCtx((16, 16, 16), lambda zc, ch, nt: zc * 1.0 + ch)
    res = autotune.tune(ctx, lambda: None, space={"zc32": (4, 8), "chunk": (2,),
                                                  "no_tma": (True,)})
    assert len(res["trials"]) == 2 and res["best"]["zc32"] == 4
    assert ctx.tuning == (4, 2, True)
