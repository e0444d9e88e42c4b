"""The autotuners' selection logic on the host, with a fake context and a
fake timer (no GPU): every candidate is tried, failing shapes are skipped,
the fastest is kept and set on the context, results are cached per key."""
from __future__ import annotations

import pytest

from oct_recon_af_v1_gb300 import autotune


class FakeStitchCtx:
    def __init__(self, cost, failing=()):
        self.cost, self.failing, self.rows, self.set_calls = cost, set(failing), None, []

    def set_stitch_rows(self, rows):
        self.set_calls.append(rows)
        self.rows = rows

    def step(self):
        if self.rows in self.failing:
            raise RuntimeError("patches exceed shared memory")


def fake_timer(ctx):
    return lambda fn, reps: (fn(), ctx.cost[ctx.rows])[1]


def test_stitch_rows_picks_fastest_and_caches():
    autotune._CACHE.clear()
    ctx = FakeStitchCtx({32: 5.0, 64: 3.0, 128: 4.0})
    rows, table = autotune.tune_stitch_rows(ctx, ctx.step, None, key="k1", timer=fake_timer(ctx))
    assert rows == 64 and table == {32: 5.0, 64: 3.0, 128: 4.0}
    assert ctx.rows == 64                                   # the choice is left on the context
    # cached: no trial again, the choice is set once more
    ctx2 = FakeStitchCtx({32: 1.0, 64: 9.0, 128: 9.0})
    rows2, table2 = autotune.tune_stitch_rows(ctx2, ctx2.step, None, key="k1", timer=fake_timer(ctx2))
    assert rows2 == 64 and table2 == table and ctx2.set_calls == [64]


def test_stitch_rows_skips_failing_shapes():
    autotune._CACHE.clear()
    ctx = FakeStitchCtx({32: 1.0, 64: 3.0, 128: 2.0}, failing={32})
    rows, table = autotune.tune_stitch_rows(ctx, ctx.step, None, key="k2", timer=fake_timer(ctx))
    assert rows == 128 and 32 not in table
    ctx = FakeStitchCtx({32: 1.0, 64: 1.0, 128: 1.0}, failing={32, 64, 128})
    with pytest.raises(RuntimeError):
        autotune.tune_stitch_rows(ctx, ctx.step, None, key="k3", timer=fake_timer(ctx))


class FakeBatchCtx:
    def __init__(self, cost):
        self.cost, self.last = cost, None

    def batch_process(self, work, threshold, grab):
        self.last = (grab, work[0][0].shape[0])


class T:
    def __init__(self, *shape):
        self.shape = shape


def test_batch_tuner_orders_and_grabs():
    autotune._CACHE.clear()
    tiles = [(T(10, 125, 8), 25, 0, None), (T(30, 125, 8), 25, 1, None)]
    # largest first puts the 30-B-scan tile first; make (grab 8, largest_first) the fastest
    cost = {(g, b): 10.0 + g * 0.1 for g in autotune.GRABS for b in (10, 30)}
    cost[(8, 30)] = 1.0
    ctx = FakeBatchCtx(cost)
    timer = lambda fn, reps: (fn(), ctx.cost[ctx.last])[1]
    grab, order, table = autotune.tune_batch(ctx, tiles, 1e-9, None, timer=timer)
    assert (grab, order) == (8, "largest_first")
    assert len(table) == len(autotune.GRABS) * len(autotune.ORDERS)
    assert autotune.ordered(tiles, "largest_first")[0][2] == 1
