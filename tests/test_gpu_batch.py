"""Continuous batching (wql_batch_*): members of different size, mesh and
physics advance in one packed stencil launch per stage and give the same
fields, fault state and seismograms as the same scenarios stepped alone;
members join and leave between steps."""
import numpy as np
import pytest

from inputs import case_text, golden_in, write

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def wqlmod():
    import wql_build
    wql_build.build()
    import wql
    return wql


@pytest.fixture(scope="module")
def ctx(wqlmod):
    c = wqlmod.Context(0)
    yield c
    c.close()


def _members(wqlmod, ctx, tmp_path):
    import wql_configs
    cart = write(tmp_path, "cart.in", golden_in("test_rup_cart_fric"))
    mt = write(tmp_path, "mt.in", case_text("mt4"))
    text1, media1 = wql_configs.config1(n=45, steps=40)
    specs = [dict(path=cart, precision=wqlmod.FP32C),
             dict(path=mt, precision=wqlmod.FP32C),
             dict(text=text1, media=media1, precision=wqlmod.FP32C),
             dict(path=cart, precision=wqlmod.FP64)]   # not packed: its own stencil launch

    def make(spec):
        if "path" in spec:
            return wqlmod.Scenario(ctx, spec["path"], precision=spec["precision"])
        return wqlmod.Scenario(ctx, text=spec["text"], precision=spec["precision"], media=spec["media"])
    return specs, make


def _same(a, b):
    for blk in range(2):
        fa, fb = a.fields(blk), b.fields(blk)
        assert np.array_equal(fa, fb), (blk, np.abs(fa - fb).max())
    for copy in range(2):
        for what in range(6):
            assert np.array_equal(a.iface(copy, what), b.iface(copy, what)), (copy, what)


def test_batch_matches_alone(ctx, wqlmod, tmp_path):
    specs, make = _members(wqlmod, ctx, tmp_path)
    alone = [make(s) for s in specs]
    mixed = [make(s) for s in specs]
    for s in alone:
        s.step(12)
    batch = wqlmod.Batch(ctx)
    for s in mixed:
        batch.add(s)
    batch.step(12)
    for a, m in zip(alone, mixed):
        m.sync(check_nan=True)
        _same(a, m)
    # fault frames and station records of the truth/1 member
    assert np.array_equal(alone[0].frames("Svel"), mixed[0].frames("Svel"))
    ia, ra = alone[0].stations(0)
    im, rm = mixed[0].stations(0)
    assert ia.tolist() == im.tolist() and np.array_equal(ra, rm)
    batch.close()


def test_members_join_and_leave(ctx, wqlmod, tmp_path):
    """A member that joins late and one that leaves early still match their
    runs alone."""
    specs, make = _members(wqlmod, ctx, tmp_path)
    a0, a1 = make(specs[0]), make(specs[2])
    m0, m1 = make(specs[0]), make(specs[2])
    a0.step(10)
    a1.step(6)
    batch = wqlmod.Batch(ctx)
    batch.add(m0)
    batch.step(4)            # m0 alone in the batch
    batch.add(m1)
    batch.step(6)            # both
    batch.remove(m0)         # m0 has 10 steps, m1 has 6
    m0.sync(check_nan=True)
    m1.sync(check_nan=True)
    _same(a0, m0)
    _same(a1, m1)
    batch.close()


def test_autotune_keeps_state(ctx, wqlmod):
    """The autotuner leaves the scenario's state alone and its choice steps
    like the per-point kernel."""
    import wql_configs
    text, media = wql_configs.config1(n=45, steps=10)
    s = wqlmod.Scenario(ctx, text=text, precision=wqlmod.FP32C, media=media)
    r = wqlmod.Scenario(ctx, text=text, precision=wqlmod.FP32C, media=media)
    s.step(2)
    r.step(2)
    before = [s.fields(b) for b in range(2)]
    v, c = s.autotune(reps=2)
    assert v in (5, 6)
    for b in range(2):
        assert np.array_equal(s.fields(b), before[b])
    r.set_tuning(1, 0)
    s.step(4)
    r.step(4)
    for b in range(2):
        a, ref = s.fields(b), r.fields(b)
        assert np.linalg.norm(a - ref) <= 2e-6 * np.linalg.norm(ref)


def test_member_replaced(ctx, wqlmod, tmp_path):
    """A member that leaves and is destroyed, then a new scenario (which may
    reuse its host address) joins: the batch's packed tables follow the new
    member, which steps as it does alone."""
    specs, make = _members(wqlmod, ctx, tmp_path)
    batch = wqlmod.Batch(ctx)
    for _ in range(3):
        m = make(specs[2])
        batch.add(m)
        batch.step(3)
        batch.remove(m)
        m.close()
    fresh, ref = make(specs[2]), make(specs[2])
    batch.add(fresh)
    batch.step(5)
    ref.step(5)
    fresh.sync(check_nan=True)
    _same(ref, fresh)
    batch.close()
