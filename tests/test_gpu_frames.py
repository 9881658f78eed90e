"""Fault frames leave the device through two rings: one fills while the
other's copy to pinned host memory runs.  The frames must come out the same
whether they are read once at the end (every ring change overlapped with
the stepping) or read between steps (every read a synchronous flush), in
both precisions, and over several ring changes."""
import numpy as np
import pytest

from inputs import block_list, problem

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def ctx():
    import wql_build
    wql_build.build()
    import wql
    c = wql.Context(0)
    yield c
    c.close()


@pytest.mark.parametrize("prec", ["fp32c", "fp64"])
def test_frames_same_overlapped_and_synchronous(ctx, prec):
    import wql
    p = wql.FP32C if prec == "fp32c" else wql.FP64
    text = problem(t_final="5d0") + block_list(17)
    steps = 150  # a ring holds 64 frames of a 17 x 17 fault: two ring changes and a partial ring
    a = wql.Scenario(ctx, text=text, precision=p)
    a.step(steps)
    fa = {k: a.frames(k) for k in ("Svel", "S", "Uhat", "trup", "state")}
    b = wql.Scenario(ctx, text=text, precision=p)
    done = 0
    for n in (1, 6, 57, 1, 63, 22):
        b.step(n)
        done += n
        assert b.frame_count() == done
        b.frames("Svel")
    assert done == steps
    fb = {k: b.frames(k) for k in fa}
    assert a.frame_count() == b.frame_count() == steps
    for k in fa:
        assert fa[k].shape[0] == steps
        np.testing.assert_array_equal(fa[k], fb[k], err_msg=k)
    # the frames advance: the last slip rate differs from the first
    assert np.abs(fa["Svel"][-1] - fa["Svel"][0]).max() > 0
    a.close()
    b.close()


def test_destroy_with_frames_in_flight(ctx):
    """wql_step returns with the last ring's copy to pinned memory possibly
    still queued; destroying the scenario right away waits for it (no read
    of freed memory), and a scenario created afterwards starts clean."""
    import wql
    text = problem(t_final="5d0") + block_list(17)
    for _ in range(3):
        s = wql.Scenario(ctx, text=text, precision=wql.FP32C)
        s.step(130)
        s.close()
    s = wql.Scenario(ctx, text=text, precision=wql.FP32C)
    s.step(3)
    assert s.frame_count() == 3
    assert s.frames("Svel").shape[0] == 3
    s.close()
