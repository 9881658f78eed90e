"""The request server (wql_server_*): served point-source requests give the
same seismograms as the same scenarios run alone, admission follows the
device-memory budget, and the footprint estimate matches what a scenario
holds."""
import time

import numpy as np
import pytest

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


@pytest.fixture(scope="module")
def medium():
    import wql_configs
    return wql_configs.config4_medium(48)


def _alone(wqlmod, ctx, text, media, steps):
    s = wqlmod.Scenario(ctx, text=text, precision=wqlmod.FP32C, media=media)
    s.step(steps)
    out = [s.stations(b)[1] for b in range(2)]
    s.close()
    return out


def test_footprint_estimate(ctx, wqlmod, medium):
    import wql_configs
    text, media, _ = wql_configs.config4_request(1, n_lo=40, n_hi=48, steps=5, medium=medium)
    res, peak = wqlmod.estimate_device_bytes(text, wqlmod.FP32C)
    s = wqlmod.Scenario(ctx, text=text, precision=wqlmod.FP32C, media=media)
    held = s.info().device_bytes
    s.close()
    assert abs(res - held) <= 0.02 * held, (res, held)
    assert peak > res


def test_served_equals_alone(ctx, wqlmod, medium):
    """Requests submitted while another runs join the running batch once
    their set-up (done beside the stepping) is ready, so each request is on
    the device while another is; each result equals the request run alone
    (bitwise)."""
    import wql_configs
    steps = 120
    reqs = [wql_configs.config4_request(i, n_lo=24, n_hi=44, steps=steps, medium=medium) for i in range(4)]
    srv = wqlmod.Server(ctx, hbm_budget_bytes=64 << 30, round_steps=4)
    ids = [srv.submit(reqs[0][0], steps, media=reqs[0][1])]
    t_end = time.time() + 60.0
    while srv.stats()["active"] < 1 and srv.stats()["completed"] < 1 and time.time() < t_end:
        time.sleep(0.001)
    for text, media, _ in reqs[1:]:
        ids.append(srv.submit(text, steps, media=media))
    for rid in ids:
        assert srv.wait(rid, 300.0) == 1
    times = [srv.result(rid, 0)[1] for rid in ids]
    # every request is on the device (admitted, not yet done) while another
    # one is: their work overlaps
    for k in range(len(ids)):
        assert any(times[j][1] < times[k][2] and times[k][1] < times[j][2] for j in range(len(ids)) if j != k), \
            (k, times)
    for (text, media, _), rid in zip(reqs, ids):
        ref = _alone(wqlmod, ctx, text, media, steps)
        for b in range(2):
            got, times = srv.result(rid, b)
            assert got.shape == ref[b].shape and got.shape[0] == steps
            assert np.array_equal(got, ref[b])
            assert times[0] <= times[1] <= times[2]
        srv.release(rid)
    srv.close()


def test_admission_by_budget(ctx, wqlmod, medium):
    """With room for one request at a time, the second is admitted only after
    the first retires."""
    import wql_configs
    steps = 8
    reqs = [wql_configs.config4_request(i, n_lo=32, n_hi=32, steps=steps, medium=medium) for i in (5, 6)]
    _, peak = wqlmod.estimate_device_bytes(reqs[0][0], wqlmod.FP32C)
    srv = wqlmod.Server(ctx, hbm_budget_bytes=int(peak * 1.5), round_steps=2)
    ids = [srv.submit(text, steps, media=media) for text, media, _ in reqs]
    for rid in ids:
        assert srv.wait(rid, 300.0) == 1
    (_, t0), (_, t1) = srv.result(ids[0], 0), srv.result(ids[1], 0)
    assert t1[1] >= t0[2]
    srv.close()
