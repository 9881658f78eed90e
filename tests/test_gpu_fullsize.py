"""Checks at the benchmark sizes (config 1: 2 x 201^3; config 2: 2 x
401x201x201), through properties that do not need the oracle: the TMA
stencil agrees with the per-point kernel, FP32C with FP64, the packed batch
with a lone run, and the fields stay finite."""
import numpy as np
import pytest

from gpu_helpers import rel_l2

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def ctx():
    import wql_build
    wql_build.build()
    import wql
    c = wql.Context(0)
    yield c
    c.close()


@pytest.fixture(scope="module")
def wqlmod():
    import wql
    return wql


def test_config1_tma_vs_pointwise(ctx, wqlmod):
    import wql_configs
    text, media = wql_configs.config1(n=201, steps=10)
    a = wqlmod.Scenario(ctx, text=text, precision=wqlmod.FP32C, media=media)
    b = wqlmod.Scenario(ctx, text=text, precision=wqlmod.FP32C, media=media)
    b.set_tuning(1, 0)
    a.step(3)
    b.step(3)
    a.sync(check_nan=True)
    b.sync(check_nan=True)
    for blk in range(2):
        fa, fb = a.fields(blk), b.fields(blk)
        assert rel_l2(fa, fb) < 1e-5
    a.close()
    b.close()


def test_config1_batch_equals_alone(ctx, wqlmod):
    import wql_configs
    text, media = wql_configs.config1(n=201, steps=10)
    a = wqlmod.Scenario(ctx, text=text, precision=wqlmod.FP32C, media=media)
    m = wqlmod.Scenario(ctx, text=text, precision=wqlmod.FP32C, media=media)
    a.step(2)
    batch = wqlmod.Batch(ctx)
    batch.add(m)
    batch.step(2)
    m.sync(check_nan=True)
    for blk in range(2):
        assert np.array_equal(a.field(blk, 0), m.field(blk, 0))
    batch.close()
    a.close()
    m.close()


def test_config2_fp32c_vs_fp64(ctx, wqlmod):
    """PML, plasticity and the von Karman medium at full size: two steps of
    FP32C against FP64."""
    import wql_configs
    text, media = wql_configs.config2(steps=10)
    d = wqlmod.Scenario(ctx, text=text, precision=wqlmod.FP64, media=media)
    f = wqlmod.Scenario(ctx, text=text, precision=wqlmod.FP32C, media=media)
    d.step(2)
    f.step(2)
    f.sync(check_nan=True)
    d.sync(check_nan=True)
    for blk in range(2):
        for c in range(3):
            assert rel_l2(f.field(blk, c), d.field(blk, c)) < 1e-5, (blk, c)
    d.close()
    f.close()
