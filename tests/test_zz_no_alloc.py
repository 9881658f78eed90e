"""wql_get_field_noalloc (fixed device scratch, no allocation) against
wql_get_field on the same scenario state, two calls in a row each; FP32C
(widened through the scratch, including a block whose row pitch differs from
nq) and FP64.  Collected last so it also runs after every other GPU test."""
import numpy as np
import pytest

from inputs import golden_in, write

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


def _check(s, nblocks=2):
    for _ in range(2):
        for b in range(nblocks):
            for c in range(9):
                ref = s.field(b, c)
                got = s.field_noalloc(b, c)
                # float -> double widening is exact: the tolerance is zero
                assert np.array_equal(got, ref), (b, c, np.abs(got - ref).max())


@pytest.mark.parametrize("prec", ["fp32c", "fp64"])
def test_noalloc_matches_get_field(ctx, wqlmod, tmp_path, prec):
    p = write(tmp_path, "cart.in", golden_in("test_rup_cart_fric"))
    s = wqlmod.Scenario(ctx, p, precision=wqlmod.FP32C if prec == "fp32c" else wqlmod.FP64)
    s.step(5)
    _check(s)
    s.step(1)
    _check(s)


def test_noalloc_pitched_rows(ctx, wqlmod):
    import wql_configs
    text, media = wql_configs.config1(n=45, steps=4)   # nq = 45, row pitch 48 in FP32
    s = wqlmod.Scenario(ctx, text=text, precision=wqlmod.FP32C, media=media)
    s.step(3)
    _check(s)
