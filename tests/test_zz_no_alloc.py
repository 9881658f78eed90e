"""wql_get_field_noalloc (fixed device scratch, no allocation) against
wql_get_field on the same scenario state, two calls in a row each; FP32C
(widened through the scratch, including a block whose row pitch differs from
nq) and FP64; the device's free memory is unchanged by a batch of calls, and
an FP32 block whose plane exceeds the scratch is refused.  Collected last so
it also runs after every other GPU test."""
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


def _device_free_bytes():
    """Free device memory from the driver (cuMemGetInfo of the context the
    library made current on this thread)."""
    import ctypes
    drv = ctypes.CDLL("libcuda.so.1")
    free, total = ctypes.c_size_t(), ctypes.c_size_t()
    assert drv.cuMemGetInfo_v2(ctypes.byref(free), ctypes.byref(total)) == 0
    return free.value


@pytest.mark.parametrize("prec", ["fp32c", "fp64"])
def test_noalloc_leaves_device_memory_unchanged(ctx, wqlmod, tmp_path, prec):
    """A batch of calls changes the device's free memory by nothing: no
    allocation is made (or cached) by the entry point."""
    p = write(tmp_path, "cart.in", golden_in("test_rup_cart_fric"))
    s = wqlmod.Scenario(ctx, p, precision=wqlmod.FP32C if prec == "fp32c" else wqlmod.FP64)
    s.step(2)
    s.field_noalloc(0, 0)  # first call on the device: resolves the array's address
    before = _device_free_bytes()
    for _ in range(5):
        for b in range(2):
            for c in range(9):
                s.field_noalloc(b, c)
    assert _device_free_bytes() == before


def test_noalloc_rejects_planes_over_the_limit(ctx, wqlmod):
    """An FP32 block whose pitched plane (1028 x 1021 points) exceeds the
    2^20-point array is refused with WQL_E_INPUT; FP64 has no limit."""
    text = f"""&problem_list
 name = 'wide', problem = 'TPV5', nblocks = 2, t_final = 0d0, CFL = 0.5d0,
 coupling = 'locked', type_of_mesh = 'cartesian', w_stride = 1, w_fault = F /
&block_list
btp(1)%nqrs = 1025, 1021, 13,
btp(1)%aqrs = -10.24d0, 0d0, -0.06d0,
btp(1)%bqrs = 0d0, 10.2d0, 0.06d0,
btp(1)%rho_s_p = 2.67d0, 3.464d0, 6d0,
btp(1)%lqrs = 1, 2, 1,
btp(1)%rqrs = 0, 1, 1,
btp(2)%nqrs = 13, 1021, 13,
btp(2)%aqrs = 0d0, 0d0, -0.06d0,
btp(2)%bqrs = 0.12d0, 10.2d0, 0.06d0,
btp(2)%rho_s_p = 2.67d0, 3.464d0, 6d0,
btp(2)%lqrs = 0, 2, 1,
btp(2)%rqrs = 1, 1, 1 /
"""
    s = wqlmod.Scenario(ctx, text=text, precision=wqlmod.FP32C)
    with pytest.raises(wqlmod.WqlError) as ei:
        s.field_noalloc(0, 0)
    assert ei.value.code == 1  # WQL_E_INPUT
    s.field_noalloc(1, 0)      # block 2's plane (16 x 1021) fits
    s.close()


def test_noalloc_pitched_rows(ctx, wqlmod):
    import wql_configs
    text, media = wql_configs.config1(n=45, steps=4)   # nq = 45, row pitch 48 in FP32
    s = wqlmod.Scenario(ctx, text=text, precision=wqlmod.FP32C, media=media)
    s.step(3)
    _check(s)
