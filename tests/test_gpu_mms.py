"""Manufactured-solution convergence of the CUDA path (FP64 and FP32C).

The same problem as tests/test_oracle_mms.py: the forcing of
src/mms.f90:100-126 on every grid point at each stage, the exact solution in
the outer SAT and the locked interface, on a curvilinear two-block grid with
a seeded nonflat fault and topography.  FP64 matches the oracle to 1e-11 and
converges at an observed L2 order between 4 and 6; FP32C follows FP64 to
1e-5 relative L2 in the fields at every size.
"""
import numpy as np
import pytest

from gpu_helpers import rel_l2
from inputs import mms_case, mms_relative_error

pytestmark = pytest.mark.gpu
SIZES = (21, 31, 41)


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


@pytest.mark.parametrize("mesh", ["curvilinear", "cartesian"])
def test_mms_fp64_matches_oracle(ctx, wqlmod, oracle_lib, mesh):
    text, media = mms_case(21, mesh=mesh)
    s = wqlmod.Scenario(ctx, text=text, media=media, precision=wqlmod.FP64)
    o = oracle_lib.Oracle(text=text, media=media)
    n = s.info().nt
    s.step(n)
    s.sync(check_nan=True)
    o.step(n)
    for b in range(2):
        assert rel_l2(s.fields(b), o.fields(b)) < 1e-11
    assert abs(mms_relative_error(s) / mms_relative_error(o) - 1.0) < 1e-9


def test_mms_convergence_fp64_and_fp32c(ctx, wqlmod):
    errs = {wqlmod.FP64: [], wqlmod.FP32C: []}
    for n in SIZES:
        text, media = mms_case(n)
        runs = {}
        for prec in errs:
            s = wqlmod.Scenario(ctx, text=text, media=media, precision=prec)
            s.step(s.info().nt)
            s.sync(check_nan=True)
            errs[prec].append((2.0 / (n - 1), mms_relative_error(s)))
            runs[prec] = s
        for b in range(2):
            assert rel_l2(runs[wqlmod.FP32C].fields(b), runs[wqlmod.FP64].fields(b)) < 1e-5
        for s in runs.values():
            s.close()
    for prec, e in errs.items():
        orders = [np.log(e1 / e2) / np.log(h1 / h2) for (h1, e1), (h2, e2) in zip(e, e[1:])]
        print(prec, ["%.3e" % v for _, v in e], ["%.2f" % p for p in orders])
        for p in orders:
            assert 4.0 <= p <= 6.0, (prec, orders)
