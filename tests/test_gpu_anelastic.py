"""The anelastic response (response = 'anelastic') on the GPU against the
oracle: FP64 fields to 1e-11 relative L2, with PML slabs (whose strain
rates lose the damped auxiliary fields), both operators and both meshes;
the FP32-compensated mode against FP64."""
import numpy as np
import pytest

from gpu_helpers import field_errors, rel_l2, run_pair
from inputs import case_text, write

pytestmark = pytest.mark.gpu
TOL = 1e-11


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


@pytest.mark.parametrize("case,steps", [("an_pml", 30), ("an_pml_curv", 20), ("an_mt4", 30),
                                        ("an0_mt4_curv", 20), ("an_up_pml", 30), ("an_up_mt4_curv", 20),
                                        ("an_up5_pml", 30)])
def test_anelastic_fp64_parity(ctx, wqlmod, oracle_lib, tmp_path, case, steps):
    p = write(tmp_path, case + ".in", case_text(case))
    s, o = run_pair(wqlmod, oracle_lib, ctx, p, steps)
    errs = field_errors(s, o)
    assert max(errs) < TOL, errs


@pytest.mark.parametrize("case,steps", [("an_pml", 40), ("an_up_pml", 40), ("an_mt4_curv", 20)])
def test_anelastic_fp32c_vs_fp64(ctx, wqlmod, tmp_path, case, steps):
    p = write(tmp_path, case + ".in", case_text(case))
    d = wqlmod.Scenario(ctx, p, precision=wqlmod.FP64)
    f = wqlmod.Scenario(ctx, p, precision=wqlmod.FP32C)
    d.step(steps)
    f.step(steps)
    f.sync(check_nan=True)
    for b in range(2):
        assert rel_l2(f.fields(b), d.fields(b)) < 1e-5


def test_anelastic_unsupported_weight_set(ctx, wqlmod, tmp_path):
    p = write(tmp_path, "w.in", case_text("an_mt4").replace("weight_exp = 0.6d0", "weight_exp = 0.3d0"))
    with pytest.raises(Exception, match="weight_exp"):
        wqlmod.Scenario(ctx, p)


@pytest.mark.parametrize("case,steps", [("an_pml_curv", 20), ("an_up_mt4", 30)])
def test_anelastic_gradient_handoff(ctx, wqlmod, tmp_path, case, steps):
    """FP32C: the anelastic kernel fed the TMA stencil's velocity gradient
    against the per-point stencil run, where it forms the gradient itself."""
    p = write(tmp_path, case + ".in", case_text(case))
    f = wqlmod.Scenario(ctx, p, precision=wqlmod.FP32C)
    g = wqlmod.Scenario(ctx, p, precision=wqlmod.FP32C)
    g.set_tuning(1, 0)
    f.step(steps)
    g.step(steps)
    f.sync(check_nan=True)
    for b in range(2):
        assert rel_l2(f.fields(b), g.fields(b)) < 1e-6


def test_anelastic_in_batch_equals_alone(ctx, wqlmod, tmp_path):
    """An anelastic scenario stepped in a packed batch (the batched TMA
    stencil also hands it the gradient) gives the fields it gives alone."""
    p = write(tmp_path, "a.in", case_text("an_pml_curv"))
    q = write(tmp_path, "b.in", case_text("pml_curv"))
    alone = wqlmod.Scenario(ctx, p, precision=wqlmod.FP32C)
    alone.step(10)
    a = wqlmod.Scenario(ctx, p, precision=wqlmod.FP32C)
    b = wqlmod.Scenario(ctx, q, precision=wqlmod.FP32C)
    bt = wqlmod.Batch(ctx)
    bt.add(a)
    bt.add(b)
    bt.step(10)
    for k in range(2):
        assert np.array_equal(a.fields(k), alone.fields(k))
    bt.close()
