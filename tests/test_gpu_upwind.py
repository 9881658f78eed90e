"""The upwind SBP operators on the GPU against the oracle: orders 6 and 5
(fd_type = 'upwind'), and the table operators (upwind orders 2, 3, 4, 7, 8,
9 and upwind_drp orders 3..7, 66, 679).  FP64 fields to 1e-11 relative L2
(rate and state to its solver tolerance), and the FP32-compensated mode
against FP64 to 1e-5."""
import numpy as np
import pytest

from gpu_helpers import field_errors, rel_l2, rs_close, run_pair
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


@pytest.mark.parametrize("case,steps", [("up_pml", 40), ("up_pml_curv", 20), ("up_plastic", 46),
                                        ("up_rs_curv", 20), ("up_mt4", 30), ("up_mt4_curv", 20),
                                        ("up5_pml", 40), ("up5_pml_curv", 20), ("up5_mt4_curv", 20)])
def test_upwind_fp64_parity(ctx, wqlmod, oracle_lib, tmp_path, case, steps):
    p = write(tmp_path, case + ".in", case_text(case))
    s, o = run_pair(wqlmod, oracle_lib, ctx, p, steps)
    errs = field_errors(s, o)
    if "_rs" in case:
        for b in range(2):
            assert rs_close(s.fields(b), o.fields(b)), errs
    else:
        assert max(errs) < TOL, errs
    # and the run differs from the traditional operator's
    t = wqlmod.Scenario(ctx, write(tmp_path, "t.in", case_text(case.split("_", 1)[1])))
    t.step(steps)
    assert rel_l2(t.fields(0), s.fields(0)) > 1e-6


@pytest.mark.parametrize("case,steps", [("up_pml", 40), ("up_pml_curv", 20), ("up_mt4_curv", 20),
                                        ("up5_pml_curv", 20)])
def test_upwind_fp32c_vs_fp64(ctx, wqlmod, tmp_path, case, steps):
    p = write(tmp_path, case + ".in", case_text(case))
    d = wqlmod.Scenario(ctx, p, precision=wqlmod.FP64)
    f = wqlmod.Scenario(ctx, p, precision=wqlmod.FP32C)
    d.step(steps)
    f.step(steps)
    f.sync(check_nan=True)
    for b in range(2):
        assert rel_l2(f.fields(b), d.fields(b)) < 1e-5


def _mt_text(n, mesh):
    from inputs import MT_CASES, block_list, problem
    _, order, _, lists = MT_CASES["mt4"]
    t = (problem("TPV5", "locked", mesh) + block_list(n) +
         f"&moment_list\n use_moment_tensor = T,\n order = {order} /\n" + lists)
    return t.replace(" w_stride = 1,", " w_stride = 1,\n fd_type = 'upwind',\n order = 6,", 1)


@pytest.mark.parametrize("case,steps", [("up_pml", 40), ("up_pml_curv", 20), ("n16_cartesian", 30),
                                        ("n16_curvilinear", 20), ("n17_curvilinear", 20)])
def test_upwind_tma_vs_pointwise(ctx, wqlmod, tmp_path, case, steps):
    """FP32C: the TMA kernel with the upwind pair (its PML gradient handed to
    the PML kernel) against the per-point kernel.  n = 16 puts the last r
    tile at 4, so it owns left closure rows read from its 4-row halo; n = 17
    (last tile at 5) runs per point in both."""
    text = case_text(case) if case.startswith("up_") else _mt_text(int(case[1:3]), case[4:])
    p = write(tmp_path, case + ".in", text)
    f = wqlmod.Scenario(ctx, p, precision=wqlmod.FP32C)
    g = wqlmod.Scenario(ctx, p, precision=wqlmod.FP32C)
    g.set_tuning(1, 0)
    d = wqlmod.Scenario(ctx, p, precision=wqlmod.FP64)
    for s in (f, g, d):
        s.step(steps)
    f.sync(check_nan=True)
    for b in range(2):
        assert rel_l2(f.fields(b), g.fields(b)) < 1e-6
        assert rel_l2(f.fields(b), d.fields(b)) < 1e-5


def test_upwind_in_batch_equals_alone(ctx, wqlmod, tmp_path):
    """An upwind scenario stepped in a batch next to a traditional one gives
    the same fields as stepped alone (its stencil stays outside the packed
    launch, which runs the central operator)."""
    pu = write(tmp_path, "u.in", case_text("up_pml_curv"))
    pt = write(tmp_path, "t.in", case_text("pml_curv"))
    alone = wqlmod.Scenario(ctx, pu, precision=wqlmod.FP32C)
    alone.step(10)
    a = wqlmod.Scenario(ctx, pu, precision=wqlmod.FP32C)
    b = wqlmod.Scenario(ctx, pt, precision=wqlmod.FP32C)
    bt = wqlmod.Batch(ctx)
    bt.add(a)
    bt.add(b)
    bt.step(10)
    for k in range(2):
        assert np.array_equal(a.fields(k), alone.fields(k))
    bt.close()


def test_upwind_unknown_orders_rejected(ctx, wqlmod, tmp_path):
    p = write(tmp_path, "u10.in", case_text("up_pml").replace("order = 6", "order = 10"))
    with pytest.raises(Exception, match="not supported"):
        wqlmod.Scenario(ctx, p)


# The table operators (orders 2, 3, 4, 7, 8, 9 and the DRP variants, read from
# the reference's routines by oracle/make_upwind_tables.py), per point.
TABLE_OPS = [("upwind", o) for o in (2, 3, 4, 7, 8, 9)] + [("upwind_drp", o) for o in (3, 4, 5, 6, 7, 66, 679)]


def _op_text(fd, order, base):
    return case_text(base).replace(" w_stride = 1,", f" w_stride = 1,\n fd_type = '{fd}',\n order = {order},", 1)


@pytest.mark.parametrize("fd,order", TABLE_OPS)
def test_table_operator_fp64_parity(ctx, wqlmod, oracle_lib, tmp_path, fd, order):
    """A point source in a locked two-block domain (2 x 21^3): FP64 fields
    against the oracle to 1e-11."""
    p = write(tmp_path, "op.in", _op_text(fd, order, "mt4"))
    s, o = run_pair(wqlmod, oracle_lib, ctx, p, 30)
    assert max(field_errors(s, o)) < TOL


@pytest.mark.parametrize("fd,order,base,steps", [("upwind", 2, "pml_curv", 20), ("upwind", 4, "pml", 30),
                                                 ("upwind", 8, "pml_curv", 20), ("upwind_drp", 66, "pml_curv", 20),
                                                 ("upwind_drp", 679, "pml", 30), ("upwind", 3, "an_pml", 20),
                                                 ("upwind_drp", 66, "an_pml", 20)])
def test_table_operator_pml_anelastic_parity(ctx, wqlmod, oracle_lib, tmp_path, fd, order, base, steps):
    """PML slabs (7 points, inside and outside the closure rows) on Cartesian
    and curvilinear grids, and the anelastic response: FP64 against the
    oracle to 1e-11, FP32C against FP64 to 1e-5.  upwind_drp 66 uses the
    interior routine's stencil inside the block and the near-boundary
    routine's on the shell, as the reference does."""
    p = write(tmp_path, "op.in", _op_text(fd, order, base))
    s, o = run_pair(wqlmod, oracle_lib, ctx, p, steps)
    assert max(field_errors(s, o)) < TOL
    f = wqlmod.Scenario(ctx, p, precision=wqlmod.FP32C)
    f.step(steps)
    f.sync(check_nan=True)
    for b in range(2):
        assert rel_l2(f.fields(b), s.fields(b)) < 1e-5


@pytest.mark.parametrize("op", ["upwind", "central"])
def test_wide_tiles_equal_32_wide(ctx, wqlmod, tmp_path, op):
    """Cartesian blocks of 38 points along q fill one 40-wide TMA tile (95 %
    of its columns) better than two 32-wide ones (59 %): variant 5 takes the
    wide tiles, variant 6 the 32-wide ones, and the fields agree bit for bit
    (the per-point arithmetic is the same; only the tiling differs), with
    PML slabs on five sides and the velocity-gradient hand-off."""
    from inputs import PML_BLOCKS, block_list, problem
    extra = ",\n fd_type = 'upwind',\n order = 6" if op == "upwind" else ""
    text = problem(extra=extra, t_final="5d0") + block_list(38, **PML_BLOCKS)
    p = write(tmp_path, "wide.in", text)
    a = wqlmod.Scenario(ctx, p, precision=wqlmod.FP32C)
    b = wqlmod.Scenario(ctx, p, precision=wqlmod.FP32C)
    b.set_tuning(6, 0)
    a.step(25)
    b.step(25)
    a.sync(check_nan=True)
    b.sync(check_nan=True)
    for blk in range(2):
        np.testing.assert_array_equal(a.fields(blk), b.fields(blk))
    np.testing.assert_array_equal(a.iface(0, 3), b.iface(0, 3))
    # back to the wide tiles: still the same
    b.set_tuning(5, 0)
    a.step(5)
    b.step(5)
    np.testing.assert_array_equal(a.fields(0), b.fields(0))
