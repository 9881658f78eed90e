"""The oracle's upwind SBP operators: orders 6 and 5 (fd_type = 'upwind',
src/JU_xJU_yJU_z6.f90:2680-3706, 17675-17983; 2049-2677, 17364-17671)
transcribed, the other orders and the DRP variants as tables read from the
reference's routines (oracle/make_upwind_tables.py).  The reference holds no
output of an upwind run, so the transcribed closure rows are pinned by the
properties that define the operators: the upwind summation-by-parts
identity H D+ + (H D-)^T = diag(-1, 0, ..., 0, 1) with a positive diagonal
norm H, and exactness on polynomials (degree 3 at the closures, 6 inside)."""
import numpy as np
import pytest

from inputs import case_text
from gpu_helpers import rel_l2


def _norm(Dp, Dm):
    """Least-squares diagonal H of H Dp + (H Dm)^T = B and the residual."""
    n = Dp.shape[0]
    B = np.zeros((n, n))
    B[0, 0], B[-1, -1] = -1.0, 1.0
    rows, rhs = [], []
    for i in range(n):
        for j in range(n):
            r = np.zeros(n)
            r[i] += Dp[i, j]
            r[j] += Dm[j, i]
            if r.any() or B[i, j]:
                rows.append(r)
                rhs.append(B[i, j])
    A, b = np.array(rows), np.array(rhs)
    h = np.linalg.lstsq(A, b, rcond=None)[0]
    return h, np.abs(A @ h - b).max()


@pytest.mark.parametrize("n", [12, 13, 30])
def test_upwind_summation_by_parts(oracle_lib, n):
    Dp = oracle_lib.fd_matrix(1, True, n)
    Dm = oracle_lib.fd_matrix(1, False, n)
    h, res = _norm(Dp, Dm)
    assert res < 1e-13
    assert (h > 0).all()
    assert abs(h[0] - 13613.0 / 43200.0) < 1e-12
    assert np.allclose(h, h[::-1], rtol=0, atol=1e-12)
    # the traditional operator: H D + (H D)^T = B with h11 = 13649/43200
    D = oracle_lib.fd_matrix(0, True, n)
    h0, res0 = _norm(D, D)
    assert res0 < 1e-13 and abs(h0[0] - 13649.0 / 43200.0) < 1e-12


def test_upwind_accuracy():
    import oracle_binding as ob
    n = 30
    x = np.arange(n, dtype=np.float64)
    for plus in (True, False):
        D = ob.fd_matrix(1, plus, n)
        for deg in range(7):
            f = x ** deg
            df = deg * x ** (deg - 1) if deg else np.zeros(n)
            err = np.abs(D @ f - df)
            scale = max(1.0, np.abs(df).max())
            assert err[6:-6].max() < 1e-11 * scale, (plus, deg)
            if deg <= 3:
                assert err.max() < 1e-11 * scale, (plus, deg)
        # the interior rows are one-sided: D+ reaches 4 points ahead, D- 4 behind
        row = D[15]
        nz = np.nonzero(row)[0] - 15
        assert (nz.min(), nz.max()) == ((-2, 4) if plus else (-4, 2))


def test_upwind_run_near_traditional(oracle_lib):
    """A moment-tensor source on 2 x 21^3 points: the upwind and traditional
    runs agree to the discretisation difference (a few per cent) and the
    upwind run stays finite."""
    a = oracle_lib.Oracle(text=case_text("mt4"))
    b = oracle_lib.Oracle(text=case_text("up_mt4"))
    a.step(40)
    b.step(40)
    for k in range(2):
        fb = b.fields(k)
        assert np.isfinite(fb).all()
        e = rel_l2(fb, a.fields(k))
        assert 1e-4 < e < 0.1


def test_upwind_unknown_orders_rejected(oracle_lib):
    """The reference has no upwind operator of order 10 (src/block.f90:195-252)."""
    text = case_text("up_pml").replace("order = 6", "order = 10")
    with pytest.raises(Exception, match="not restated"):
        oracle_lib.Oracle(text=text)


# The other upwind operators, read from the reference's routines into tables
# by oracle/make_upwind_tables.py.  Orders 8 and 9 as the reference writes
# them: their D+ closure rows 7 and 8 stop short of the points their mirrored
# D- rows reach (src/JU_xJU_yJU_z6.f90:5264-5276 for order 8, row 8, ends at
# point 11), so those rows do not even differentiate a constant exactly, and
# no diagonal norm makes the pair summation-by-parts; one D- row near the
# right end differs between the axes.  They are restated as written.
NOT_SBP = {("upwind", 8), ("upwind", 9)}


def _inconsistent_rows(fd, order, ax, plus, n):
    """0-based rows that do not differentiate constants and linears exactly,
    as the reference writes the operators: orders 8 and 9 (above), and
    upwind_drp 679, whose closure rows 4..8 and their mirrors have nonzero
    weight sums although the pair is summation-by-parts."""
    if (fd, order) == ("upwind", 8):
        return {6, 7} if plus else ({n - 8} if ax else set())
    if (fd, order) == ("upwind", 9):
        return {6, 7} if plus else ({7, n - 8} if ax else {7})
    if (fd, order) == ("upwind_drp", 679):
        return set(range(3, 8)) | set(range(n - 8, n - 4)) if plus else set(range(4, 8)) | set(range(n - 8, n - 3))
    return set()


def _tables():
    import oracle_binding as ob
    return ob.up_tables()


def test_table_operators_cover_the_reference():
    names = {(fd, o) for fd, o, _, _ in _tables()}
    assert names == {("upwind", o) for o in (2, 3, 4, 5, 6, 7, 8, 9)} | \
        {("upwind_drp", o) for o in (3, 4, 5, 6, 7, 66, 679)}
    tau = {(fd, o): t for fd, o, _, t in _tables()}
    # src/block.f90:195-252
    assert tau[("upwind", 2)] == 4.0 and tau[("upwind", 3)] == 12.0 / 5.0
    assert tau[("upwind", 8)] == 25401600.0 / 7489399.0 and tau[("upwind_drp", 66)] == 1198.0 / 377.0


def test_tables_reproduce_the_order_6_and_5_rows():
    """The tables read from the reference by the generator equal the order-6
    and order-5 rows transcribed into the oracle, on every axis."""
    import oracle_binding as ob
    for k, (fd, o, _, _) in enumerate(_tables()):
        if fd == "upwind" and o in (5, 6):
            for plus in (True, False):
                ref = ob.fd_matrix(1 if o == 6 else 2, plus, 30)
                for ax in range(3):
                    assert np.abs(ob.up_matrix(k, plus, 30, ax) - ref).max() < 1e-15, (o, plus, ax)


@pytest.mark.parametrize("k", range(15))
def test_table_operator_sbp_and_accuracy(k):
    """Each operator as the near-boundary routine forms it: the upwind
    summation-by-parts identity with a positive diagonal norm, exactness to
    degree 1 on every row and to degree 2 inside, the same rows on the three
    axes, and interior rows that lean forward (D+) and backward (D-).  The
    exceptions are exactly those of the reference's tables noted above."""
    import oracle_binding as ob
    fd, order, R, tau0 = _tables()[k]
    n = 2 * R + 20
    Dp, Dm = ob.up_matrix(k, True, n), ob.up_matrix(k, False, n)
    h, res = _norm(Dp, Dm)
    if (fd, order) in NOT_SBP:
        assert res > 1e-3
    else:
        assert res < 1e-12 and (h > 0).all()
        assert np.allclose(h, h[::-1], rtol=0, atol=1e-12)
    x = np.arange(n, dtype=np.float64) / n
    for ax in range(3):
        for plus in (True, False):
            D = ob.up_matrix(k, plus, n, ax)
            bad = set()
            for deg in (0, 1):
                err = np.abs(D @ x ** deg * n - (deg * x ** (deg - 1) if deg else 0.0))
                bad |= {i for i in range(n) if err[i] > 1e-9}
            assert bad == _inconsistent_rows(fd, order, ax, plus, n), (fd, order, plus, ax, sorted(bad))
            err = np.abs(D @ x ** 2 * n - 2 * x)
            assert err[R:n - R].max() < 1e-9  # second order inside
    for ax in (1, 2):
        for plus, D in ((True, Dp), (False, Dm)):
            diff = np.abs(ob.up_matrix(k, plus, n, ax) - D)
            if (fd, order) in NOT_SBP:
                assert (diff > 1e-12).sum() <= 2  # the one D- entry the q axis has in addition
            else:
                assert diff.max() == 0.0
    mid = n // 2
    # D+ leans forward, D- backward
    assert (np.nonzero(Dp[mid])[0] - mid).sum() > 0 > (np.nonzero(Dm[mid])[0] - mid).sum()


def test_drp_interior_routines_differ_for_66_and_679():
    """upwind_drp 66 and 679: the interior routine's stencil is not the
    near-boundary routine's interior case (both are kept, each where the
    reference applies it); for the other operators they agree to rounding."""
    import oracle_binding as ob
    for k, (fd, o, R, _) in enumerate(_tables()):
        n = 2 * R + 20
        a = ob.up_matrix(k, True, n, interior=False)[n // 2]
        b = ob.up_matrix(k, True, n, interior=True)[n // 2]
        if fd == "upwind_drp" and o in (66, 679):
            assert np.abs(a - b).max() > 1e-4
        else:
            assert np.abs(a - b).max() < 1e-14


@pytest.mark.parametrize("fd,order", [("upwind", 2), ("upwind", 4), ("upwind", 8), ("upwind_drp", 3),
                                      ("upwind_drp", 66), ("upwind_drp", 679)])
def test_table_operator_runs(oracle_lib, fd, order):
    """A moment-tensor source on 2 x 21^3 points with the operator: finite,
    and within the discretisation difference of the traditional run."""
    text = case_text("mt4").replace(" w_stride = 1,", f" w_stride = 1,\n fd_type = '{fd}',\n order = {order},", 1)
    a = oracle_lib.Oracle(text=case_text("mt4"))
    b = oracle_lib.Oracle(text=text)
    a.step(30)
    b.step(30)
    for blk in range(2):
        fb = b.fields(blk)
        assert np.isfinite(fb).all()
        assert rel_l2(fb, a.fields(blk)) < 0.5


@pytest.mark.parametrize("n", [12, 30])
def test_upwind5_summation_by_parts(oracle_lib, n):
    """Order 5: the same identity with h11 = 251/720 = 1/tau0, exactness of
    degree 2 at the closures and 5 inside, one-sided reach of 3 points."""
    Dp = oracle_lib.fd_matrix(2, True, n)
    Dm = oracle_lib.fd_matrix(2, False, n)
    h, res = _norm(Dp, Dm)
    assert res < 1e-13 and (h > 0).all()
    assert abs(h[0] - 251.0 / 720.0) < 1e-12
    x = np.arange(n, dtype=np.float64)
    for D in (Dp, Dm):
        for deg in range(6):
            f = x ** deg
            df = deg * x ** (deg - 1) if deg else np.zeros(n)
            err = np.abs(D @ f - df)
            scale = max(1.0, np.abs(df).max())
            assert err[4:-4].max() < 1e-11 * scale
            if deg <= 2:
                assert err.max() < 1e-11 * scale
    nz = np.nonzero(Dp[n // 2])[0] - n // 2
    assert (nz.min(), nz.max()) == (-2, 3)
    nz = np.nonzero(Dm[n // 2])[0] - n // 2
    assert (nz.min(), nz.max()) == (-3, 2)
