"""The oracle's upwind SBP operators of orders 6 and 5 (fd_type = 'upwind',
src/JU_xJU_yJU_z6.f90:2680-3706, 17675-17983; 2049-2677, 17364-17671).  The reference holds no
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


def test_upwind_other_orders_rejected(oracle_lib):
    text = case_text("up_pml").replace("order = 6", "order = 4")
    with pytest.raises(Exception, match="not restated"):
        oracle_lib.Oracle(text=text)


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
