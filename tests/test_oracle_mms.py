"""Manufactured-solution convergence of the oracle (CPU).

The reference's MMS module (src/mms.f90) is never called and its norm
routine returns |F| instead of the error (src/fields.f90:194-218), so the
convergence test is new: the forcing of src/mms.f90:100-126 is added at every
stage, and the exact solution enters the outer SAT and the locked interface
as the reference's hooks intend (src/BoundaryConditions.f90:86-92, 126;
src/CouplingForcing.f90:147-185).  On a curvilinear two-block grid with a
nonflat fault and topography, the SBP-6 scheme (interior order 6, boundary
closures order 3) must converge at an observed L2 order between 4 and 6.
"""
import numpy as np
import pytest

from inputs import mms_case, mms_relative_error

SIZES = (21, 31, 41)


def _errors(oracle_lib, mesh):
    out = []
    for n in SIZES:
        text, media = mms_case(n, mesh=mesh)
        o = oracle_lib.Oracle(text=text, media=media)
        o.step(o.nt)
        out.append((2.0 / (n - 1), mms_relative_error(o)))
    return out


@pytest.mark.parametrize("mesh", ["curvilinear", "cartesian"])
def test_mms_convergence_order(oracle_lib, mesh):
    errs = _errors(oracle_lib, mesh)
    orders = [np.log(e1 / e2) / np.log(h1 / h2) for (h1, e1), (h2, e2) in zip(errs, errs[1:])]
    print(mesh, ["%.3e" % e for _, e in errs], ["%.2f" % p for p in orders])
    assert errs[-1][1] < 5e-3
    for p in orders:
        assert 4.0 <= p <= 6.0, orders


def test_mms_initial_state_is_exact(oracle_lib):
    """At t = 0 the fields are the manufactured solution (error 0) and the
    first step leaves an error at the level of the scheme's truncation."""
    text, media = mms_case(21)
    o = oracle_lib.Oracle(text=text, media=media)
    assert mms_relative_error(o) == 0.0
    o.step(1)
    assert 0.0 < mms_relative_error(o) < 1e-2


def test_mms_rejects_friction(oracle_lib):
    text, media = mms_case(21)
    with pytest.raises(RuntimeError, match="use_mms"):
        oracle_lib.Oracle(text=text.replace("coupling = 'locked'", "coupling = 'slip-weakening_friction'"),
                          media=media)
