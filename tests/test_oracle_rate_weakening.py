"""The oracle's problem 'rate-weakening' and its default plastic model
(plastic_flow), checked on the CPU: the uniform initial stress
(src/initial_stress_condition.f90:184-193), the implicit relation the
closed-form plastic update satisfies at every yielding point
(src/plastic.f90:245-271: eta*lambda = Y(s) after the update), the plastic
strain accumulating as dt*lambda, and the rejection of plastic_flow for
problems that leave mu_beta_eta undefined."""
import math

import numpy as np
import pytest

from inputs import case_text

MU, BETA, ETA = 0.5735, 0.2867, 0.2775


def rw_s0():
    psi = 50.0 / 180.0 * 3.14159265359
    s0 = np.zeros(6)
    s0[0], s0[4] = -126.0, 42.0
    s0[2] = (1.0 - 2.0 * s0[4] / (s0[0] * math.tan(2.0 * psi))) * s0[0]
    s0[1] = 0.5 * (s0[0] + s0[2])
    return s0


def invariants(sa):
    sigma = (sa[0] + sa[1] + sa[2]) / 3.0
    J2 = ((sa[0] - sa[1]) ** 2 + (sa[1] - sa[2]) ** 2 + (sa[2] - sa[0]) ** 2) / 6.0 + sa[3] ** 2 + sa[4] ** 2 + sa[5] ** 2
    return np.sqrt(J2), sigma


def test_initial_stress_below_yield():
    """The uniform tensor is below the plastic_flow yield surface
    (Y = tau + mu*sigma < 0): yielding comes only from the rupture."""
    tau, sigma = invariants(rw_s0())
    assert tau + MU * sigma < -20.0


def test_plastic_flow_consistency(oracle_lib):
    o = oracle_lib.Oracle(text=case_text("rw_plastic"))
    dt = None
    gam_prev = [np.zeros_like(o.field(b, 10)) for b in range(2)]
    yielded = 0
    for step in range(1, 41):
        o.step(1)
        for b in range(2):
            lam, gam = o.field(b, 9), o.field(b, 10)
            if dt is None and (lam > 0).any():
                # the time step from the first increment of gammap
                k = np.argmax(lam)
                dt = (gam.flat[k] - gam_prev[b].flat[k]) / lam.flat[k]
            if dt is not None:
                # gammap grows by dt*lambda where the point yields, and not elsewhere
                np.testing.assert_allclose(gam, gam_prev[b] + dt * lam, rtol=1e-12, atol=1e-14)
            y = lam > 0
            yielded += int(y.sum())
            if y.any():
                s0 = rw_s0()
                F = o.fields(b)
                sa = [F[3 + c][y] + s0[c] for c in range(6)]
                tau, sigma = invariants(sa)
                # after the update the yield function equals eta*lambda
                np.testing.assert_allclose(tau + MU * sigma, ETA * lam[y], rtol=1e-9, atol=1e-9)
            gam_prev[b] = gam
    assert dt is not None and yielded > 100


def test_rate_weakening_nucleates_and_ruptures(oracle_lib):
    """The Gaussian pulse (twice 0.2429 |Tn| at (y, z) = (8, 0) for t > 0,
    src/Interface_Condition.f90:2387-2423) starts the rupture; the state
    variable starts at 0.4367 everywhere (:2819-2843)."""
    o = oracle_lib.Oracle(text=case_text("rw"))
    np.testing.assert_array_equal(o.iface(0, 4), 0.4367)
    o.step(30)
    trup = o.iface(0, 5)
    assert (trup < 1e8).sum() > 300
    assert np.all(o.iface(0, 4) != 0.4367)


def test_plastic_flow_needs_rate_weakening(oracle_lib):
    text = case_text("plastic").replace("plastic_model = 'scec'", "plastic_model = 'default'")
    with pytest.raises(Exception):
        oracle_lib.Oracle(text=text)
