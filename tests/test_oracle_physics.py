"""Self-consistency checks of the oracle on the physics the reference's
fixtures do not pin (rate and state, PML): mirror symmetry of a rupture
that is symmetric in z, and PML absorption and long-run stability.  CPU
only; the GPU is compared with the oracle elsewhere."""
import numpy as np
import pytest

from inputs import PML_BLOCKS, block_list, problem


def test_rate_state_mirror_symmetry(oracle_lib):
    """TPV101 nucleates at z = 0 on blocks symmetric about z = 0, with the same
    boundary on both z sides, and its loading flips sign with z only through
    the shear component: slip, state and rupture time are even in z, and
    every field component is either even or odd in z (to rounding)."""
    o = oracle_lib.Oracle(text=problem("TPV101", "rate-and-state_friction", t_final="3.0d0") + block_list())
    o.step(90)
    for copy in range(2):
        for what in (3, 4, 5):  # slip magnitude, state, rupture time
            a = o.iface(copy, what)
            scale = max(np.abs(a).max(), 1e-30)
            assert np.abs(a - a[::-1, :]).max() <= 1e-8 * scale, (copy, what)
    slip = o.iface(0, 3)
    assert slip.max() > 1e-3 * np.abs(slip).max() and slip.max() > 0  # it slipped
    for b in range(2):
        F = o.fields(b)
        for c in range(9):
            scale = max(np.abs(F[c]).max(), 1e-30)
            even = np.abs(F[c] - F[c, ::-1]).max()
            odd = np.abs(F[c] + F[c, ::-1]).max()
            assert min(even, odd) <= 1e-8 * scale, (b, c, even / scale, odd / scale)


def _pulse_run(oracle_lib, text, steps):
    """Locked interface, a Gaussian velocity pulse in block 1; returns the sum
    of squared velocities of both blocks after each requested step count."""
    o = oracle_lib.Oracle(text=text)
    x, y, z = (o.geom(0, c) for c in range(3))
    r2 = (x + 1.5) ** 2 + (y - 7.5) ** 2 + z ** 2
    o.set_field(0, 0, np.exp(-r2 / 0.09).ravel())
    out, done = [], 0
    for n in steps:
        o.step(n - done)
        done = n
        out.append(sum(float((o.fields(b)[:3] ** 2).sum()) for b in range(2)))
    return out


def test_pml_absorbs_and_stays_bounded(oracle_lib):
    """With PML layers (and absorbing outer faces) the pulse leaves the
    domain: far less velocity energy remains than in the same box with
    free-surface faces, and it keeps decreasing over a long run (no PML
    growth)."""
    steps = (60, 200, 400)
    pml = _pulse_run(oracle_lib, problem("TPV5", "locked") + block_list(25, **PML_BLOCKS), steps)
    free = block_list(25).replace("btp(1)%lqrs = 1, 2, 1,", "btp(1)%lqrs = 2, 2, 2,") \
                         .replace("btp(1)%rqrs = 0, 1, 1,", "btp(1)%rqrs = 0, 2, 2,") \
                         .replace("btp(2)%lqrs = 0, 2, 1,", "btp(2)%lqrs = 0, 2, 2,") \
                         .replace("btp(2)%rqrs = 1, 1, 1,", "btp(2)%rqrs = 2, 2, 2,")
    box = _pulse_run(oracle_lib, problem("TPV5", "locked") + free, steps)
    assert all(np.isfinite(pml)) and all(np.isfinite(box))
    assert pml[1] < 0.05 * box[1]
    assert pml[2] <= pml[1] <= pml[0]
