"""Shared helpers for the GPU parity tests (CUDA path vs the oracle)."""
import numpy as np


def rel_l2(a, b):
    den = np.linalg.norm(b)
    return np.linalg.norm(a - b) / (den if den > 0 else 1.0)


def run_pair(wql, oracle_lib, ctx, path, steps, precision=0):
    s = wql.Scenario(ctx, path, precision=precision)
    o = oracle_lib.Oracle(path)
    s.step(steps)
    s.sync(check_nan=True)
    o.step(steps)
    return s, o


def field_errors(s, o):
    return [rel_l2(s.fields(b), o.fields(b)) for b in range(2)]


def rs_close(a, b, rel=1e-7, floor=1e-9):
    """Rate-and-state comparison.  The reference's Regula-Falsi stops once
    |dV| < 1e-12 m/s (src/Interface_Condition.f90:1188-1194), so slip rates
    -- and the fields they drive -- are defined only to about that level;
    errors are bounded relative to the field plus an absolute floor of
    1e-9 per point (1000x the solver tolerance)."""
    return np.linalg.norm(a - b) <= rel * np.linalg.norm(b) + floor * np.sqrt(b.size)
