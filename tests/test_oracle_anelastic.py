"""The oracle's anelastic response (response = 'anelastic', four relaxation
mechanisms per stress component, src/material.f90:11-142,
src/RHS_Interior.f90:2390-2509).  The reference holds no output of an
anelastic run, so the restatement is checked by its limits: as the quality
factor grows (c -> infinity) the run tends to the elastic one, the
difference falling as 1/Q; unsupported weight sets are refused."""
import numpy as np
import pytest

from gpu_helpers import rel_l2
from inputs import case_text


def _run(oracle_lib, text, steps):
    o = oracle_lib.Oracle(text=text)
    o.step(steps)
    return [o.fields(b) for b in range(2)]


def test_elastic_limit_and_q_scaling(oracle_lib):
    el = _run(oracle_lib, case_text("mt4"), 30)
    an = case_text("an_mt4")
    d = {}
    for c in ("1d3", "1d4", "1d12"):
        f = _run(oracle_lib, an.replace("c = 2.0d0", f"c = {c}"), 30)
        assert all(np.isfinite(x).all() for x in f)
        d[c] = max(rel_l2(f[b], el[b]) for b in range(2))
    assert d["1d12"] < 1e-11
    ratio = d["1d3"] / d["1d4"]
    assert 8.0 < ratio < 12.5, d


def test_attenuation_changes_the_run(oracle_lib):
    for case in ("pml", "up_pml"):
        el = _run(oracle_lib, case_text(case), 20)
        an = _run(oracle_lib, case_text("an_" + case), 20)
        for b in range(2):
            assert np.isfinite(an[b]).all()
            assert 1e-3 < rel_l2(an[b], el[b]) < 0.5


def test_unsupported_weight_set_refused(oracle_lib):
    text = case_text("an_mt4").replace("weight_exp = 0.6d0", "weight_exp = 0.3d0")
    with pytest.raises(Exception, match="weight_exp"):
        oracle_lib.Oracle(text=text)
