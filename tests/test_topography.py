"""Free-surface topography read from files (use_topography = T,
src/grid.f90:1349-1875): the oracle's restatement and the library's host
grid generator.  The reference ships no run with topography, so the grid is
pinned by its defining properties: the top face and the fault face are the
files' surfaces, a flat topography file gives the flat curvilinear grid, and
the library's grid equals the oracle's."""
import os

import numpy as np
import pytest

from inputs import golden_in, set_key, topography_case, write


def _grid(o, b):
    return np.stack([o.geom(b, c) for c in range(3)])  # (3, ns, nr, nq)


def test_flat_topography_file_gives_the_flat_grid(oracle_lib, tmp_path):
    text = topography_case(tmp_path, amp=0.0, fault_file=False)
    o = oracle_lib.Oracle(write(tmp_path, "topo.in", text))
    flat = set_key(golden_in("test_rup_cart_fric"), "type_of_mesh", "'curvilinear'")
    f = oracle_lib.Oracle(write(tmp_path, "flat.in", flat))
    for b in range(2):
        assert np.abs(_grid(o, b) - _grid(f, b)).max() < 1e-13


def test_surfaces_follow_the_files(oracle_lib, tmp_path):
    text = topography_case(tmp_path)
    o = oracle_lib.Oracle(write(tmp_path, "topo.in", text))
    n = 21
    for b in range(2):
        rows = np.loadtxt(os.path.join(str(tmp_path), f"topo_{b + 1}.dat")).reshape(n, n, 3)  # (i, k, xyz)
        g = _grid(o, b)
        top = g[:, :, 0, :]  # (3, k, i) on j = 1
        assert np.abs(top[0] - rows[:, :, 0].T).max() < 1e-14
        assert np.abs(top[1] - (6.0 + rows[:, :, 1].T)).max() < 1e-14
        assert np.abs(top[2] - rows[:, :, 2].T).max() < 1e-14
        assert np.abs(rows[:, :, 1]).max() > 0.02
    fault = np.loadtxt(os.path.join(str(tmp_path), "fault.dat")).reshape(n, n, 3)  # (k, j, xyz)
    for b, iq in ((0, -1), (1, 0)):
        g = _grid(o, b)[:, :, :, iq]  # (3, k, j)
        for c in range(3):
            assert np.abs(g[c] - fault[:, :, c]).max() < 1e-14


def test_library_grid_equals_the_oracle(oracle_lib, tmp_path):
    import wql
    text = topography_case(tmp_path)
    o = oracle_lib.Oracle(write(tmp_path, "topo.in", text))
    out = tmp_path / "grids"
    out.mkdir()
    wql.write_block_grids(text, str(out), base_dir=str(tmp_path))
    for b in range(2):
        g = _grid(o, b)
        for c, ext in enumerate("XYZ"):
            x = np.fromfile(str(out / f"block_grid_{b + 1}.{ext}"), dtype=np.float64).reshape(g[c].shape)
            assert np.abs(x - g[c]).max() < 1e-12, (b, ext)


def test_topography_run_is_finite_and_departs_from_flat(oracle_lib, tmp_path):
    text = topography_case(tmp_path)
    o = oracle_lib.Oracle(write(tmp_path, "topo.in", text))
    f = oracle_lib.Oracle(write(tmp_path, "flat.in", set_key(golden_in("test_rup_cart_fric"), "type_of_mesh",
                                                             "'curvilinear'")))
    o.step(10)
    f.step(10)
    a, b = o.fields(0), f.fields(0)
    assert np.isfinite(a).all()
    assert np.linalg.norm(a - b) > 1e-3 * np.linalg.norm(b)


def test_unknown_topography_type_is_refused(oracle_lib, tmp_path):
    text = topography_case(tmp_path).replace("'read_topo_from_memory'", "'spline'")
    with pytest.raises(RuntimeError, match="topography"):
        oracle_lib.Oracle(write(tmp_path, "bad.in", text))
