"""FP64 parity of the CUDA path against the oracle (and the reference's
truth/1 and truth/2 fixtures).  Bar: 1e-11 relative L2 in the fields; fault streams to
float32 rounding of the fixture."""
import os

import numpy as np
import pytest

from gpu_helpers import field_errors, rel_l2, run_pair
from inputs import GOLDEN, golden_in, set_key, with_groups, write

pytestmark = pytest.mark.gpu

WEIGHTED = "&gb300_list\n bc_penalty = 'weighted' /"
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


def test_truth1_fault_streams(ctx, wqlmod, oracle_lib, tmp_path):
    """The GPU FP64 path reproduces test_problems/truth/1 (read_binary.py bar
    1e-3 abs; observed ~1e-12) and the oracle's fields to 1e-11."""
    p = write(tmp_path, "cart.in", with_groups(golden_in("test_rup_cart_fric"), WEIGHTED))
    s, o = run_pair(wqlmod, oracle_lib, ctx, p, 46)
    truth = np.load(os.path.join(GOLDEN, "truth_cart.npz"))
    for name in ["S", "Svel", "Uface", "Vface", "Uhat", "Vhat", "trup", "state"]:
        got = s.frames(name).astype(np.float64)
        ref = truth[name]
        assert got.shape == ref.shape
        scale = max(np.abs(ref).max(), 1.0)
        assert np.abs(got - ref).max() <= 1e-9 * scale, name
    for e in field_errors(s, o):
        assert e < TOL
    # station seismograms: grid points, the oracle's records, and the truth
    # files (printed to 6 decimals)
    for block, name in ((0, "station_21_11_11"), (1, "station_1_11_11")):
        idx, rec = s.stations(block)
        oidx, orec = o.stations(block)
        assert idx.tolist() == oidx.tolist()
        assert rec.shape == orec.shape == (46, 1, 4)
        assert np.abs(rec - orec).max() <= 1e-11 * max(np.abs(orec).max(), 1.0)
        assert np.abs(rec[:, 0, :] - truth[name]).max() <= 5.1e-7


def test_truth2_fault_streams(ctx, wqlmod, oracle_lib, tmp_path):
    """The GPU FP64 path reproduces test_problems/truth/2 (TPV28 on the
    curvilinear bump fault; the fixture's TPV28 tensor has szz = -60 MPa)
    in every frame of the eight fault streams, and the stations placed on
    the bump's crest match truth/2's station files."""
    text = with_groups(golden_in("test_rup_curv_fric"),
                       "&gb300_list\n bc_penalty = 'weighted', tpv28_prestress = 'benchmark' /")
    text = text.replace(" -0d0 7.5d0 0d0", " 0.1d0 7.5d0 0d0").replace(" 0d0 7.5d0 0d0", " 0.1d0 7.5d0 0d0")
    p = write(tmp_path, "curv.in", text)
    s, o = run_pair(wqlmod, oracle_lib, ctx, p, 46)
    truth = np.load(os.path.join(GOLDEN, "truth_curv.npz"))
    for name in ["S", "Svel", "Uface", "Vface", "Uhat", "Vhat", "trup", "state"]:
        got = s.frames(name).astype(np.float64)
        ref = truth[name]
        assert got.shape == ref.shape
        scale = max(np.abs(ref).max(), 1.0)
        assert np.abs(got - ref).max() <= 1e-9 * scale, name
    for e in field_errors(s, o):
        assert e < TOL
    for block, name in ((0, "station_21_11_11"), (1, "station_1_11_11")):
        idx, rec = s.stations(block)
        assert rec.shape == (46, 1, 4)
        assert np.abs(rec[:, 0, :] - truth[name]).max() <= 5.1e-7


def test_cartesian_characteristic_bc(ctx, wqlmod, oracle_lib, tmp_path):
    p = write(tmp_path, "cart.in", golden_in("test_rup_cart_fric"))
    s, o = run_pair(wqlmod, oracle_lib, ctx, p, 46)
    for e in field_errors(s, o):
        assert e < TOL
    for name in ["S", "Uhat", "Vhat", "Svel"]:
        assert rel_l2(s.frames(name).astype(np.float64), o.frames(name).astype(np.float64)) < 1e-6


def test_curvilinear_bumpy_fault(ctx, wqlmod, oracle_lib, tmp_path):
    """truth/2's geometry (analytical_test_problem, TPV28): GPU vs oracle."""
    p = write(tmp_path, "curv.in", golden_in("test_rup_curv_fric"))
    s, o = run_pair(wqlmod, oracle_lib, ctx, p, 46)
    for e in field_errors(s, o):
        assert e < TOL
    slip = np.linalg.norm(o.iface(0, 3))
    for copy in range(2):
        for c in range(4):
            # S(1) (opening) is rounding noise; compare against the slip scale
            assert np.linalg.norm(s.iface(copy, c) - o.iface(copy, c)) < 1e-9 * slip


def test_curvilinear_path_flat_grid_truth1(ctx, wqlmod, oracle_lib, tmp_path):
    text = set_key(golden_in("test_rup_cart_fric"), "type_of_mesh", "'curvilinear'")
    p = write(tmp_path, "cc.in", with_groups(text, WEIGHTED))
    s, o = run_pair(wqlmod, oracle_lib, ctx, p, 46)
    truth = np.load(os.path.join(GOLDEN, "truth_cart.npz"))
    for name in ["S", "Uface", "Uhat"]:
        got = s.frames(name).astype(np.float64)
        assert np.abs(got - truth[name]).max() <= 1e-7 * max(np.abs(truth[name]).max(), 1.0), name
    for e in field_errors(s, o):
        assert e < TOL


@pytest.mark.parametrize("variant,prec", [(0, "fp64"), (2, "fp64"), (3, "fp64"),
                                          (2, "fp32c"), (3, "fp32c"), (4, "fp32c"), (5, "fp32c"),
                                          (6, "fp32c")])
def test_tiled_matches_pointwise(ctx, wqlmod, tmp_path, variant, prec):
    """The tiled stencil variants compute the same stencil as the per-point
    form (curvilinear bumpy fault, closures in all three axes, small s chunks
    so chunk edges fall on closure rows).  FP64 agrees to rounding; FP32C to
    float rounding of the differently contracted sums."""
    p = write(tmp_path, "curv.in", golden_in("test_rup_curv_fric"))
    pr = wqlmod.FP64 if prec == "fp64" else wqlmod.FP32C
    a = wqlmod.Scenario(ctx, p, precision=pr)
    b = wqlmod.Scenario(ctx, p, precision=pr)
    a.set_tuning(1, 0)
    b.set_tuning(variant, 5)
    a.step(10)
    b.step(10)
    tol = 1e-13 if prec == "fp64" else 2e-6
    for blk in range(2):
        assert rel_l2(b.fields(blk), a.fields(blk)) < tol


@pytest.mark.parametrize("cfg,schunk", [("config0", 0), ("config0", 7), ("config1", 0), ("config1", 5)])
def test_tma_matches_pointwise(ctx, wqlmod, cfg, schunk):
    """The TMA-pipelined FP32 stencil against the per-point form on the
    seeded workloads at 41^3 (Cartesian) and 45^3 (curvilinear): two q
    tiles, a shifted last r tile, several s chunks (automatic and 7 or 5
    planes) next to the per-point s-boundary planes."""
    import wql_configs
    text, media = (wql_configs.config0(steps=10) if cfg == "config0"
                   else wql_configs.config1(n=45, steps=10))
    a = wqlmod.Scenario(ctx, text=text, precision=wqlmod.FP32C, media=media)
    b = wqlmod.Scenario(ctx, text=text, precision=wqlmod.FP32C, media=media)
    a.set_tuning(1, 0)
    b.set_tuning(5, schunk)
    a.step(6)
    b.step(6)
    b.sync(check_nan=True)
    for blk in range(2):
        assert rel_l2(b.fields(blk), a.fields(blk)) < 2e-6


def test_output_files(ctx, wqlmod, tmp_path):
    """wql_write_outputs: the eight fault streams as raw float32 frames and one
    (4f15.10) text file per station, in the reference's names and layout;
    their contents are the frames and records of the run (truth/1)."""
    p = write(tmp_path, "cart.in", with_groups(golden_in("test_rup_cart_fric"), WEIGHTED))
    s = wqlmod.Scenario(ctx, p)
    s.step(46)
    out = tmp_path / "out"
    s.write_outputs(out)
    truth = np.load(os.path.join(GOLDEN, "truth_cart.npz"))
    ncomp = {"Uface": 9, "Vface": 9, "S": 4, "Uhat": 6, "Vhat": 6, "Svel": 3, "trup": 1, "state": 1}
    for ext, nc in ncomp.items():
        f = out / "data" / f"test_rup_cart_fric_interface.{ext}"
        raw = np.fromfile(f, dtype="<f4")
        assert raw.size == 46 * nc * 21 * 21, ext
        assert np.array_equal(raw.reshape(46, nc, 21, 21), s.frames(ext)), ext
        assert np.abs(raw.reshape(46, nc, 21, 21) - truth[ext]).max() <= 1e-9 * max(np.abs(truth[ext]).max(), 1.0)
    for block, (ijk, tname) in enumerate((((21, 11, 11), "station_21_11_11"), ((1, 11, 11), "station_1_11_11"))):
        b = block + 1
        f = out / "seismogram" / f"block{b}" / "data" / f"test_rup_cart_fric_{ijk[0]}_{ijk[1]}_{ijk[2]}_block{b}.dat"
        lines = f.read_text().splitlines()
        assert len(lines) == 46 and all(len(l) == 60 for l in lines)
        vals = np.array([[float(l[15 * c:15 * (c + 1)]) for c in range(4)] for l in lines])
        _, rec = s.stations(block)
        assert np.abs(vals - rec[:, 0, :]).max() <= 0.51e-10
        assert np.abs(vals - truth[tname]).max() <= 5.1e-7
    s.close()


def test_mesh_and_material_from_files(ctx, wqlmod, tmp_path):
    """mesh_source = 'file' (block_grid_<id>.X/Y/Z) and material_source =
    'file' (btp%material_path) give the same run as the computed grid and the
    preset material they were written from (bitwise, FP64)."""
    text = golden_in("test_rup_curv_fric")
    wqlmod.write_block_grids(text, tmp_path)
    n = 21 ** 3
    rho, cs, cp = 2.67, 3.464, 6.0
    lam, mu = rho * (cp * cp - 2.0 * cs * cs), rho * cs * cs
    for b in (1, 2):
        for name, v in (("lam", lam), ("mu", mu), ("rho", rho)):
            np.full(n, v, dtype="<f8").tofile(tmp_path / f"{name}{b}.bin")
    ftext = text.replace("type_of_mesh='curvilinear',",
                         "type_of_mesh='curvilinear',\n mesh_source = 'file',\n material_source = 'file',")
    assert ftext != text
    for b in (1, 2):
        ftext = ftext.replace(f"btp({b})%rho_s_p", f"btp({b})%material_path = 'lam{b}.bin', 'mu{b}.bin', "
                                                   f"'rho{b}.bin',\nbtp({b})%rho_s_p")
    a = wqlmod.Scenario(ctx, text=text)
    f = wqlmod.Scenario(ctx, text=ftext, base_dir=str(tmp_path))
    a.step(10)
    f.step(10)
    for blk in range(2):
        assert np.array_equal(a.fields(blk), f.fields(blk))
    assert np.array_equal(a.frames("Svel"), f.frames("Svel"))
    a.close()
    f.close()
    # a missing grid file is an input error, not a crash
    (tmp_path / "block_grid_2.Z").unlink()
    with pytest.raises(wqlmod.WqlError):
        wqlmod.Scenario(ctx, text=ftext, base_dir=str(tmp_path))


def test_fault_profile_file_vs_oracle(ctx, wqlmod, oracle_lib, tmp_path):
    """A fault surface read from a profile file (profile_type
    'read_from_memomry_fractal'): GPU FP64 against the oracle."""
    from test_host_cpu import _fractal_case
    text, _ = _fractal_case(tmp_path)
    p = write(tmp_path, "fractal.in", text)
    s, o = run_pair(wqlmod, oracle_lib, ctx, p, 20)
    for e in field_errors(s, o):
        assert e < TOL


@pytest.mark.parametrize("prec", ["fp64", "fp32c"])
def test_stage_by_stage_equals_step(ctx, wqlmod, tmp_path, prec):
    """wql_stage 1..5 advances a step exactly as wql_step does (fields, fault
    state and frames, bitwise); stages out of order and a step in the middle
    of one are refused."""
    p = write(tmp_path, "cart.in", golden_in("test_rup_cart_fric"))
    precision = wqlmod.FP64 if prec == "fp64" else wqlmod.FP32C
    a = wqlmod.Scenario(ctx, p, precision=precision)
    b = wqlmod.Scenario(ctx, p, precision=precision)
    a.step(3)
    for _ in range(3):
        for st in range(1, 6):
            b.stage(st)
    for blk in range(2):
        assert np.array_equal(a.fields(blk), b.fields(blk))
    for copy in range(2):
        for what in range(6):
            assert np.array_equal(a.iface(copy, what), b.iface(copy, what))
    assert np.array_equal(a.frames("Svel"), b.frames("Svel"))
    with pytest.raises(wqlmod.WqlError):
        b.stage(2)
    b.stage(1)
    with pytest.raises(wqlmod.WqlError):
        b.step(1)
    for st in range(2, 6):
        b.stage(st)
    b.step(1)
    a.close()
    b.close()
