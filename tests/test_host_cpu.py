"""Host-side logic of the library, run without a device: the block grid
files that mesh_source = 'file' reads (wql_write_block_grids, the role of
the reference's preprocessor) and the device-footprint estimate used for
admission."""
import os

import numpy as np
import pytest

from inputs import golden_in, set_key


@pytest.fixture(scope="module")
def wqlmod():
    import shutil
    if shutil.which("nvcc") is None:
        pytest.skip("nvcc not available")
    import wql_build
    wql_build.build()
    import wql
    return wql


def _grid(path, n):
    return np.fromfile(path, dtype="<f8").reshape(n[2], n[1], n[0])  # q fastest


def test_block_grid_files_cartesian(wqlmod, tmp_path):
    """Cartesian blocks: x = a + i*h per axis (src/grid.f90 cartesian_grid_3d),
    written as raw FP64, q fastest, one file per coordinate and block."""
    wqlmod.write_block_grids(golden_in("test_rup_cart_fric"), tmp_path)
    n = (21, 21, 21)
    boxes = {1: ((-3.0, 6.0, -1.5), (0.0, 9.0, 1.5)), 2: ((0.0, 6.0, -1.5), (3.0, 9.0, 1.5))}
    for b, (lo, hi) in boxes.items():
        for c, ext in enumerate("XYZ"):
            f = tmp_path / f"block_grid_{b}.{ext}"
            assert f.stat().st_size == 8 * 21 ** 3
            x = _grid(f, n)
            line = lo[c] + np.arange(21) * ((hi[c] - lo[c]) / 20.0)
            shape = [1, 1, 1]
            shape[2 - c] = 21
            assert np.array_equal(x, np.broadcast_to(line.reshape(shape), x.shape)), (b, ext)


def test_block_grid_files_curvilinear(wqlmod, tmp_path):
    """Curvilinear blocks (transfinite interpolation with the bumpy fault of
    truth/2): the faces away from the fault stay flat, the fault faces of the
    two blocks coincide, and q increases along every row."""
    wqlmod.write_block_grids(golden_in("test_rup_curv_fric"), tmp_path)
    n = (21, 21, 21)
    X1, X2 = _grid(tmp_path / "block_grid_1.X", n), _grid(tmp_path / "block_grid_2.X", n)
    Y1, Y2 = _grid(tmp_path / "block_grid_1.Y", n), _grid(tmp_path / "block_grid_2.Y", n)
    Z1, Z2 = _grid(tmp_path / "block_grid_1.Z", n), _grid(tmp_path / "block_grid_2.Z", n)
    assert np.ptp(X1[:, :, 0]) < 1e-12 and np.ptp(X2[:, :, -1]) < 1e-12
    assert np.ptp(X1[:, :, -1]) > 0.0  # the fault is not flat
    assert np.allclose(X1[:, :, -1], X2[:, :, 0], rtol=0, atol=1e-12)
    assert np.allclose(Y1[:, :, -1], Y2[:, :, 0], rtol=0, atol=1e-12)
    assert np.allclose(Z1[:, :, -1], Z2[:, :, 0], rtol=0, atol=1e-12)
    assert (np.diff(X1, axis=2) > 0).all() and (np.diff(X2, axis=2) > 0).all()


def test_block_grid_files_bad_directory(wqlmod, tmp_path):
    bad = tmp_path / "f"
    bad.write_text("")
    with pytest.raises(wqlmod.WqlError):
        wqlmod.write_block_grids(golden_in("test_rup_cart_fric"), bad / "sub")


def test_footprint_estimate_host(wqlmod):
    """The admission estimate grows with the grid, is larger in FP64 than in
    FP32C, and counts PML slabs."""
    text = golden_in("test_rup_cart_fric")
    r32, p32 = wqlmod.estimate_device_bytes(text, wqlmod.FP32C)
    r64, p64 = wqlmod.estimate_device_bytes(text, wqlmod.FP64)
    assert 0 < r32 < p32 and 0 < r64 < p64 and r64 > r32
    big = text.replace("btp(1)%nqrs = 21, 21, 21", "btp(1)%nqrs = 41, 21, 21")
    assert wqlmod.estimate_device_bytes(big, wqlmod.FP32C)[0] > r32
    pml = text.replace("btp(1)%rqrs = 0, 1, 1,", "btp(1)%rqrs = 0, 1, 1,\nbtp(1)%pml_lqrs = T, F, F,\nbtp(1)%npml = 5,")
    assert wqlmod.estimate_device_bytes(pml, wqlmod.FP32C)[0] > r32


def test_footprint_estimate_anelastic(wqlmod):
    """The anelastic response adds its 48 memory-variable arrays and 1/Q per
    block (and the FP32C gradient hand-off array when no PML holds one)."""
    text = golden_in("test_rup_cart_fric")
    an = text.replace("response = 'elastic'", "response = 'anelastic'") \
        if "response = 'elastic'" in text else text.replace(" coupling", " response = 'anelastic',\n coupling", 1)
    r32 = wqlmod.estimate_device_bytes(text, wqlmod.FP32C)[0]
    a32 = wqlmod.estimate_device_bytes(an, wqlmod.FP32C)[0]
    np_pts = 2 * 24 * 21 * 21  # two blocks, pitch 24 floats, 21 x 21 rows
    assert a32 - r32 >= (2 * 24 + 1 + 9) * 4 * np_pts
    r64 = wqlmod.estimate_device_bytes(text, wqlmod.FP64)[0]
    a64 = wqlmod.estimate_device_bytes(an, wqlmod.FP64)[0]
    assert a64 - r64 >= (2 * 24 + 1) * 8 * 2 * 22 * 21 * 21


def _fractal_case(tmp_path, n=21):
    """The truth/2 curvilinear input with profile_type
    'read_from_memomry_fractal': a fault surface file of n*n rows (x, y, z),
    r fastest, written with Fortran exponents."""
    rng = np.random.default_rng(7)
    j, k = np.meshgrid(np.arange(n), np.arange(n), indexing="xy")  # j fastest in ravel
    x1 = 0.03 * np.sin(0.7 * j + 0.2) * np.cos(0.5 * k) + 0.005 * rng.standard_normal((n, n))
    with open(tmp_path / "fault.dat", "w") as f:
        for xv, yv, zv in zip(x1.ravel(), (6.0 + 0.15 * j).ravel(), (-1.5 + 0.15 * k).ravel()):
            f.write(f"{xv:.17e} {yv:.6f} {zv:.6f}\n".replace("e", "d"))
    text = golden_in("test_rup_curv_fric").replace("'analytical_test_problem'", "'read_from_memomry_fractal'") \
                                          .replace("'No-path'", "'fault.dat'")
    return text, x1


def test_fault_profile_file(wqlmod, tmp_path):
    """profile_type 'read_from_memomry_fractal': the fault faces are the block
    faces plus lc (block 1, q = nq) or rc (block 2, q = 1) times the file's x
    column (src/grid.f90:832-924)."""
    text, x1 = _fractal_case(tmp_path)
    out = tmp_path / "grids"
    wqlmod.write_block_grids(text, out, base_dir=tmp_path)
    n = (21, 21, 21)
    X1 = _grid(out / "block_grid_1.X", n)
    X2 = _grid(out / "block_grid_2.X", n)
    assert np.allclose(X1[:, :, -1], 0.0 + x1, rtol=0, atol=1e-15)
    assert np.allclose(X2[:, :, 0], 0.0 + x1, rtol=0, atol=1e-15)
    assert np.ptp(X1[:, :, 0]) < 1e-12 and np.ptp(X2[:, :, -1]) < 1e-12
    (tmp_path / "fault.dat").write_text("1 2 3\n")
    with pytest.raises(wqlmod.WqlError):
        wqlmod.write_block_grids(text, out, base_dir=tmp_path)


_TABLE_PROBE = r"""
#include <cstdio>
#include <cstdlib>
#include "wql_sbp.cuh"
// Dense n x n matrices of the library's upwind pair of one order from its
// tables: left closure rows, right rows as the negated mirror images of the
// other operator's left rows, interior rows from the interior weights.
int main() {
  const double t6[2][6][10] = WQL_UP_TABLE;
  const double t5[2][4][7] = WQL_UP5_TABLE;
  const double c6[7] = WQL_UP_CF, c5[6] = WQL_UP5_CF;
  const int n = 30;
  for (int order = 6; order >= 5; --order) {
    const int R = order == 6 ? 6 : 4, NC = order == 6 ? 10 : 7, PHI = order == 6 ? 4 : 3;
    for (int op = 0; op < 2; ++op) {
      static double D[30][30];
      for (int i = 0; i < n; ++i)
        for (int j = 0; j < n; ++j) D[i][j] = 0.0;
      for (int i = 0; i < n; ++i) {
        if (i < R) {
          for (int c = 0; c < NC; ++c) D[i][c] = order == 6 ? t6[op][i][c] : t5[op][i][c];
        } else if (i >= n - R) {
          const int k = n - 1 - i;
          for (int c = 0; c < NC; ++c) D[i][n - 1 - c] = -(order == 6 ? t6[1 - op][k][c] : t5[1 - op][k][c]);
        } else {
          for (int o = -PHI; o <= PHI; ++o) {
            const double* cf = order == 6 ? c6 : c5;
            if (op == 0 && o >= -2) D[i][i + o] = cf[o + 2];
            if (op == 1 && o <= 2) D[i][i + o] = -cf[2 - o];
          }
        }
      }
      for (int i = 0; i < n; ++i)
        for (int j = 0; j < n; ++j) std::printf("%.17g\n", D[i][j]);
    }
  }
  // the central SBP-6 operator: closure rows, right rows as their negated
  // mirror images, interior (kC1, kC2, kC3)
  const double ts[6][9] = WQL_SBP_TABLE;
  const double cc[3] = {wql::kC1, wql::kC2, wql::kC3};
  for (int i = 0; i < n; ++i)
    for (int j = 0; j < n; ++j) {
      double w = 0.0;
      if (i < 6) w = j < 9 ? ts[i][j] : 0.0;
      else if (i >= n - 6) w = (n - 1 - j) < 9 ? -ts[n - 1 - i][n - 1 - j] : 0.0;
      else if (j != i && std::abs(j - i) <= 3) w = (j > i ? 1.0 : -1.0) * cc[std::abs(j - i) - 1];
      std::printf("%.17g\n", w);
    }
  return 0;
}
"""


def test_library_upwind_tables_match_oracle(oracle_lib, tmp_path):
    """The library's transcription of the operator tables (wql_sbp.cuh, read
    by the kernels) against the oracle's, row by row: the upwind pairs of
    orders 6 and 5 and the central SBP-6 operator."""
    import os
    import subprocess
    csrc = os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "waveqlab3d-gh_gb300", "csrc")
    src = tmp_path / "probe.cpp"
    src.write_text(_TABLE_PROBE)
    exe = tmp_path / "probe"
    subprocess.run(["g++", "-std=c++17", "-O0", "-I" + csrc, str(src), "-o", str(exe)], check=True)
    vals = np.array([float(v) for v in subprocess.run([str(exe)], check=True, capture_output=True,
                                                       text=True).stdout.split()])
    mats = vals.reshape(5, 30, 30)
    ref = [oracle_lib.fd_matrix(1, True, 30), oracle_lib.fd_matrix(1, False, 30),
           oracle_lib.fd_matrix(2, True, 30), oracle_lib.fd_matrix(2, False, 30),
           oracle_lib.fd_matrix(0, True, 30)]
    for got, want in zip(mats, ref):
        assert np.abs(got - want).max() < 1e-15


def test_upwind_table_copies_agree():
    """The library's and the oracle's copies of the table upwind operators
    (written by oracle/make_upwind_tables.py) hold the same numbers."""
    import re
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    lib = open(os.path.join(root, "waveqlab3d-gh_gb300", "csrc", "wql_upwind_tables.h")).read()
    orc = open(os.path.join(root, "oracle", "upwind_tables.inc")).read()

    def data(text):
        body = text[text.index("= {"):]
        return re.findall(r'"[a-z_]+"|-?\d+\.?\d*(?:e[+-]?\d+)?', body)
    a, b = data(lib), data(orc)
    assert len(a) == len(b) > 15 * 1300
    assert a == b


_SCLOSE_PROBE = r"""
#include <cmath>
#include <cstdio>
#include "wql_sbp.cuh"
using namespace wql;
// The s-closure rows as the TMA stencil forms them: columns whose window
// position (s_close_vpos / s_close_fpos) lies in 0..6 come from the register
// window, the others from memory.  The window holds planes s-3..s+3 for the
// central operator; velocities of s-2..s+4 and fluxes of s-4..s+2 for the
// upwind pair (zeros outside the block).
int main() {
  const int n = 30;
  double v[n], g[n];
  for (int s = 0; s < n; ++s) {
    v[s] = std::sin(0.37 * s + 0.1) + 0.01 * s * s;
    g[s] = std::cos(0.23 * s) - 0.02 * s;
  }
  for (int fd = 0; fd < 2; ++fd) {
    const int ov = fd ? 2 : 3, of = fd ? 4 : 3;  // window position of plane s
    for (int right = 0; right < 2; ++right)
      for (int row = 0; row < 6; ++row) {
        const int s = right ? n - 1 - row : row;
        double dv = 0.0, df = 0.0;
        int from_memory = 0;
        for (int t = 0; t < (fd ? 10 : 9); ++t) {
          const double wv = s_close_w(fd, right, false, row, t), wf = s_close_w(fd, right, true, row, t);
          const int plane = s + s_close_off(right, row, t);
          const int pv = s_close_vpos(fd, right, row, t), pf = s_close_fpos(fd, right, row, t);
          auto win = [&](const double* a, int pos, int o) {
            const int q = s + pos - o;
            return q >= 0 && q < n ? a[q] : 0.0;
          };
          if (wv != 0.0) {
            const bool w = pv >= 0 && pv <= 6;
            dv += wv * (w ? win(v, pv, ov) : v[plane]);
            from_memory += !w;
          }
          if (wf != 0.0) {
            const bool w = pf >= 0 && pf <= 6;
            df += wf * (w ? win(g, pf, of) : g[plane]);
            from_memory += !w;
          }
        }
        std::printf("%d %d %d %.17g %.17g %d\n", fd, right, s, dv, df, from_memory);
      }
  }
  return 0;
}
"""


def test_s_closure_rows_from_window(oracle_lib, tmp_path):
    """The TMA stencil's s-closure rows (wql_sbp.cuh s_close_*: weights,
    plane offsets and register-window positions) give the rows of the
    oracle's operators: the central SBP-6 operator on velocities and fluxes,
    and the order-6 upwind pair (D+ on velocities, D- on fluxes), at both
    ends; at most four (quantity, plane) pairs of a row are read from
    memory."""
    import subprocess
    csrc = os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "waveqlab3d-gh_gb300", "csrc")
    src = tmp_path / "sclose.cpp"
    src.write_text(_SCLOSE_PROBE)
    exe = tmp_path / "sclose"
    subprocess.run(["g++", "-std=c++17", "-O0", "-I" + csrc, str(src), "-o", str(exe)], check=True)
    out = subprocess.run([str(exe)], check=True, capture_output=True, text=True).stdout.split("\n")
    n = 30
    sv = np.arange(n)
    v = np.sin(0.37 * sv + 0.1) + 0.01 * sv * sv
    g = np.cos(0.23 * sv) - 0.02 * sv
    D = oracle_lib.fd_matrix(0, True, n)
    Dp, Dm = oracle_lib.fd_matrix(1, True, n), oracle_lib.fd_matrix(1, False, n)
    rows = [line.split() for line in out if line.strip()]
    assert len(rows) == 24
    for fd, right, s, dv, df, nmem in rows:
        fd, s = int(fd), int(s)
        want_v = (Dp if fd else D)[s] @ v
        want_f = (Dm if fd else D)[s] @ g
        assert abs(float(dv) - want_v) <= 1e-13 * max(1.0, abs(want_v))
        assert abs(float(df) - want_f) <= 1e-13 * max(1.0, abs(want_f))
        assert int(nmem) <= 4
