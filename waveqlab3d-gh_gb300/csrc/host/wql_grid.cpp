// Block coordinates on the host (one-time FP64 setup); see wql_grid.h.
#include "wql_grid.h"

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <string>
#include <thread>
#include <vector>

namespace wql {
namespace {

const double kPi = 3.141592653589793;

// f(k) for k in [0, n) on up to 16 host threads, each taking a contiguous
// range (every k is independent: the result does not depend on the split).
template <typename F>
void parallel_k(int n, F&& f) {
  const unsigned hw = std::max(1u, std::min(16u, std::thread::hardware_concurrency()));
  if (n < 16 || hw == 1) {
    for (int k = 0; k < n; ++k) f(k);
    return;
  }
  const int per = (n + (int)hw - 1) / (int)hw;
  std::vector<std::thread> th;
  for (int lo = 0; lo < n; lo += per) {
    const int hi = std::min(n, lo + per);
    th.emplace_back([lo, hi, &f] {
      for (int k = lo; k < hi; ++k) f(k);
    });
  }
  for (auto& t : th) t.join();
}

// 2D transfinite interpolation of one face from its four edge curves
// (Gen_Surf_Mesh, src/grid.f90:2418-2455).  L/R run along the second index
// (length nb), B/T along the first (length na).  Output index a + na*b.
void face_tfi(int na, int nb, const std::vector<double>& L, const std::vector<double>& R,
              const std::vector<double>& Bo, const std::vector<double>& T,
              std::vector<double>& out) {
  out.assign((size_t)na * nb, 0.0);
  const double ha = 1.0 / (double)(na - 1), hb = 1.0 / (double)(nb - 1);
  for (int b = 0; b < nb; ++b)
    for (int a = 0; a < na; ++a) {
      const double q = (double)a * ha, r = (double)b * hb;
      out[(size_t)a + (size_t)na * b] = (1.0 - q) * L[b] + q * R[b] + (1.0 - r) * Bo[a] + r * T[a] -
                                        (1.0 - q) * (1.0 - r) * L[0] - q * (1.0 - r) * R[0] -
                                        r * (1.0 - q) * T[0] - (r * q) * T[na - 1];
    }
}

struct Faces {  // one coordinate component on the six faces
  std::vector<double> left, right;   // (j,k): j + nr*k
  std::vector<double> top, bottom;   // (i,k): i + nq*k   (top = r-min face)
  std::vector<double> front, back;   // (i,j): i + nq*j   (front = s-min face)
};

// 3D transfinite interpolation (Gen3_Curve_Mesh, src/grid.f90:2290-2416).
void block_tfi(int nq, int nr, int ns, const Faces& f, std::vector<double>& x) {
  x.assign((size_t)nq * nr * ns, 0.0);
  const double hq = 1.0 / (double)(nq - 1), hr = 1.0 / (double)(nr - 1), hs = 1.0 / (double)(ns - 1);
  auto LK = [&](const std::vector<double>& a, int j, int k) { return a[(size_t)j + (size_t)nr * k]; };
  auto IK = [&](const std::vector<double>& a, int i, int k) { return a[(size_t)i + (size_t)nq * k]; };
  auto IJ = [&](const std::vector<double>& a, int i, int j) { return a[(size_t)i + (size_t)nq * j]; };
  parallel_k(ns, [&](int k) {
    for (int j = 0; j < nr; ++j)
      for (int i = 0; i < nq; ++i) {
        const double q = (double)i * hq, r = (double)j * hr, s = (double)k * hs;
        const double U = (1.0 - q) * LK(f.left, j, k) + q * LK(f.right, j, k);
        const double V = (1.0 - r) * IK(f.top, i, k) + r * IK(f.bottom, i, k);
        const double W = (1.0 - s) * IJ(f.front, i, j) + s * IJ(f.back, i, j);
        const double UW = (1.0 - q) * ((1.0 - r) * LK(f.left, 0, k) + r * LK(f.left, nr - 1, k)) +
                          q * ((1.0 - r) * LK(f.right, 0, k) + r * LK(f.right, nr - 1, k));
        const double UV = (1.0 - r) * ((1.0 - s) * IK(f.top, i, 0) + s * IK(f.top, i, ns - 1)) +
                          r * ((1.0 - s) * IK(f.bottom, i, 0) + s * IK(f.bottom, i, ns - 1));
        const double VW = (1.0 - s) * ((1.0 - q) * IJ(f.front, 0, j) + q * IJ(f.front, nq - 1, j)) +
                          s * ((1.0 - q) * IJ(f.back, 0, j) + q * IJ(f.back, nq - 1, j));
        const double C1 = (1.0 - q) * ((1.0 - r) * ((1.0 - s) * IK(f.top, 0, 0) + s * IK(f.top, 0, ns - 1)) +
                                       r * ((1.0 - s) * IK(f.bottom, 0, 0) + s * IK(f.bottom, 0, ns - 1)));
        const double C2 = q * ((1.0 - r) * ((1.0 - s) * IK(f.top, nq - 1, 0) + s * IK(f.top, nq - 1, ns - 1)) +
                               r * ((1.0 - s) * IK(f.bottom, nq - 1, 0) + s * IK(f.bottom, nq - 1, ns - 1)));
        x[(size_t)i + (size_t)nq * ((size_t)j + (size_t)nr * k)] = U + V + W - UV - UW - VW + C1 + C2;
      }
  });
}

// The fault surface file of profile_type 'read_from_memomry_fractal'
// (read_2darray + reshape_2darray, src/grid.f90:832-838, 2457-2500): n rows
// of three list-directed numbers (x, y, z); the x column, r fastest.
int read_fault_profile(const std::string& path, size_t n, std::vector<double>& x1, std::string& err) {
  std::FILE* f = std::fopen(path.c_str(), "r");
  if (!f) {
    err = "cannot open fault profile " + path;
    return 1;
  }
  x1.resize(n);
  char line[4096];
  size_t row = 0;
  while (row < n && std::fgets(line, sizeof(line), f)) {
    for (char* c = line; *c; ++c)
      if (*c == 'd' || *c == 'D') *c = 'e';  // Fortran exponent letters
      else if (*c == ',') *c = ' ';
    double v[3];
    if (std::sscanf(line, "%lf %lf %lf", &v[0], &v[1], &v[2]) != 3) continue;  // blank or comment line
    x1[row++] = v[0];
  }
  std::fclose(f);
  if (row != n) {
    err = path + " holds " + std::to_string(row) + " rows of x y z, not " + std::to_string(n);
    return 1;
  }
  return 0;
}

// A list-directed text file of `n` rows of three numbers (read_2darray,
// src/grid.f90:2457-2481); Fortran exponent letters and commas accepted,
// lines that do not hold three numbers skipped.  Output column-major: the
// c-th column is out[c*n .. (c+1)*n).
int read_xyz_rows(const std::string& path, size_t n, std::vector<double>& out, std::string& err) {
  std::FILE* f = std::fopen(path.c_str(), "r");
  if (!f) {
    err = "cannot open " + path;
    return 1;
  }
  out.assign(3 * n, 0.0);
  char line[4096];
  size_t row = 0;
  while (row < n && std::fgets(line, sizeof(line), f)) {
    for (char* c = line; *c; ++c)
      if (*c == 'd' || *c == 'D') *c = 'e';
      else if (*c == ',') *c = ' ';
    double v[3];
    if (std::sscanf(line, "%lf %lf %lf", &v[0], &v[1], &v[2]) != 3) continue;
    for (int c = 0; c < 3; ++c) out[(size_t)c * n + row] = v[c];
    ++row;
  }
  std::fclose(f);
  if (row != n) {
    err = path + " holds " + std::to_string(row) + " rows of x y z, not " + std::to_string(n);
    return 1;
  }
  return 0;
}

// Curvilinear block with a free-surface topography on the r-min face
// (use_topography = T, src/grid.f90:1349-1875).  The top face comes from
// 'read_topo_from_memory' (a file of nq*ns rows x y z, s fastest, with
// y = ay + topo * the file's y; :1394-1425) or 'analytical_topography'
// (:1364-1392).  The x faces: (y, z) meshed from edges that run from the
// topography down to by (:1440-1518), x = ax / bx, or, with
// 'read_from_memomry_fractal', the fault file's rows taken whole on the
// interface face: x = ax (bx) + the file's x, y and z the file's (:1538-1676).
// The s faces join the x faces, the topography's edge and y = by
// (:1695-1805); the bottom face joins the others (:1826-1858).
int curvilinear_topo(const Problem& P, const BlockParams& bp, BlockGrid& G, std::string& err) {
  const int mx = G.nq, my = G.nr, mz = G.ns;
  const double ax = bp.aqrs[0], bx = bp.bqrs[0], ay = bp.aqrs[1], by = bp.bqrs[1];
  const double az = bp.aqrs[2], bz = bp.bqrs[2];
  Faces X, Y, Z;
  const size_t ntop = (size_t)mx * mz;
  X.top.resize(ntop);
  Y.top.resize(ntop);
  Z.top.resize(ntop);
  if (bp.topography_type == "read_topo_from_memory") {
    std::vector<double> t;
    if (read_xyz_rows(resolve_path(P.base_dir, bp.topography_path), ntop, t, err)) return 1;
    for (int k = 0; k < mz; ++k)
      for (int i = 0; i < mx; ++i) {
        const size_t row = (size_t)k + (size_t)mz * i, o = (size_t)i + (size_t)mx * k;
        X.top[o] = t[row];
        Y.top[o] = ay + P.topo * t[ntop + row];
        Z.top[o] = t[2 * ntop + row];
      }
  } else if (bp.topography_type == "analytical_topography") {
    const double hx = (bx - ax) / (double)(mx - 1), hz = (bz - az) / (double)(mz - 1);
    for (int k = 0; k < mz; ++k)
      for (int i = 0; i < mx; ++i) {
        const size_t o = (size_t)i + (size_t)mx * k;
        X.top[o] = ax + (double)i * hx;
        Z.top[o] = az + (double)k * hz;
        const double r1 = std::sqrt((X.top[o] - 10.0) * (X.top[o] - 10.0) + (Z.top[o] - 10.0) * (Z.top[o] - 10.0));
        const double f = r1 <= 3.0 ? -0.3 * (1.0 + std::cos(kPi * r1 / 3.0)) : 0.0;
        Y.top[o] = ay - P.topo * 1.5 * f;
      }
  } else {
    err = "topography_type '" + bp.topography_type + "' is not supported ('read_topo_from_memory' or "
          "'analytical_topography')";
    return 1;
  }
  auto top = [&](const std::vector<double>& a, int i, int k) { return a[(size_t)i + (size_t)mx * k]; };
  // x faces: y from the topography's edge down to by, z uniform
  const size_t nx = (size_t)my * mz;
  const double hr = 1.0 / (double)(my - 1), hs = 1.0 / (double)(mz - 1);
  for (int side = 0; side < 2; ++side) {
    const int i = side == 0 ? 0 : mx - 1;
    std::vector<double> yL(mz), yR(mz, by), yB(my), yT(my), zL(mz), zR(mz), zB(my, az), zT(my, bz);
    for (int j = 0; j < my; ++j) {
      const double r = (double)j * hr;
      yT[j] = top(Y.top, i, mz - 1) + (by - top(Y.top, i, mz - 1)) * r;
      yB[j] = top(Y.top, i, 0) + (by - top(Y.top, i, 0)) * r;
    }
    for (int k = 0; k < mz; ++k) {
      zL[k] = zR[k] = az + (bz - az) * ((double)k * hs);
      yL[k] = top(Y.top, i, k);
    }
    face_tfi(my, mz, yL, yR, yB, yT, side == 0 ? Y.left : Y.right);
    face_tfi(my, mz, zL, zR, zB, zT, side == 0 ? Z.left : Z.right);
  }
  X.left.assign(nx, ax);
  X.right.assign(nx, bx);
  const std::string& pt = bp.profile_type;
  if (pt == "read_from_memomry_fractal") {
    std::vector<double> f;
    if (read_xyz_rows(resolve_path(P.base_dir, bp.profile_path), nx, f, err)) return 1;
    for (size_t p = 0; p < nx; ++p) {
      if (bp.rc != 0.0) {
        X.left[p] = ax + f[p];
        Y.left[p] = f[nx + p];
        Z.left[p] = f[2 * nx + p];
      }
      if (bp.lc != 0.0) {
        X.right[p] = bx + f[p];
        Y.right[p] = f[nx + p];
        Z.right[p] = f[2 * nx + p];
      }
    }
  } else if (pt != "no_path") {
    err = "with use_topography, profile_type must be 'no_path' or 'read_from_memomry_fractal'";
    return 1;
  }
  auto lr = [&](const std::vector<double>& a, int j, int k) { return a[(size_t)j + (size_t)my * k]; };
  // s faces (front k = 0, back k = mz - 1)
  for (int side = 0; side < 2; ++side) {
    const int k = side == 0 ? 0 : mz - 1;
    std::vector<double> xL(my), xR(my), xB(mx), xT(mx), yL(my), yR(my), yB(mx), yT(mx, by);
    const double hq = 1.0 / (double)(mx - 1);
    for (int i = 0; i < mx; ++i) {
      const double q = (double)i * hq;
      xT[i] = lr(X.left, my - 1, k) + (lr(X.right, my - 1, k) - lr(X.left, my - 1, k)) * q;
      xB[i] = top(X.top, i, k);
      yB[i] = top(Y.top, i, k);
    }
    for (int j = 0; j < my; ++j) {
      xL[j] = lr(X.left, j, k);
      xR[j] = lr(X.right, j, k);
      yL[j] = lr(Y.left, j, k);
      yR[j] = lr(Y.right, j, k);
    }
    face_tfi(mx, my, xL, xR, xB, xT, side == 0 ? X.front : X.back);
    face_tfi(mx, my, yL, yR, yB, yT, side == 0 ? Y.front : Y.back);
  }
  Z.front.assign((size_t)mx * my, az);
  Z.back.assign((size_t)mx * my, bz);
  // bottom face (j = my - 1): y = by, x and z from the edges of the others
  {
    std::vector<double> xL(mz), xR(mz), xB(mx), xT(mx), zL(mz), zR(mz), zB(mx), zT(mx);
    for (int i = 0; i < mx; ++i) {
      xT[i] = X.back[(size_t)i + (size_t)mx * (my - 1)];
      xB[i] = X.front[(size_t)i + (size_t)mx * (my - 1)];
      zT[i] = Z.back[(size_t)i + (size_t)mx * (my - 1)];
      zB[i] = Z.front[(size_t)i + (size_t)mx * (my - 1)];
    }
    for (int k = 0; k < mz; ++k) {
      xL[k] = lr(X.left, my - 1, k);
      xR[k] = lr(X.right, my - 1, k);
      zL[k] = lr(Z.left, my - 1, k);
      zR[k] = lr(Z.right, my - 1, k);
    }
    face_tfi(mx, mz, xL, xR, xB, xT, X.bottom);
    face_tfi(mx, mz, zL, zR, zB, zT, Z.bottom);
  }
  Y.bottom.assign(ntop, by);
  block_tfi(mx, my, mz, X, G.x[0]);
  block_tfi(mx, my, mz, Y, G.x[1]);
  block_tfi(mx, my, mz, Z, G.x[2]);
  return 0;
}

int curvilinear(const BlockParams& bp, const std::string& base_dir, BlockGrid& G, std::string& err) {
  const int mx = G.nq, my = G.nr, mz = G.ns;
  const double ax = bp.aqrs[0], bx = bp.bqrs[0], ay = bp.aqrs[1], by = bp.bqrs[1];
  const double az = bp.aqrs[2], bz = bp.bqrs[2];
  const std::string& pt = bp.profile_type;
  const bool flat = pt.empty() || pt == "No-path" || pt == "no_path" || pt == "none";
  const bool fractal = pt == "read_from_memomry_fractal";  // the reference's spelling
  if (!(flat || fractal || pt == "analytical_tpv28" || pt == "analytical_test_problem")) {
    err = "profile_type '" + pt + "' is not supported";
    return 1;
  }
  const size_t nx = (size_t)my * mz;
  Faces X, Y, Z;
  X.left.resize(nx); X.right.resize(nx);
  Y.left.resize(nx); Y.right.resize(nx);
  Z.left.resize(nx); Z.right.resize(nx);
  const double hy = (by - ay) / (double)(my - 1), hz = (bz - az) / (double)(mz - 1);
  // x-faces (src/grid.f90:593-620): uniform (y,z) with the fault profile on x
  for (int k = 0; k < mz; ++k)
    for (int j = 0; j < my; ++j) {
      const size_t p = (size_t)j + (size_t)my * k;
      const double y = ay + (double)j * hy, z = az + (double)k * hz;
      Y.left[p] = Y.right[p] = y;
      Z.left[p] = Z.right[p] = z;
      X.left[p] = ax;
      X.right[p] = bx;
      if (pt == "analytical_tpv28") {  // two cosine bumps (src/grid.f90:664-681)
        double f = 0.0;
        const double r1 = std::sqrt((z + 10.5) * (z + 10.5) + (y - 7.5) * (y - 7.5));
        const double r2 = std::sqrt((z - 10.5) * (z - 10.5) + (y - 7.5) * (y - 7.5));
        if (r1 <= 3.0) f = -0.3 * (1.0 + std::cos(kPi * r1 / 3.0));
        if (r2 <= 3.0) f = -0.3 * (1.0 + std::cos(kPi * r2 / 3.0));
        X.left[p] += bp.rc * f;
        X.right[p] += bp.lc * f;
      }
    }
  if (fractal) {
    // (y, z) meshed from straight edges, x = the face position plus rc (left)
    // or lc (right) times the file's x column (src/grid.f90:832-924)
    std::vector<double> x1;
    if (read_fault_profile(resolve_path(base_dir, bp.profile_path), nx, x1, err)) return 1;
    std::vector<double> eyL(mz, ay), eyR(mz, by), eyB(my), eyT(my), ezL(mz), ezR(mz), ezB(my, az),
        ezT(my, bz);
    for (int j = 0; j < my; ++j) eyB[j] = eyT[j] = ay + (double)j * hy;
    for (int k = 0; k < mz; ++k) ezL[k] = ezR[k] = az + (double)k * hz;
    face_tfi(my, mz, eyL, eyR, eyB, eyT, Y.left);
    face_tfi(my, mz, ezL, ezR, ezB, ezT, Z.left);
    Y.right = Y.left;
    Z.right = Z.left;
    for (size_t p = 0; p < nx; ++p) {
      X.left[p] = ax;
      if (bp.rc != 0.0) X.left[p] += bp.rc * x1[p];
      X.right[p] = bx;
      if (bp.lc != 0.0) X.right[p] += bp.lc * x1[p];
    }
  }
  if (pt == "analytical_test_problem") {
    // (y,z) meshed by Gen_Surf_Mesh from straight edges, then a Gaussian bump
    // plus a sine product on x (src/grid.f90:790-841)
    std::vector<double> eyL(mz, ay), eyR(mz, by), eyB(my), eyT(my), ezL(mz), ezR(mz), ezB(my, az),
        ezT(my, bz);
    for (int j = 0; j < my; ++j) eyB[j] = eyT[j] = ay + (double)j * hy;
    for (int k = 0; k < mz; ++k) ezL[k] = ezR[k] = az + (double)k * hz;
    face_tfi(my, mz, eyL, eyR, eyB, eyT, Y.left);
    face_tfi(my, mz, ezL, ezR, ezB, ezT, Z.left);
    Y.right = Y.left;
    Z.right = Z.left;
    for (size_t p = 0; p < nx; ++p) {
      auto bump = [&](double y, double z) {
        const double dy = 1.0 * y - 0.5 * (ay + by), dz = z - 0.5 * (az + bz);
        return 0.1 * std::exp(-(dy * dy + 1.0 * (dz * dz)) / 0.025) +
               0.1 * std::sin(2.0 / (by - ay) * kPi * y) * std::sin(2.0 / (bz - az) * kPi * z);
      };
      X.left[p] = ax + bp.rc * bump(Y.left[p], Z.left[p]);
      X.right[p] = bx + bp.lc * bump(Y.right[p], Z.right[p]);
    }
  }
  auto L = [&](const std::vector<double>& a, int j, int k) { return a[(size_t)j + (size_t)my * k]; };
  // s-faces (front k=0, back k=mz-1): edges from the x-faces, straight in q
  auto s_face = [&](int k, const Faces& C, std::vector<double>& out, bool use_y_edges) {
    std::vector<double> eL(my), eR(my), eB(mx), eT(mx);
    for (int j = 0; j < my; ++j) {
      eL[j] = L(C.left, j, k);
      eR[j] = L(C.right, j, k);
    }
    for (int i = 0; i < mx; ++i) {
      double h = (L(C.right, 0, k) - L(C.left, 0, k)) / (double)(mx - 1);
      eB[i] = L(C.left, 0, k) + (double)i * h;
      h = (L(C.right, my - 1, k) - L(C.left, my - 1, k)) / (double)(mx - 1);
      eT[i] = L(C.left, my - 1, k) + (double)i * h;
    }
    (void)use_y_edges;
    face_tfi(mx, my, eL, eR, eB, eT, out);
  };
  s_face(0, X, X.front, false);
  s_face(0, Y, Y.front, true);
  s_face(mz - 1, X, X.back, false);
  s_face(mz - 1, Y, Y.back, true);
  Z.front.assign((size_t)mx * my, az);
  Z.back.assign((size_t)mx * my, bz);
  // r-faces (top j=0, bottom j=my-1)
  auto r_face = [&](int j, const Faces& C, std::vector<double>& out, double zb, double zt, bool zcomp) {
    std::vector<double> eL(mz), eR(mz), eB(mx), eT(mx);
    for (int k = 0; k < mz; ++k) {
      eL[k] = L(C.left, j, k);
      eR[k] = L(C.right, j, k);
    }
    for (int i = 0; i < mx; ++i) {
      if (zcomp) {
        eB[i] = zb;
        eT[i] = zt;
      } else {
        double h = (L(C.right, j, 0) - L(C.left, j, 0)) / (double)(mx - 1);
        eB[i] = L(C.left, j, 0) + (double)i * h;
        h = (L(C.right, j, mz - 1) - L(C.left, j, mz - 1)) / (double)(mx - 1);
        eT[i] = L(C.left, j, mz - 1) + (double)i * h;
      }
    }
    face_tfi(mx, mz, eL, eR, eB, eT, out);
  };
  r_face(0, X, X.top, 0, 0, false);
  r_face(0, Z, Z.top, az, bz, true);
  r_face(my - 1, X, X.bottom, 0, 0, false);
  r_face(my - 1, Z, Z.bottom, az, bz, true);
  Y.top.assign((size_t)mx * mz, ay);
  Y.bottom.assign((size_t)mx * mz, by);
  block_tfi(mx, my, mz, X, G.x[0]);
  block_tfi(mx, my, mz, Y, G.x[1]);
  block_tfi(mx, my, mz, Z, G.x[2]);
  return 0;
}

}  // namespace

std::string resolve_path(const std::string& base_dir, const std::string& name) {
  if (name.empty() || name[0] == '/' || base_dir.empty()) return name;
  return base_dir + "/" + name;
}

int read_f64(const std::string& path, size_t n, std::vector<double>& out, std::string& err) {
  std::FILE* f = std::fopen(path.c_str(), "rb");
  if (!f) {
    err = "cannot open " + path;
    return 1;
  }
  out.resize(n);
  const size_t got = std::fread(out.data(), sizeof(double), n, f);
  const bool more = std::fgetc(f) != EOF;
  std::fclose(f);
  if (got != n || more) {
    err = path + " does not hold " + std::to_string(n) + " FP64 values";
    return 1;
  }
  return 0;
}

int write_block_grids(const Problem& P, const std::string& out_dir, std::string& err) {
  Problem Q = P;
  Q.mesh_source = "compute";
  static const char ext[3] = {'X', 'Y', 'Z'};
  for (int b = 0; b < 2; ++b) {
    BlockGrid G;
    if (make_block_grid(Q, b, SurfaceMods(), G, err)) return 1;
    for (int c = 0; c < 3; ++c) {
      const std::string path = resolve_path(out_dir, "block_grid_" + std::to_string(b + 1) + "." + ext[c]);
      std::FILE* f = std::fopen(path.c_str(), "wb");
      if (!f) {
        err = "cannot write " + path;
        return 1;
      }
      const size_t n = std::fwrite(G.x[c].data(), sizeof(double), G.x[c].size(), f);
      std::fclose(f);
      if (n != G.x[c].size()) {
        err = "short write to " + path;
        return 1;
      }
    }
  }
  return 0;
}

int make_block_grid(const Problem& P, int block, const SurfaceMods& mods, BlockGrid& G,
                    std::string& err) {
  const BlockParams& bp = P.btp[block];
  G.nq = bp.nqrs[0];
  G.nr = bp.nqrs[1];
  G.ns = bp.nqrs[2];
  const size_t np = (size_t)G.nq * G.nr * G.ns;
  if (P.mesh_source == "file") {
    // init_grid_from_file (src/grid.f90:146-211): block_grid_<id>.X/Y/Z,
    // raw FP64 coordinates, q fastest; the seeded surface offsets do not apply
    static const char ext[3] = {'X', 'Y', 'Z'};
    for (int c = 0; c < 3; ++c) {
      const std::string path = resolve_path(P.base_dir, "block_grid_" + std::to_string(block + 1) + "." + ext[c]);
      if (read_f64(path, np, G.x[c], err)) return 1;
    }
    return 0;
  }
  if (P.mesh_source != "compute") {
    err = "mesh_source '" + P.mesh_source + "' is not supported ('compute' or 'file')";
    return 1;
  }
  if (P.type_of_mesh == "cartesian") {
    const double bh[3] = {(bp.bqrs[0] - bp.aqrs[0]) / (double)(G.nq - 1),
                          (bp.bqrs[1] - bp.aqrs[1]) / (double)(G.nr - 1),
                          (bp.bqrs[2] - bp.aqrs[2]) / (double)(G.ns - 1)};
    for (int c = 0; c < 3; ++c) G.x[c].resize(np);
    parallel_k(G.ns, [&](int k) {
      for (int j = 0; j < G.nr; ++j)
        for (int i = 0; i < G.nq; ++i) {
          const size_t p = (size_t)i + (size_t)G.nq * ((size_t)j + (size_t)G.nr * k);
          G.x[0][p] = bp.aqrs[0] + (double)i * bh[0];
          G.x[1][p] = bp.aqrs[1] + (double)j * bh[1];
          G.x[2][p] = bp.aqrs[2] + (double)k * bh[2];
        }
    });
  } else if (P.type_of_mesh == "curvilinear") {
    if (P.use_topography) {
      if (curvilinear_topo(P, bp, G, err)) return 1;
    } else if (curvilinear(bp, P.base_dir, G, err)) {
      return 1;
    }
  } else {
    err = "unknown type_of_mesh '" + P.type_of_mesh + "'";
    return 1;
  }
  // Seeded surface displacements, blended linearly into the block so the
  // opposite faces stay put.
  if (!mods.fault_offset.empty()) {
    if (mods.fault_offset.size() != (size_t)G.nr * G.ns) {
      err = "fault_offset has the wrong size";
      return 1;
    }
    parallel_k(G.ns, [&](int k) {
      for (int j = 0; j < G.nr; ++j)
        for (int i = 0; i < G.nq; ++i) {
          const double q = (double)i / (double)(G.nq - 1);
          const double w = (block == 0) ? q : 1.0 - q;
          G.x[0][(size_t)i + (size_t)G.nq * ((size_t)j + (size_t)G.nr * k)] +=
              w * mods.fault_offset[(size_t)j + (size_t)G.nr * k];
        }
    });
  }
  if (!mods.topo_offset.empty()) {
    if (mods.topo_offset.size() != (size_t)G.nq * G.ns) {
      err = "topo_offset has the wrong size";
      return 1;
    }
    parallel_k(G.ns, [&](int k) {
      for (int j = 0; j < G.nr; ++j)
        for (int i = 0; i < G.nq; ++i) {
          const double w = 1.0 - (double)j / (double)(G.nr - 1);
          G.x[1][(size_t)i + (size_t)G.nq * ((size_t)j + (size_t)G.nr * k)] +=
              w * mods.topo_offset[(size_t)i + (size_t)G.nq * k];
        }
    });
  }
  return 0;
}

namespace {

// Bounding box of every q row (j, k) of a block: min x, y, z then max x, y, z.
std::vector<double> row_boxes(const BlockGrid& G) {
  const int nq = G.nq, nr = G.nr, ns = G.ns;
  std::vector<double> box(6 * (size_t)nr * ns);
  parallel_k(ns, [&](int k) {
    for (size_t row = (size_t)nr * k; row < (size_t)nr * (k + 1); ++row) {
      double* b = &box[6 * row];
      for (int c = 0; c < 3; ++c) {
        const double* x = &G.x[c][row * nq];
        b[c] = *std::min_element(x, x + nq);
        b[3 + c] = *std::max_element(x, x + nq);
      }
    }
  });
  return box;
}

// Distance from p to a row's box: no point of the row is closer.  Each step
// (difference, square, sum, root) rounds monotonically, so the floating-point
// value is also at most that of any point of the row.
double box_distance(const double* b, const double* p) {
  double s = 0.0;
  for (int c = 0; c < 3; ++c) {
    const double e = p[c] < b[c] ? b[c] - p[c] : (p[c] > b[3 + c] ? p[c] - b[3 + c] : 0.0);
    s += e * e;
  }
  return std::sqrt(s);
}

}  // namespace

void find_station_points(const BlockGrid& G, const std::vector<double>& xyz, std::vector<int>& ijk,
                         std::vector<int>* which) {
  const int nq = G.nq, nr = G.nr, ns = G.ns;
  auto at = [&](int c, int i, int j, int k) {  // 1-based point
    return G.x[c][(size_t)(i - 1) + (size_t)nq * ((size_t)(j - 1) + (size_t)nr * (k - 1))];
  };
  auto half_diag = [&](int i, int j, int k) {
    const double hx = i < nq ? at(0, i + 1, j, k) - at(0, i, j, k) : at(0, nq, j, k) - at(0, nq - 1, j, k);
    const double hy = j < nr ? at(1, i, j + 1, k) - at(1, i, j, k) : at(1, i, nr, k) - at(1, i, nr - 1, k);
    const double hz = k < ns ? at(2, i, j, k + 1) - at(2, i, j, k) : at(2, i, j, ns) - at(2, i, j, ns - 1);
    return 0.5 * std::sqrt(hx * hx + hy * hy + hz * hz);
  };
  // A point is admissible only within half its local cell diagonal, so a
  // station scans only the rows whose box lies within the block's largest
  // half diagonal; the rows it skips hold no admissible point, and the scan
  // order (s, r, q with "<=": the last point at equal distance wins) is the
  // reference's, so the chosen point is the one the full scan picks.
  std::vector<double> plane_reach(ns, 0.0);
  parallel_k(ns, [&](int k0) {
    double m = 0.0;
    for (int j = 1; j <= nr; ++j)
      for (int i = 1; i <= nq; ++i) m = std::max(m, half_diag(i, j, k0 + 1));
    plane_reach[k0] = m;
  });
  const double reach = *std::max_element(plane_reach.begin(), plane_reach.end());
  const std::vector<double> box = row_boxes(G);
  for (size_t st = 0; st + 2 < xyz.size(); st += 3) {
    const double* p = &xyz[st];
    int best[3] = {-1, -1, -1};
    double mind = 1.0e8;
    for (int k = 1; k <= ns; ++k)
      for (int j = 1; j <= nr; ++j) {
        if (box_distance(&box[6 * ((size_t)(j - 1) + (size_t)nr * (k - 1))], p) > reach) continue;
        for (int i = 1; i <= nq; ++i) {
          const double dx = at(0, i, j, k) - p[0], dy = at(1, i, j, k) - p[1], dz = at(2, i, j, k) - p[2];
          const double d = std::sqrt(dx * dx + dy * dy + dz * dz);
          if (d <= mind && d <= half_diag(i, j, k)) {
            best[0] = i; best[1] = j; best[2] = k;
            mind = d;
          }
        }
      }
    if (best[0] > 0) {
      ijk.insert(ijk.end(), best, best + 3);
      if (which) which->push_back((int)(st / 3));
    }
  }
}

void nearest_grid_point(const BlockGrid& G, const double p[3], int n0[3]) {
  const int nq = G.nq, nr = G.nr, ns = G.ns;
  auto X = [&](int c, int i, int j, int k) {  // 0-based
    return G.x[c][(size_t)i + (size_t)nq * ((size_t)j + (size_t)nr * k)];
  };
  const std::vector<double> box = row_boxes(G);
  const size_t nrow = (size_t)nr * ns;
  auto row_min = [&](size_t row) {
    const int j = (int)(row % nr), k = (int)(row / nr);
    double m = 1.0e300;
    for (int i = 0; i < nq; ++i) {
      const double dx = X(0, i, j, k) - p[0], dy = X(1, i, j, k) - p[1], dz = X(2, i, j, k) - p[2];
      m = std::min(m, std::sqrt(dx * dx + dy * dy + dz * dz));
    }
    return m;
  };
  // an upper bound on the nearest distance from the row whose box is
  // closest, then the reference's scan (s, r, q with "<=") over the rows
  // that can hold a point that near
  size_t r0 = 0;
  double b0 = 1.0e300;
  for (size_t row = 0; row < nrow; ++row) {
    const double b = box_distance(&box[6 * row], p);
    if (b < b0) {
      b0 = b;
      r0 = row;
    }
  }
  const double bound = row_min(r0);
  n0[0] = n0[1] = n0[2] = 0;
  double mind = 1.0e8;
  for (int k = 0; k < ns; ++k)
    for (int j = 0; j < nr; ++j) {
      if (box_distance(&box[6 * ((size_t)j + (size_t)nr * k)], p) > bound) continue;
      for (int i = 0; i < nq; ++i) {
        const double dx = X(0, i, j, k) - p[0], dy = X(1, i, j, k) - p[1], dz = X(2, i, j, k) - p[2];
        const double d = std::sqrt(dx * dx + dy * dy + dz * dz);
        if (d <= mind) {
          n0[0] = i; n0[1] = j; n0[2] = k;
          mind = d;
        }
      }
    }
}

}  // namespace wql
