// Host-side block geometry: grid point coordinates for one block.
//
// Cartesian blocks follow cartesian_grid_3d (src/grid.f90:213-240).
// Curvilinear blocks follow Curve_Grid_3D3 (src/grid.f90:471-1875): six
// boundary surfaces, each face meshed by 2D transfinite interpolation
// (Gen_Surf_Mesh, src/grid.f90:2418-2455), then 3D transfinite interpolation
// (Gen3_Curve_Mesh, src/grid.f90:2290-2416).  Without topography (:592-1160)
// the supported fault profiles are flat (default / 'No-path' / 'no_path'),
// 'analytical_tpv28' (:650-683), 'analytical_test_problem' (:790-841) and
// 'read_from_memomry_fractal' (:832-924); with use_topography = T
// (:1349-1875) the top face comes from 'read_topo_from_memory' or
// 'analytical_topography', and the fault is 'no_path' or
// 'read_from_memomry_fractal'.  Two extensions feed the seeded rough-fault and
// topography generators: `fault_offset` displaces the interface face along x
// and `topo_offset` displaces the r-min face along y (both given on the
// face's own (r,s) / (q,s) grid, see wql_surfaces.h).
#pragma once
#include <string>
#include <vector>

#include "wql_input.h"

namespace wql {

struct BlockGrid {
  int nq = 0, nr = 0, ns = 0;
  std::vector<double> x[3];  // index (i-1) + nq*((j-1) + nr*(k-1))
};

// Optional surface displacements (empty = none).
struct SurfaceMods {
  std::vector<double> fault_offset;  // nr*ns, x-offset of the interface face
  std::vector<double> topo_offset;   // nq*ns, y-offset of the r=1 face
};

int make_block_grid(const Problem& P, int block, const SurfaceMods& mods, BlockGrid& G,
                    std::string& err);

// name relative to base_dir (unchanged when absolute or base_dir is empty).
std::string resolve_path(const std::string& base_dir, const std::string& name);
// Reads exactly n FP64 values from a raw file.
int read_f64(const std::string& path, size_t n, std::vector<double>& out, std::string& err);
// The computed grids of both blocks as block_grid_<id>.X/Y/Z in out_dir,
// the files mesh_source = 'file' reads (what the reference's preprocessor
// program prepares, src/preprocessor.f90).
int write_block_grids(const Problem& P, const std::string& out_dir, std::string& err);

// Seismogram stations (Find_Coordinates, src/seismogram.f90:531-650): for
// each requested (x, y, z) the grid point nearest to it among the points
// within half their local cell diagonal; requests with no such point are
// dropped.  Appends 1-based (i, j, k) triples to ijk.
// which, if given, receives the request index of each point found.
void find_station_points(const BlockGrid& G, const std::vector<double>& xyz, std::vector<int>& ijk,
                         std::vector<int>* which = nullptr);

// The 0-based grid point nearest to p (scan order s, r, q; the last point at
// equal distance wins), the rule of the moment-tensor source placement.
void nearest_grid_point(const BlockGrid& G, const double p[3], int n0[3]);

}  // namespace wql
