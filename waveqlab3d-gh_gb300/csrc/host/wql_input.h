// Reader for WaveQLab3D `.in` input files (Fortran namelist subset).
//
// The reference reads its inputs with Fortran namelist I/O:
//   &problem_list   src/domain.f90:105-108 (defaults :115-133)
//   &block_list     src/domain.f90:110, type block_temp_parameters src/datatypes.f90:255-266
//                   (optionally from an external file, src/input_utils.f90:9-35)
//   &moment_list    src/block.f90:63
//   &output_list    src/seismogram.f90:58
//   marker blocks   !---begin:station_listU--- ... (src/seismogram.f90:181-202)
// This reader accepts the same syntax: `&group key = value, ... /`, `d`/`D`
// exponents, T/F/.true./.false., quoted strings, `btp(1)%nqrs = a, b, c`
// element syntax, `!` comments, and an absent group (tolerated like the
// reference's `iostat<0`).  Extension groups that the reference ignores
// (`&fault_list`, `&plastic_list`, `&gb300_list`) carry the parameters that
// the reference hard-codes per problem preset.
#pragma once
#include <map>
#include <string>
#include <vector>

namespace wql {

struct BlockParams {
  int nqrs[3] = {0, 0, 0};
  double aqrs[3] = {0, 0, 0}, bqrs[3] = {0, 0, 0};
  double lc = 0, rc = 0;
  double rho_s_p[3] = {0, 0, 0};
  double mu_beta_eta[3] = {0, 0, 0};
  int lqrs[3] = {0, 0, 0}, rqrs[3] = {0, 0, 0};
  std::string profile_type, profile_path, topography_type, topography_path;
  // material_source = 'file': lambda, mu, rho as raw FP64 arrays, q fastest
  // (init_material_from_file, src/material.f90:706-747)
  std::string material_path[3];
  bool pml_lqrs[3] = {false, false, false}, pml_rqrs[3] = {false, false, false};
  int npml = 0;
  int faultsize[2] = {0, 0};
};

// Parameters the reference hard-codes per `problem` preset; the extension
// groups override them (used by the seeded configurations).
struct FrictionExt {
  bool set = false;          // &fault_list present
  // slip weakening (IC:1283-1299 defaults for TPV5)
  double fs = 0.677, fd = 0.525, Dc = 0.4;
  double barrier_y = 15.0, barrier_z = 15.0;
  // rate and state, aging law (IC:386-393, IC:433)
  double a = 0.008, b = 0.012, V0 = 1.0e-6, f0 = 0.6, L = 0.02, Vini = 1.0e-12;
  // uniform background stress tensor (sxx, syy, szz, sxy, sxz, syz), projected
  // on each fault point's (n, m, l) frame like the TPV101 preset
  // (src/Interface_Condition.f90:2324-2342), plus a Gaussian overstress
  double s0[6] = {-120.0, 0.0, -120.0, 0.0, 75.0, 0.0};
  // optional depth-dependent tensor instead of s0: the name of a preset
  // with an initial_stress_tensor (e.g. 'TPV26', src/initial_stress_condition.f90:26-50)
  std::string stress_profile;
  double nuc_amp = 0.0, nuc_radius = 1.5, nuc_y = 7.5, nuc_z = 0.0, nuc_rise = 1.0;
};

struct PlasticExt {
  bool set = false;          // &plastic_list present
  double cohesion = 1.36, friction = 0.1934, Tv = 0.03;   // src/plastic.f90:174-176
};

// &anelastic_list (src/material.f90:28-41): quality factor scale c
// (Qs = c * vs), the weight-set selector weight_exp (0 or 0.6) and the
// reference frequency fref (Hz) of the unrelaxed moduli.
struct AnelasticParams {
  double c = 1.0, weight_exp = 0.0, fref = 1.0;
};

// One moment-tensor point source, a line of a tensor list
// (src/moment_tensor.f90:232-246): source_type duration t_init
// mXX mYY mZZ mXY mXZ mYZ x y z alpha.
struct MomentSource {
  std::string type = "gaussian";
  double duration = 0.0, t_init = 0.0;
  double m[6] = {0, 0, 0, 0, 0, 0};  // XX, YY, ZZ, XY, XZ, YZ (stress components 4..9)
  double x = 0.0, y = 0.0, z = 0.0;
  int alpha = 0;
};

struct Problem {
  // &problem_list (defaults from src/domain.f90:115-133)
  std::string name = "default", problem = "TPV5", response = "elastic",
              plastic_model = "default", coupling = "locked",
              fd_type = "traditional", type_of_mesh = "cartesian",
              mesh_source = "compute", material_source = "hardcode";
  // directory that relative file names of the input resolve against (the
  // .in file's directory; empty: the process's working directory)
  std::string base_dir;
  int nblocks = 2, nt = 0, order = 5, w_stride = 1;
  double CFL = 0.5, t_final = 0.0, topo = 1.0;
  bool w_fault = true, interpol = false, use_topography = false,
       mollify_source = false;
  BlockParams btp[2];
  AnelasticParams anel;  // response = 'anelastic'
  // &moment_list (src/block.f90:63)
  bool use_moment_tensor = false;
  int mt_order = 2;
  int mt_block_preference = 1;
  // tensor lists (src/moment_tensor.f90:106-260): the unified
  // '!---begin:tensor_list---' for both blocks, else tensor_listU / tensor_listV
  bool mt_unified = false;
  std::vector<MomentSource> tensors, tensorsU, tensorsV;
  // &mms_list (src/mms.f90:17-49): the manufactured solution
  // u = cos(nt pi t) * (sin sin sin for velocities, cos cos cos for stresses)
  // of (nx pi x, ny pi y, nz pi z), defaults nt = 2, nx = ny = nz = 1
  bool use_mms = false;
  double mms_nt = 2.0, mms_nx = 1.0, mms_ny = 1.0, mms_nz = 1.0;
  // &output_list (src/seismogram.f90:58-82): seismograms on/off, the station
  // file directory (default 'seismogram') and the file naming by physical
  // position instead of grid index
  bool output_seismograms = false;
  std::string station_file_directory = "seismogram";
  bool station_xyz_index = false;
  // station marker blocks (src/seismogram.f90:181-202): x y z per line
  std::vector<double> stationsU, stationsV;
  // one list for both blocks ('!---begin:station_list---', src/seismogram.f90:157-176);
  // when present it replaces the per-block lists
  std::vector<double> stations;
  // &gb300_list: boundary SAT penalty weights.  'characteristic' is the form
  // compiled by the reference (src/BoundaryConditions.f90:777-918 followed by
  // structure(), src/RHS_Interior.f90:2203-2223); 'weighted' is the
  // alpha/theta form of src/BoundaryConditions3.f90:777-903, which the
  // reference's regression fixtures (test_problems/truth/1) were produced with.
  std::string bc_penalty = "characteristic";
  // &gb300_list tpv28_prestress: 'source' is the TPV28 stress tensor of
  // src/initial_stress_condition.f90:78-83 (szz = +60 MPa); 'benchmark' has
  // szz = -60 MPa, the SCEC TPV28 value.  The reference's curvilinear
  // regression fixture (test_problems/truth/2) was produced with 'benchmark'.
  std::string tpv28_prestress = "source";
  // &gb300_list rs_tol, rs_maxit: tolerance and iteration cap of the FP64
  // rate-and-state regula falsi (src/Interface_Condition.f90:1188, :1194).
  // The defaults are the reference's; a tolerance of 1e-300 iterates to a
  // floating-point fixed point, which lets two implementations of the solve
  // be compared to rounding.
  double rs_tol = 1.0e-12;
  int rs_maxit = 5000;
  // &gb300_list fp32c_fault: in the FP32-compensated mode the fault's
  // characteristic algebra works on the FP32 fields in FP32 ('fp32'), or
  // reads the compensated face values (F - C) and runs in FP64
  // ('compensated').  Measured on 2 x 201^3 curvilinear rate and state over
  // 2000 steps: velocity error against FP64 2.27e-5 ('fp32') and 2.25e-5
  // ('compensated'), for 0.07 against 0.22 ms per interface launch.
  std::string fp32c_fault = "fp32";
  FrictionExt fric;
  PlasticExt plast;
  // raw groups for anything not mapped above
  std::map<std::string, std::map<std::string, std::string>> raw;
};

// Parse a .in file. Returns 0 on success; on failure fills `err`.
int parse_in_file(const std::string& path, Problem& P, std::string& err);
int parse_in_text(const std::string& text, const std::string& base_dir,
                  Problem& P, std::string& err);

}  // namespace wql
