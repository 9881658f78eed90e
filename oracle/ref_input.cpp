// ORACLE — test infrastructure only.  Nothing in the product links or calls
// this file; only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline
// leg load it (inside oracle/_build/libwqlref.so).
//
// The oracle's own reader of the reference's `.in` input files, written apart
// from the library's reader (csrc/host/wql_input.cpp) so that the parity
// tests check the library's parsing too: tests/test_oracle_input.py compares
// the two readers' results field by field on every input the tests use.  It
// fills the shared wql::Problem record, but assigns every default itself.
//
// Syntax: Fortran namelist input as the reference's decks use it
// (`&group key = value, ... /`, `btp(1)%field = a, b, c`, quoted strings,
// d/D exponents, T/F/.true./.false., `!` comments), an absent group read as
// the defaults (the reference's `iostat < 0`), the block list from an
// external file (`&block_list = 'file'`, src/input_utils.f90:9-90), and the
// station and moment-tensor marker blocks (src/seismogram.f90:157-202,
// src/moment_tensor.f90:106-260).
#include <cctype>
#include <cmath>
#include <cstdlib>
#include <fstream>
#include <map>
#include <sstream>
#include <string>
#include <vector>

#include "wql_input.h"

namespace oref {
namespace {

using wql::Problem;

std::string low(std::string s) {
  for (auto& c : s) c = (char)std::tolower((unsigned char)c);
  return s;
}

std::string strip(const std::string& s) {
  size_t a = 0, b = s.size();
  while (a < b && std::isspace((unsigned char)s[a])) ++a;
  while (b > a && std::isspace((unsigned char)s[b - 1])) --b;
  return s.substr(a, b - a);
}

// One namelist token: a quoted string (its text), a bare word, or '='.
struct Tok {
  enum Kind { STR, WORD, EQ } kind;
  std::string text;
};

// Tokens of every `&name ... /` group of the text, by lower-case group name
// (a group may occur more than once; the occurrences are concatenated).
std::map<std::string, std::vector<Tok>> scan_groups(const std::string& text) {
  std::map<std::string, std::vector<Tok>> out;
  // drop comments: '!' outside quotes to the end of the line
  std::string t;
  char q = 0;
  for (size_t i = 0; i < text.size(); ++i) {
    char c = text[i];
    if (q) {
      if (c == q) q = 0;
      if (c == '\n') q = 0;
      t += c;
      continue;
    }
    if (c == '\'' || c == '"') q = c;
    if (c == '!') {
      while (i < text.size() && text[i] != '\n') ++i;
      t += '\n';
      continue;
    }
    t += c;
  }
  size_t i = 0;
  while ((i = t.find('&', i)) != std::string::npos) {
    size_t e = i + 1;
    while (e < t.size() && (std::isalnum((unsigned char)t[e]) || t[e] == '_')) ++e;
    const std::string name = low(t.substr(i + 1, e - i - 1));
    std::vector<Tok>& toks = out[name];
    size_t k = e;
    while (k < t.size()) {
      const char c = t[k];
      if (c == '/') {
        ++k;
        break;
      }
      if (std::isspace((unsigned char)c) || c == ',') {
        ++k;
        continue;
      }
      if (c == '=') {
        toks.push_back({Tok::EQ, "="});
        ++k;
        continue;
      }
      if (c == '\'' || c == '"') {
        const size_t end = t.find(c, k + 1);
        const size_t stop = end == std::string::npos ? t.size() : end;
        toks.push_back({Tok::STR, t.substr(k + 1, stop - k - 1)});
        k = stop + 1;
        continue;
      }
      size_t w = k;
      while (w < t.size() && !std::isspace((unsigned char)t[w]) && t[w] != ',' && t[w] != '=' && t[w] != '/') ++w;
      toks.push_back({Tok::WORD, t.substr(k, w - k)});
      k = w;
    }
    i = k;
  }
  return out;
}

// key = values assignments of a token list, keys in lower case.
std::vector<std::pair<std::string, std::vector<std::string>>> assignments(const std::vector<Tok>& toks) {
  std::vector<std::pair<std::string, std::vector<std::string>>> out;
  for (size_t i = 0; i < toks.size(); ++i) {
    if (toks[i].kind == Tok::WORD && i + 1 < toks.size() && toks[i + 1].kind == Tok::EQ) {
      out.push_back({low(toks[i].text), {}});
      ++i;
      continue;
    }
    if (!out.empty() && toks[i].kind != Tok::EQ) out.back().second.push_back(toks[i].text);
  }
  return out;
}

double num(const std::string& v) {
  std::string s = v;
  for (auto& c : s)
    if (c == 'd' || c == 'D') c = 'e';
  return std::strtod(s.c_str(), nullptr);
}

int inum(const std::string& v) { return (int)std::lround(num(v)); }

bool logical(const std::string& v) {
  std::string s = low(strip(v));
  if (!s.empty() && s[0] == '.') s.erase(0, 1);
  return !s.empty() && s[0] == 't';
}

// Lines between `!---begin:<tag>---` and `!---end:<tag>---`, blank and
// comment lines left out.
std::vector<std::string> marker_lines(const std::string& text, const std::string& tag, bool* present) {
  std::vector<std::string> out;
  std::istringstream in(text);
  std::string line;
  bool inside = false;
  if (present) *present = false;
  while (std::getline(in, line)) {
    const std::string s = strip(line);
    if (s == "!---begin:" + tag + "---") {
      inside = true;
      if (present) *present = true;
      continue;
    }
    if (s == "!---end:" + tag + "---") break;
    if (inside && !s.empty() && s[0] != '!') out.push_back(s);
  }
  return out;
}

std::vector<std::string> words(const std::string& line) {
  std::vector<std::string> out;
  std::string w;
  char q = 0;
  for (char c : line + " ") {
    if (q) {
      if (c == q) q = 0;
      else w += c;
      continue;
    }
    if (c == '\'' || c == '"') {
      q = c;
      continue;
    }
    if (std::isspace((unsigned char)c) || c == ',') {
      if (!w.empty()) out.push_back(w);
      w.clear();
    } else {
      w += c;
    }
  }
  return out;
}

void defaults(Problem& P) {
  // &problem_list: src/domain.f90:115-133; type_of_mesh and nblocks have no
  // default there (the decks always set them): cartesian and 2 here
  P.name = "default";
  P.problem = "TPV5";
  P.response = "elastic";
  P.plastic_model = "default";
  P.nt = 0;
  P.CFL = 0.5;
  P.coupling = "locked";
  P.t_final = 0.0;
  P.w_fault = true;
  P.mesh_source = "compute";
  P.material_source = "hardcode";
  P.w_stride = 1;
  P.interpol = false;
  P.use_topography = false;
  P.mollify_source = false;
  P.topo = 1.0;
  P.fd_type = "traditional";
  P.order = 5;
  P.type_of_mesh = "cartesian";
  P.nblocks = 2;
  // block_temp_parameters (src/datatypes.f90:255-266) has no initial values:
  // zeros and empty strings
  for (auto& b : P.btp) b = wql::BlockParams();
  for (auto& b : P.btp) {
    for (int d = 0; d < 3; ++d) {
      b.nqrs[d] = 0;
      b.aqrs[d] = b.bqrs[d] = b.rho_s_p[d] = b.mu_beta_eta[d] = 0.0;
      b.lqrs[d] = b.rqrs[d] = 0;
      b.pml_lqrs[d] = b.pml_rqrs[d] = false;
      b.material_path[d].clear();
    }
    b.lc = b.rc = 0.0;
    b.profile_type.clear();
    b.profile_path.clear();
    b.topography_type.clear();
    b.topography_path.clear();
    b.npml = 0;
    b.faultsize[0] = b.faultsize[1] = 0;
  }
  // &moment_list: src/block.f90:72-74
  P.use_moment_tensor = false;
  P.mt_order = 2;
  P.mt_block_preference = 1;
  // &output_list: src/seismogram.f90:66-80
  P.output_seismograms = false;
  P.station_file_directory = "seismogram";
  P.station_xyz_index = false;
  // &anelastic_list: src/material.f90:30-32
  P.anel.c = 1.0;
  P.anel.weight_exp = 0.0;
  P.anel.fref = 1.0;
  // &mms_list: src/mms.f90:32-36
  P.use_mms = false;
  P.mms_nt = 2.0;
  P.mms_nx = P.mms_ny = P.mms_nz = 1.0;
  // extension groups of this build (not in the reference)
  P.bc_penalty = "characteristic";
  P.tpv28_prestress = "source";
  P.rs_tol = 1.0e-12;  // the reference's tolerance, src/Interface_Condition.f90:1188
  P.rs_maxit = 5000;   // src/Interface_Condition.f90:1194
  P.fp32c_fault = "fp32";
  P.fric = wql::FrictionExt();
  P.fric.set = false;
  P.fric.fs = 0.677; P.fric.fd = 0.525; P.fric.Dc = 0.4;   // IC:1283-1299
  P.fric.barrier_y = 15.0; P.fric.barrier_z = 15.0;
  P.fric.a = 0.008; P.fric.b = 0.012; P.fric.V0 = 1.0e-6; P.fric.f0 = 0.6; P.fric.L = 0.02;  // IC:386-393
  P.fric.Vini = 1.0e-12;  // IC:2782
  const double s0[6] = {-120.0, 0.0, -120.0, 0.0, 75.0, 0.0};  // src/initial_stress_condition.f90:114-120
  for (int c = 0; c < 6; ++c) P.fric.s0[c] = s0[c];
  P.fric.stress_profile.clear();
  P.fric.nuc_amp = 0.0; P.fric.nuc_radius = 1.5; P.fric.nuc_y = 7.5; P.fric.nuc_z = 0.0; P.fric.nuc_rise = 1.0;
  P.plast = wql::PlasticExt();
  P.plast.set = false;
  P.plast.cohesion = 1.36; P.plast.friction = 0.1934; P.plast.Tv = 0.03;  // src/plastic.f90:174-176
  P.stationsU.clear();
  P.stationsV.clear();
  P.stations.clear();
  P.tensors.clear();
  P.tensorsU.clear();
  P.tensorsV.clear();
  P.mt_unified = false;
  P.raw.clear();
}

void block_field(wql::BlockParams& b, const std::string& f, const std::vector<std::string>& v) {
  auto nums = [&](double* d, int n) {
    for (int i = 0; i < n && i < (int)v.size(); ++i) d[i] = num(v[i]);
  };
  auto ints = [&](int* d, int n) {
    for (int i = 0; i < n && i < (int)v.size(); ++i) d[i] = inum(v[i]);
  };
  auto logs = [&](bool* d, int n) {
    for (int i = 0; i < n && i < (int)v.size(); ++i) d[i] = logical(v[i]);
  };
  const std::string first = v.empty() ? std::string() : v[0];
  if (f == "nqrs") ints(b.nqrs, 3);
  else if (f == "aqrs") nums(b.aqrs, 3);
  else if (f == "bqrs") nums(b.bqrs, 3);
  else if (f == "rho_s_p") nums(b.rho_s_p, 3);
  else if (f == "mu_beta_eta") nums(b.mu_beta_eta, 3);
  else if (f == "lqrs") ints(b.lqrs, 3);
  else if (f == "rqrs") ints(b.rqrs, 3);
  else if (f == "lc") b.lc = num(first);
  else if (f == "rc") b.rc = num(first);
  else if (f == "profile_type") b.profile_type = first;
  else if (f == "profile_path") b.profile_path = first;
  else if (f == "topography_type") b.topography_type = first;
  else if (f == "topography_path") b.topography_path = first;
  else if (f == "pml_lqrs") logs(b.pml_lqrs, 3);
  else if (f == "pml_rqrs") logs(b.pml_rqrs, 3);
  else if (f == "npml") b.npml = inum(first);
  else if (f == "faultsize") ints(b.faultsize, 2);
  else if (f == "material_path")
    for (int i = 0; i < 3 && i < (int)v.size(); ++i) b.material_path[i] = v[i];
  else if (f.compare(0, 14, "material_path(") == 0) {
    const int i = std::atoi(f.c_str() + 14) - 1;
    if (i >= 0 && i < 3) b.material_path[i] = first;
  }
}

}  // namespace

int read_in_text(const std::string& text, const std::string& base_dir, Problem& P, std::string& err) {
  defaults(P);
  P.base_dir = base_dir;
  auto groups = scan_groups(text);
  auto assign = [&](const char* g) { return assignments(groups[g]); };
  for (auto& [k, v] : assign("problem_list")) {
    const std::string s = v.empty() ? std::string() : v[0];
    if (k == "name") P.name = s;
    else if (k == "problem") P.problem = s;
    else if (k == "response") P.response = s;
    else if (k == "plastic_model") P.plastic_model = s;
    else if (k == "nblocks") P.nblocks = inum(s);
    else if (k == "nt") P.nt = inum(s);
    else if (k == "cfl") P.CFL = num(s);
    else if (k == "coupling") P.coupling = s;
    else if (k == "fd_type") P.fd_type = s;
    else if (k == "order") P.order = inum(s);
    else if (k == "t_final") P.t_final = num(s);
    else if (k == "mesh_source") P.mesh_source = s;
    else if (k == "type_of_mesh") P.type_of_mesh = s;
    else if (k == "material_source") P.material_source = s;
    else if (k == "interpol") P.interpol = logical(s);
    else if (k == "w_stride") P.w_stride = inum(s);
    else if (k == "w_fault") P.w_fault = logical(s);
    else if (k == "use_topography") P.use_topography = logical(s);
    else if (k == "topo") P.topo = num(s);
    else if (k == "mollify_source") P.mollify_source = logical(s);
  }
  // src/domain.f90:146-162
  if (P.response != "elastic" && P.response != "plastic" && P.response != "anelastic") {
    err = "invalid response option '" + P.response + "'";
    return 1;
  }
  // &block_list, or the file it names (src/input_utils.f90:54-90)
  std::vector<Tok> bl = groups["block_list"];
  if (bl.size() >= 2 && bl[0].kind == Tok::EQ) {
    std::string path = bl[1].text;
    if (!path.empty() && path[0] != '/' && !base_dir.empty()) path = base_dir + "/" + path;
    std::ifstream f(path);
    if (!f) {
      err = "error opening block list file " + path;
      return 1;
    }
    std::stringstream ss;
    ss << f.rdbuf();
    bl = scan_groups(ss.str())["block_list"];
  }
  for (auto& [k, v] : assignments(bl)) {
    if (k.compare(0, 4, "btp(") != 0) continue;
    const size_t close = k.find(')'), pct = k.find('%');
    if (close == std::string::npos || pct == std::string::npos) continue;
    const int blk = std::atoi(k.c_str() + 4) - 1;
    if (blk >= 0 && blk < 2) block_field(P.btp[blk], k.substr(pct + 1), v);
  }
  for (auto& [k, v] : assign("moment_list")) {
    const std::string s = v.empty() ? std::string() : v[0];
    if (k == "use_moment_tensor") P.use_moment_tensor = logical(s);
    else if (k == "order") P.mt_order = inum(s);
    else if (k == "tensor_block_preference") P.mt_block_preference = inum(s);
  }
  for (auto& [k, v] : assign("output_list")) {
    const std::string s = v.empty() ? std::string() : v[0];
    if (k == "output_seismograms") P.output_seismograms = logical(s);
    else if (k == "station_file_directory") P.station_file_directory = s;
    else if (k == "station_xyz_index") P.station_xyz_index = logical(s);
  }
  for (auto& [k, v] : assign("anelastic_list")) {
    const double x = v.empty() ? 0.0 : num(v[0]);
    if (k == "c") P.anel.c = x;
    else if (k == "weight_exp") P.anel.weight_exp = x;
    else if (k == "fref") P.anel.fref = x;
  }
  for (auto& [k, v] : assign("mms_list")) {
    const std::string s = v.empty() ? std::string() : v[0];
    if (k == "use_mms") P.use_mms = logical(s);
    else if (k == "nt") P.mms_nt = num(s);
    else if (k == "nx") P.mms_nx = num(s);
    else if (k == "ny") P.mms_ny = num(s);
    else if (k == "nz") P.mms_nz = num(s);
  }
  for (auto& [k, v] : assign("gb300_list")) {
    const std::string s = v.empty() ? std::string() : v[0];
    if (k == "bc_penalty") P.bc_penalty = s;
    else if (k == "tpv28_prestress") P.tpv28_prestress = s;
    else if (k == "rs_tol") P.rs_tol = num(s);
    else if (k == "rs_maxit") P.rs_maxit = inum(s);
    else if (k == "fp32c_fault") P.fp32c_fault = s;
  }
  if (groups.count("fault_list")) {
    P.fric.set = true;
    for (auto& [k, v] : assign("fault_list")) {
      if (k == "stress_profile") {
        P.fric.stress_profile = v.empty() ? std::string() : v[0];
        continue;
      }
      const double x = v.empty() ? 0.0 : num(v[0]);
      if (k == "fs") P.fric.fs = x;
      else if (k == "fd") P.fric.fd = x;
      else if (k == "dc") P.fric.Dc = x;
      else if (k == "barrier_y") P.fric.barrier_y = x;
      else if (k == "barrier_z") P.fric.barrier_z = x;
      else if (k == "a") P.fric.a = x;
      else if (k == "b") P.fric.b = x;
      else if (k == "v0") P.fric.V0 = x;
      else if (k == "f0") P.fric.f0 = x;
      else if (k == "l") P.fric.L = x;
      else if (k == "vini") P.fric.Vini = x;
      else if (k == "nuc_amp") P.fric.nuc_amp = x;
      else if (k == "nuc_radius") P.fric.nuc_radius = x;
      else if (k == "nuc_y") P.fric.nuc_y = x;
      else if (k == "nuc_z") P.fric.nuc_z = x;
      else if (k == "nuc_rise") P.fric.nuc_rise = x;
      else if (k == "s0")
        for (int c = 0; c < 6 && c < (int)v.size(); ++c) P.fric.s0[c] = num(v[c]);
    }
  }
  if (groups.count("plastic_list")) {
    P.plast.set = true;
    for (auto& [k, v] : assign("plastic_list")) {
      const double x = v.empty() ? 0.0 : num(v[0]);
      if (k == "cohesion") P.plast.cohesion = x;
      else if (k == "friction") P.plast.friction = x;
      else if (k == "tv") P.plast.Tv = x;
    }
  }
  // station marker blocks: x y z per line
  auto xyz = [&](const char* tag) {
    std::vector<double> out;
    for (auto& line : marker_lines(text, tag, nullptr))
      for (auto& w : words(line)) out.push_back(num(w));
    return out;
  };
  P.stationsU = xyz("station_listU");
  P.stationsV = xyz("station_listV");
  P.stations = xyz("station_list");
  // moment-tensor lists: source_type duration t_init mXX mYY mZZ mXY mXZ mYZ x y z alpha
  auto tensors = [&](const char* tag, bool* present) {
    std::vector<wql::MomentSource> out;
    for (auto& line : marker_lines(text, tag, present)) {
      auto w = words(line);
      if (w.size() < 13) continue;
      wql::MomentSource m;
      m.type = w[0];
      m.duration = num(w[1]);
      m.t_init = num(w[2]);
      for (int c = 0; c < 6; ++c) m.m[c] = num(w[3 + c]);
      m.x = num(w[9]);
      m.y = num(w[10]);
      m.z = num(w[11]);
      m.alpha = inum(w[12]);
      out.push_back(m);
    }
    return out;
  };
  P.tensors = tensors("tensor_list", &P.mt_unified);
  P.tensorsU = tensors("tensor_listU", nullptr);
  P.tensorsV = tensors("tensor_listV", nullptr);
  return 0;
}

int read_in_file(const std::string& path, Problem& P, std::string& err) {
  std::ifstream f(path);
  if (!f) {
    err = "cannot open " + path;
    return 1;
  }
  std::stringstream ss;
  ss << f.rdbuf();
  const size_t slash = path.find_last_of('/');
  return read_in_text(ss.str(), slash == std::string::npos ? std::string() : path.substr(0, slash), P, err);
}

}  // namespace oref
