// Namelist reader for WaveQLab3D `.in` files; see wql_input.h for the
// reference locations of every group.
#include "wql_input.h"

#include <cctype>
#include <cmath>
#include <cstdlib>
#include <fstream>
#include <sstream>

namespace wql {
namespace {

std::string lower(std::string s) {
  for (auto& c : s) c = (char)std::tolower((unsigned char)c);
  return s;
}

std::string trim(const std::string& s) {
  size_t a = 0, b = s.size();
  while (a < b && std::isspace((unsigned char)s[a])) ++a;
  while (b > a && std::isspace((unsigned char)s[b - 1])) --b;
  return s.substr(a, b - a);
}

// Remove `!` comments that are outside quotes.
std::string strip_comment(const std::string& line) {
  char q = 0;
  for (size_t i = 0; i < line.size(); ++i) {
    char c = line[i];
    if (q) {
      if (c == q) q = 0;
    } else if (c == '\'' || c == '"') {
      q = c;
    } else if (c == '!') {
      return line.substr(0, i);
    }
  }
  return line;
}

// Split the body of one namelist group into `key = values` items.  A new item
// starts at an identifier followed by `=` (outside quotes).
struct Item {
  std::string key;
  std::vector<std::string> values;
};

std::vector<std::string> split_values(const std::string& rhs) {
  std::vector<std::string> out;
  std::string cur;
  char q = 0;
  for (size_t i = 0; i < rhs.size(); ++i) {
    char c = rhs[i];
    if (q) {
      if (c == q) {
        q = 0;
      } else {
        cur += c;
      }
      continue;
    }
    if (c == '\'' || c == '"') {
      q = c;
      continue;
    }
    if (c == ',' || std::isspace((unsigned char)c)) {
      if (!trim(cur).empty()) out.push_back(trim(cur));
      cur.clear();
      continue;
    }
    cur += c;
  }
  if (!trim(cur).empty()) out.push_back(trim(cur));
  return out;
}

std::vector<Item> split_items(const std::string& body) {
  // Find positions of '=' outside quotes and walk back to the key start.
  std::vector<std::pair<size_t, size_t>> keys;  // (key_start, eq_pos)
  char q = 0;
  for (size_t i = 0; i < body.size(); ++i) {
    char c = body[i];
    if (q) {
      if (c == q) q = 0;
      continue;
    }
    if (c == '\'' || c == '"') {
      q = c;
      continue;
    }
    if (c == '=') {
      size_t e = i;
      while (e > 0 && std::isspace((unsigned char)body[e - 1])) --e;
      size_t s = e;
      while (s > 0) {
        char p = body[s - 1];
        if (std::isalnum((unsigned char)p) || p == '_' || p == '%' || p == '(' ||
            p == ')' || p == ':')
          --s;
        else
          break;
      }
      keys.push_back({s, i});
    }
  }
  std::vector<Item> items;
  for (size_t k = 0; k < keys.size(); ++k) {
    size_t vs = keys[k].second + 1;
    size_t ve = (k + 1 < keys.size()) ? keys[k + 1].first : body.size();
    Item it;
    it.key = lower(trim(body.substr(keys[k].first, keys[k].second - keys[k].first)));
    it.values = split_values(body.substr(vs, ve - vs));
    items.push_back(it);
  }
  return items;
}

double to_double(const std::string& v) {
  std::string s = v;
  for (auto& c : s)
    if (c == 'd' || c == 'D') c = 'e';
  return std::strtod(s.c_str(), nullptr);
}

bool to_bool(const std::string& v) {
  std::string s = lower(v);
  if (!s.empty() && s[0] == '.') s = s.substr(1);
  return !s.empty() && s[0] == 't';
}

// Collect `&group ... /` bodies.  The terminating `/` is outside quotes.
std::map<std::string, std::vector<std::string>> groups_of(const std::string& text) {
  std::map<std::string, std::vector<std::string>> out;
  std::string clean;
  {
    std::istringstream is(text);
    std::string line;
    while (std::getline(is, line)) clean += strip_comment(line) + "\n";
  }
  size_t i = 0;
  while (true) {
    size_t a = clean.find('&', i);
    if (a == std::string::npos) break;
    size_t e = a + 1;
    while (e < clean.size() && (std::isalnum((unsigned char)clean[e]) || clean[e] == '_')) ++e;
    std::string gname = lower(clean.substr(a + 1, e - a - 1));
    char q = 0;
    size_t j = e;
    for (; j < clean.size(); ++j) {
      char c = clean[j];
      if (q) {
        if (c == q) q = 0;
        continue;
      }
      if (c == '\'' || c == '"') {
        q = c;
        continue;
      }
      if (c == '/') break;
    }
    out[gname].push_back(clean.substr(e, j - e));
    i = j + 1;
  }
  return out;
}

// Parse `btp(1)%nqrs` -> (block index, field); plain keys give block -1.
bool parse_btp_key(const std::string& key, int& blk, std::string& field) {
  if (key.rfind("btp(", 0) != 0) return false;
  size_t close = key.find(')');
  if (close == std::string::npos) return false;
  blk = std::atoi(key.substr(4, close - 4).c_str()) - 1;
  size_t pct = key.find('%', close);
  if (pct == std::string::npos) return false;
  field = key.substr(pct + 1);
  return true;
}

void set_block_field(BlockParams& b, const std::string& field,
                     const std::vector<std::string>& v) {
  auto dv = [&](double* dst, int n) {
    for (int i = 0; i < n && i < (int)v.size(); ++i) dst[i] = to_double(v[i]);
  };
  auto iv = [&](int* dst, int n) {
    for (int i = 0; i < n && i < (int)v.size(); ++i) dst[i] = (int)std::lround(to_double(v[i]));
  };
  auto bv = [&](bool* dst, int n) {
    for (int i = 0; i < n && i < (int)v.size(); ++i) dst[i] = to_bool(v[i]);
  };
  auto sv = [&]() { return v.empty() ? std::string() : v[0]; };
  if (field == "nqrs") iv(b.nqrs, 3);
  else if (field == "aqrs") dv(b.aqrs, 3);
  else if (field == "bqrs") dv(b.bqrs, 3);
  else if (field == "lc") dv(&b.lc, 1);
  else if (field == "rc") dv(&b.rc, 1);
  else if (field == "rho_s_p") dv(b.rho_s_p, 3);
  else if (field == "mu_beta_eta") dv(b.mu_beta_eta, 3);
  else if (field == "lqrs") iv(b.lqrs, 3);
  else if (field == "rqrs") iv(b.rqrs, 3);
  else if (field == "profile_type") b.profile_type = sv();
  else if (field == "profile_path") b.profile_path = sv();
  else if (field == "topography_type") b.topography_type = sv();
  else if (field == "topography_path") b.topography_path = sv();
  else if (field == "pml_lqrs") bv(b.pml_lqrs, 3);
  else if (field == "pml_rqrs") bv(b.pml_rqrs, 3);
  else if (field == "npml") iv(&b.npml, 1);
  else if (field == "faultsize") iv(b.faultsize, 2);
  else if (field == "material_path")
    for (int i = 0; i < 3 && i < (int)v.size(); ++i) b.material_path[i] = v[i];
  else if (field.rfind("material_path(", 0) == 0) {
    const int i = std::atoi(field.c_str() + 14) - 1;
    if (i >= 0 && i < 3) b.material_path[i] = sv();
  }
}

std::vector<double> marker_block(const std::string& text, const std::string& tag) {
  std::vector<double> out;
  std::istringstream is(text);
  std::string line;
  bool in = false;
  while (std::getline(is, line)) {
    std::string t = trim(line);
    if (t == "!---begin:" + tag + "---") {
      in = true;
      continue;
    }
    if (t == "!---end:" + tag + "---") break;
    if (!in || t.empty() || t[0] == '!') continue;
    for (auto& s : split_values(t)) out.push_back(to_double(s));
  }
  return out;
}

bool has_marker(const std::string& text, const std::string& tag) {
  std::istringstream is(text);
  std::string line;
  while (std::getline(is, line))
    if (trim(line) == "!---begin:" + tag + "---") return true;
  return false;
}

// Moment-tensor lines between markers (blank and '!' lines skipped,
// src/moment_tensor.f90:24-30).
std::vector<MomentSource> tensor_block(const std::string& text, const std::string& tag) {
  std::vector<MomentSource> out;
  std::istringstream is(text);
  std::string line;
  bool in = false;
  while (std::getline(is, line)) {
    std::string t = trim(line);
    if (t == "!---begin:" + tag + "---") {
      in = true;
      continue;
    }
    if (t == "!---end:" + tag + "---") break;
    if (!in || t.empty() || t[0] == '!') continue;
    auto v = split_values(t);
    if (v.size() < 13) continue;
    MomentSource m;
    m.type = v[0];
    m.duration = to_double(v[1]);
    m.t_init = to_double(v[2]);
    for (int c = 0; c < 6; ++c) m.m[c] = to_double(v[3 + c]);
    m.x = to_double(v[9]);
    m.y = to_double(v[10]);
    m.z = to_double(v[11]);
    m.alpha = (int)to_double(v[12]);
    out.push_back(m);
  }
  return out;
}

}  // namespace

int parse_in_text(const std::string& text, const std::string& base_dir,
                  Problem& P, std::string& err) {
  P.base_dir = base_dir;
  auto groups = groups_of(text);
  auto items_of = [&](const char* g) {
    std::vector<Item> all;
    auto it = groups.find(g);
    if (it == groups.end()) return all;
    for (auto& body : it->second)
      for (auto& item : split_items(body)) all.push_back(item);
    return all;
  };
  for (auto& kv : groups)
    for (auto& body : kv.second)
      for (auto& item : split_items(body))
        P.raw[kv.first][item.key] = item.values.empty() ? "" : item.values[0];

  for (auto& it : items_of("problem_list")) {
    auto s = it.values.empty() ? std::string() : it.values[0];
    const auto& k = it.key;
    if (k == "name") P.name = s;
    else if (k == "problem") P.problem = s;
    else if (k == "response") P.response = s;
    else if (k == "plastic_model") P.plastic_model = s;
    else if (k == "coupling") P.coupling = s;
    else if (k == "fd_type") P.fd_type = s;
    else if (k == "type_of_mesh") P.type_of_mesh = s;
    else if (k == "mesh_source") P.mesh_source = s;
    else if (k == "material_source") P.material_source = s;
    else if (k == "nblocks") P.nblocks = (int)to_double(s);
    else if (k == "nt") P.nt = (int)to_double(s);
    else if (k == "order") P.order = (int)to_double(s);
    else if (k == "w_stride") P.w_stride = (int)to_double(s);
    else if (k == "cfl") P.CFL = to_double(s);
    else if (k == "t_final") P.t_final = to_double(s);
    else if (k == "topo") P.topo = to_double(s);
    else if (k == "w_fault") P.w_fault = to_bool(s);
    else if (k == "interpol") P.interpol = to_bool(s);
    else if (k == "use_topography") P.use_topography = to_bool(s);
    else if (k == "mollify_source") P.mollify_source = to_bool(s);
  }
  // response validation (src/domain.f90:146-162)
  if (P.response != "elastic" && P.response != "plastic" && P.response != "anelastic") {
    err = "invalid response option in &problem_list: \"" + P.response + "\"";
    return 1;
  }

  // &block_list, inline or from an external file (src/input_utils.f90:9-35)
  std::vector<Item> blist;
  auto gi = groups.find("block_list");
  bool external = false;
  if (gi != groups.end()) {
    for (auto& body : gi->second) {
      std::string t = trim(body);
      if (!t.empty() && t[0] == '=') {
        auto vals = split_values(t.substr(1));
        if (!vals.empty()) {
          std::string path = vals[0];
          if (!path.empty() && path[0] != '/' && !base_dir.empty()) path = base_dir + "/" + path;
          std::ifstream f(path);
          if (!f) {
            err = "error opening block list file " + path;
            return 1;
          }
          std::stringstream ss;
          ss << f.rdbuf();
          auto g2 = groups_of(ss.str());
          for (auto& b2 : g2["block_list"])
            for (auto& item : split_items(b2)) blist.push_back(item);
          external = true;
        }
      }
    }
    if (!external) blist = items_of("block_list");
  }
  for (auto& it : blist) {
    int blk;
    std::string field;
    if (parse_btp_key(it.key, blk, field) && blk >= 0 && blk < 2)
      set_block_field(P.btp[blk], field, it.values);
  }

  for (auto& it : items_of("mms_list")) {
    auto s = it.values.empty() ? std::string() : it.values[0];
    if (it.key == "use_mms") P.use_mms = to_bool(s);
    else if (it.key == "nt") P.mms_nt = to_double(s);
    else if (it.key == "nx") P.mms_nx = to_double(s);
    else if (it.key == "ny") P.mms_ny = to_double(s);
    else if (it.key == "nz") P.mms_nz = to_double(s);
  }
  for (auto& it : items_of("moment_list")) {
    auto s = it.values.empty() ? std::string() : it.values[0];
    if (it.key == "use_moment_tensor") P.use_moment_tensor = to_bool(s);
    else if (it.key == "order") P.mt_order = (int)to_double(s);
    else if (it.key == "tensor_block_preference") P.mt_block_preference = (int)to_double(s);
  }
  P.mt_unified = has_marker(text, "tensor_list");
  P.tensors = tensor_block(text, "tensor_list");
  P.tensorsU = tensor_block(text, "tensor_listU");
  P.tensorsV = tensor_block(text, "tensor_listV");
  for (auto& it : items_of("output_list")) {
    auto s = it.values.empty() ? std::string() : it.values[0];
    if (it.key == "output_seismograms") P.output_seismograms = to_bool(s);
    else if (it.key == "station_file_directory") P.station_file_directory = s;
    else if (it.key == "station_xyz_index") P.station_xyz_index = to_bool(s);
  }
  for (auto& it : items_of("gb300_list")) {
    auto s = it.values.empty() ? std::string() : it.values[0];
    if (it.key == "bc_penalty") P.bc_penalty = s;
    else if (it.key == "tpv28_prestress") P.tpv28_prestress = s;
    else if (it.key == "rs_tol") P.rs_tol = to_double(s);
    else if (it.key == "rs_maxit") P.rs_maxit = (int)to_double(s);
    else if (it.key == "fp32c_fault") P.fp32c_fault = s;
  }
  if (P.bc_penalty != "characteristic" && P.bc_penalty != "weighted") {
    err = "bc_penalty must be 'characteristic' or 'weighted'";
    return 1;
  }
  if (P.tpv28_prestress != "source" && P.tpv28_prestress != "benchmark") {
    err = "tpv28_prestress must be 'source' or 'benchmark'";
    return 1;
  }
  if (P.fp32c_fault != "compensated" && P.fp32c_fault != "fp32") {
    err = "fp32c_fault must be 'compensated' or 'fp32'";
    return 1;
  }
  if (!(P.rs_tol > 0.0) || P.rs_maxit < 1 || P.rs_maxit > 1000000) {
    err = "rs_tol must be positive and rs_maxit in 1..1000000";
    return 1;
  }
  if (groups.count("fault_list")) {
    P.fric.set = true;
    for (auto& it : items_of("fault_list"))
      if (it.key == "stress_profile" && !it.values.empty()) P.fric.stress_profile = it.values[0];
    for (auto& it : items_of("fault_list")) {
      double v = it.values.empty() ? 0.0 : to_double(it.values[0]);
      const auto& k = it.key;
      if (k == "fs") P.fric.fs = v;
      else if (k == "fd") P.fric.fd = v;
      else if (k == "dc") P.fric.Dc = v;
      else if (k == "barrier_y") P.fric.barrier_y = v;
      else if (k == "barrier_z") P.fric.barrier_z = v;
      else if (k == "a") P.fric.a = v;
      else if (k == "b") P.fric.b = v;
      else if (k == "v0") P.fric.V0 = v;
      else if (k == "f0") P.fric.f0 = v;
      else if (k == "l") P.fric.L = v;
      else if (k == "vini") P.fric.Vini = v;
      else if (k == "s0")
        for (int c = 0; c < 6 && c < (int)it.values.size(); ++c) P.fric.s0[c] = to_double(it.values[c]);
      else if (k == "nuc_amp") P.fric.nuc_amp = v;
      else if (k == "nuc_radius") P.fric.nuc_radius = v;
      else if (k == "nuc_y") P.fric.nuc_y = v;
      else if (k == "nuc_z") P.fric.nuc_z = v;
      else if (k == "nuc_rise") P.fric.nuc_rise = v;
    }
  }
  if (groups.count("plastic_list")) {
    P.plast.set = true;
    for (auto& it : items_of("plastic_list")) {
      double v = it.values.empty() ? 0.0 : to_double(it.values[0]);
      if (it.key == "cohesion") P.plast.cohesion = v;
      else if (it.key == "friction") P.plast.friction = v;
      else if (it.key == "tv") P.plast.Tv = v;
    }
  }
  if (groups.count("anelastic_list")) {
    for (auto& it : items_of("anelastic_list")) {
      double v = it.values.empty() ? 0.0 : to_double(it.values[0]);
      if (it.key == "c") P.anel.c = v;
      else if (it.key == "weight_exp") P.anel.weight_exp = v;
      else if (it.key == "fref") P.anel.fref = v;
    }
  }
  P.stationsU = marker_block(text, "station_listU");
  P.stationsV = marker_block(text, "station_listV");
  P.stations = marker_block(text, "station_list");

  if (P.nblocks != 2) {
    err = "only two blocks joined by one q-interface are supported (src/domain.f90:243-244)";
    return 1;
  }
  for (int b = 0; b < 2; ++b)
    for (int d = 0; d < 3; ++d)
      if (P.btp[b].nqrs[d] < 12) {
        err = "block " + std::to_string(b + 1) +
              " needs at least 12 points per axis for the 6th-order SBP closures";
        return 1;
      }
  return 0;
}

int parse_in_file(const std::string& path, Problem& P, std::string& err) {
  std::ifstream f(path);
  if (!f) {
    err = "cannot open input file " + path;
    return 1;
  }
  std::stringstream ss;
  ss << f.rdbuf();
  std::string base;
  size_t slash = path.find_last_of('/');
  if (slash != std::string::npos) base = path.substr(0, slash);
  return parse_in_text(ss.str(), base, P, err);
}

}  // namespace wql
