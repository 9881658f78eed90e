"""The library's `.in` reader (csrc/host/wql_input.cpp) against the oracle's
own reader (oracle/ref_input.cpp), written apart from it: both parse every
input the tests and the benchmark use, and every field of the parsed record
must agree.  A parsing or default-value error in either shows up here
instead of hiding inside parity runs that share it."""
import os
import subprocess

import pytest

from inputs import MT_CASES, case_text, golden_in, mms_case, set_key, topography_case, with_groups

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HOST = os.path.join(ROOT, "waveqlab3d-gh_gb300", "csrc", "host")

# One program per reader: reads a .in path, prints every field of the record.
_DUMP = r"""
#include <cstdio>
#include <string>
#include "wql_input.h"
READER_DECL
static void d(const char* k, double v) { std::printf("%s %.17g\n", k, v); }
static void s(const char* k, const std::string& v) { std::printf("%s [%s]\n", k, v.c_str()); }
int main(int argc, char** argv) {
  wql::Problem P;
  std::string err;
  if (READER(argv[1], P, err)) { std::printf("error\n"); return 0; }
  s("name", P.name); s("problem", P.problem); s("response", P.response); s("plastic_model", P.plastic_model);
  s("coupling", P.coupling); s("fd_type", P.fd_type); s("type_of_mesh", P.type_of_mesh);
  s("mesh_source", P.mesh_source); s("material_source", P.material_source); s("base_dir", P.base_dir);
  d("nblocks", P.nblocks); d("nt", P.nt); d("order", P.order); d("w_stride", P.w_stride); d("CFL", P.CFL);
  d("t_final", P.t_final); d("topo", P.topo); d("w_fault", P.w_fault); d("interpol", P.interpol);
  d("use_topography", P.use_topography); d("mollify_source", P.mollify_source);
  for (int b = 0; b < 2; ++b) {
    const wql::BlockParams& B = P.btp[b];
    for (int i = 0; i < 3; ++i) {
      d("nqrs", B.nqrs[i]); d("aqrs", B.aqrs[i]); d("bqrs", B.bqrs[i]); d("rho_s_p", B.rho_s_p[i]);
      d("mu_beta_eta", B.mu_beta_eta[i]); d("lqrs", B.lqrs[i]); d("rqrs", B.rqrs[i]);
      d("pml_lqrs", B.pml_lqrs[i]); d("pml_rqrs", B.pml_rqrs[i]); s("material_path", B.material_path[i]);
    }
    d("lc", B.lc); d("rc", B.rc); d("npml", B.npml); d("faultsize0", B.faultsize[0]); d("faultsize1", B.faultsize[1]);
    s("profile_type", B.profile_type); s("profile_path", B.profile_path);
    s("topography_type", B.topography_type); s("topography_path", B.topography_path);
  }
  d("anel_c", P.anel.c); d("anel_w", P.anel.weight_exp); d("anel_fref", P.anel.fref);
  d("use_moment_tensor", P.use_moment_tensor); d("mt_order", P.mt_order); d("mt_pref", P.mt_block_preference);
  d("mt_unified", P.mt_unified);
  for (auto* L : {&P.tensors, &P.tensorsU, &P.tensorsV}) {
    d("tensors", (double)L->size());
    for (auto& m : *L) {
      s("type", m.type); d("duration", m.duration); d("t_init", m.t_init);
      for (int c = 0; c < 6; ++c) d("m", m.m[c]);
      d("x", m.x); d("y", m.y); d("z", m.z); d("alpha", m.alpha);
    }
  }
  d("output_seismograms", P.output_seismograms); s("station_dir", P.station_file_directory);
  d("station_xyz_index", P.station_xyz_index);
  for (auto* L : {&P.stationsU, &P.stationsV, &P.stations}) {
    d("stations", (double)L->size());
    for (double v : *L) d("xyz", v);
  }
  s("bc_penalty", P.bc_penalty); s("tpv28_prestress", P.tpv28_prestress); d("rs_tol", P.rs_tol);
  d("rs_maxit", P.rs_maxit); s("fp32c_fault", P.fp32c_fault);
  d("fric_set", P.fric.set); d("fs", P.fric.fs); d("fd", P.fric.fd); d("Dc", P.fric.Dc);
  d("barrier_y", P.fric.barrier_y); d("barrier_z", P.fric.barrier_z); d("a", P.fric.a); d("b", P.fric.b);
  d("V0", P.fric.V0); d("f0", P.fric.f0); d("L", P.fric.L); d("Vini", P.fric.Vini);
  for (int c = 0; c < 6; ++c) d("s0", P.fric.s0[c]);
  s("stress_profile", P.fric.stress_profile); d("nuc_amp", P.fric.nuc_amp); d("nuc_radius", P.fric.nuc_radius);
  d("nuc_y", P.fric.nuc_y); d("nuc_z", P.fric.nuc_z); d("nuc_rise", P.fric.nuc_rise);
  d("plast_set", P.plast.set); d("cohesion", P.plast.cohesion); d("friction", P.plast.friction); d("Tv", P.plast.Tv);
  d("use_mms", P.use_mms); d("mms_nt", P.mms_nt); d("mms_nx", P.mms_nx); d("mms_ny", P.mms_ny);
  d("mms_nz", P.mms_nz);
  return 0;
}
"""


@pytest.fixture(scope="module")
def readers(tmp_path_factory):
    d = tmp_path_factory.mktemp("readers")
    out = {}
    for name, decl, call, src in (
            ("library", "", "wql::parse_in_file", os.path.join(HOST, "wql_input.cpp")),
            ("oracle", "namespace oref { int read_in_file(const std::string&, wql::Problem&, std::string&); }",
             "oref::read_in_file", os.path.join(ROOT, "oracle", "ref_input.cpp"))):
        cpp = d / f"{name}.cpp"
        cpp.write_text(_DUMP.replace("READER_DECL", decl).replace("READER", call))
        exe = d / name
        subprocess.run(["g++", "-std=c++17", "-O0", "-I" + HOST, str(cpp), src, "-o", str(exe)], check=True)
        out[name] = str(exe)
    return out


def _decks(tmp_path):
    import wql_configs
    decks = {"truth1": golden_in("test_rup_cart_fric"), "truth2": golden_in("test_rup_curv_fric"),
             "truth2_bench": with_groups(golden_in("test_rup_curv_fric"),
                                         "&gb300_list\n bc_penalty = 'weighted', tpv28_prestress = 'benchmark',\n"
                                         " rs_tol = 1d-300, rs_maxit = 200000, fp32c_fault = 'compensated' /"),
             "curv_flat": set_key(golden_in("test_rup_cart_fric"), "type_of_mesh", "'curvilinear'")}
    for c in ("pml", "pml_curv", "plastic", "rs", "rs_curv", "locked", "linear_mt4", "an_up_pml", "an0_pml",
              "up5_pml", *MT_CASES):
        decks[c] = case_text(c)
    decks["mms"] = mms_case(21)[0]
    decks["topography"] = topography_case(tmp_path)
    decks["config0"] = wql_configs.config0()[0]
    decks["config1"] = wql_configs.config1(n=33, steps=5)[0]
    decks["config2"] = wql_configs.config2(nq=33, nrs=25, steps=5, npml=6)[0]
    decks["config3"] = wql_configs.config3_scenario(0, n_lo=32, n_hi=40, steps=5)[0]
    decks["config4"] = wql_configs.config4_request(0, n_lo=32, n_hi=40, steps=5)[0]
    decks["upwind"] = wql_configs.upwind_pml12(steps=5)[0]
    decks["upwind_drp"] = case_text("mt4").replace(" w_stride = 1,", " w_stride = 1,\n fd_type = 'upwind_drp',\n"
                                                                     " order = 66,", 1)
    return decks


def test_readers_agree_on_every_deck(readers, tmp_path):
    decks = _decks(tmp_path)
    for name, text in decks.items():
        path = tmp_path / f"{name}.in"
        path.write_text(text)
        dumps = {k: subprocess.run([exe, str(path)], check=True, capture_output=True, text=True).stdout
                 for k, exe in readers.items()}
        assert "error" not in dumps["oracle"], name
        lib, orc = dumps["library"].splitlines(), dumps["oracle"].splitlines()
        assert len(lib) == len(orc), name
        diff = [(a, b) for a, b in zip(lib, orc) if a != b]
        assert not diff, (name, diff[:5])


def test_readers_agree_on_the_external_block_list(readers, tmp_path):
    """&block_list = 'file' reads the block list from that file
    (src/input_utils.f90:54-90)."""
    text = golden_in("test_rup_cart_fric")
    start, end = text.index("&block_list"), text.index("/", text.index("&block_list"))
    (tmp_path / "blocks.nml").write_text(text[start:end + 1] + "\n")
    main = text[:start] + "&block_list = 'blocks.nml' /" + text[end + 1:]
    path = tmp_path / "ext.in"
    path.write_text(main)
    inline = tmp_path / "inline.in"
    inline.write_text(text)
    outs = [subprocess.run([exe, str(p)], check=True, capture_output=True, text=True).stdout
            for exe in readers.values() for p in (path, inline)]
    strip = lambda s: [l for l in s.splitlines() if not l.startswith("base_dir")]  # noqa: E731
    assert strip(outs[0]) == strip(outs[1]) == strip(outs[2]) == strip(outs[3])
