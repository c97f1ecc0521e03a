// ini.cpp -- see ini.hpp.
#include "ini.hpp"

#include <algorithm>
#include <cctype>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <iomanip>
#include <sstream>

#include "../csrc/problems.h"

namespace fv2d {

namespace {
std::string lower(std::string s) {
  std::transform(s.begin(), s.end(), s.begin(), [](unsigned char c) { return (char)std::tolower(c); });
  return s;
}
std::string rstrip(const std::string &s) {
  size_t e = s.size();
  while (e > 0 && std::isspace((unsigned char)s[e - 1])) --e;
  return s.substr(0, e);
}
std::string lskip(const std::string &s) {
  size_t b = 0;
  while (b < s.size() && std::isspace((unsigned char)s[b])) ++b;
  return s.substr(b);
}
// First of `chars`, or a ';' preceded by whitespace (inline comment).
size_t find_chars_or_comment(const std::string &s, const char *chars) {
  bool was_space = false;
  for (size_t k = 0; k < s.size(); ++k) {
    const char c = s[k];
    if (chars && std::strchr(chars, c)) return k;
    if (was_space && c == ';') return k;
    was_space = std::isspace((unsigned char)c) != 0;
  }
  return std::string::npos;
}
}  // namespace

std::string IniFile::key(const std::string &section, const std::string &name) { return lower(section + "=" + name); }

IniFile::IniFile(const std::string &path) {
  std::ifstream f(path);
  if (!f) {
    error_ = -1;
    return;
  }
  parse(f);
}

IniFile IniFile::from_string(const std::string &text) {
  IniFile ini;
  std::istringstream in(text);
  ini.parse(in);
  return ini;
}

void IniFile::parse(std::istream &in) {
  std::string line, section, prev_name;
  int lineno = 0;
  auto handle = [&](const std::string &name, const std::string &value) {
    std::string &slot = values_[key(section, name)];
    if (!slot.empty()) slot += "\n";
    slot += value;
    sections_.insert(section);
  };
  while (std::getline(in, line)) {
    ++lineno;
    if (lineno == 1 && line.size() >= 3 && (unsigned char)line[0] == 0xEF && (unsigned char)line[1] == 0xBB &&
        (unsigned char)line[2] == 0xBF)
      line = line.substr(3);
    const std::string start = lskip(rstrip(line));
    const bool indented = !line.empty() && std::isspace((unsigned char)line[0]);
    if (start.empty() || start[0] == ';' || start[0] == '#') continue;
    if (!prev_name.empty() && indented) {
      handle(prev_name, start);
    } else if (start[0] == '[') {
      const size_t e = find_chars_or_comment(start.substr(1), "]");
      if (e != std::string::npos && start[1 + e] == ']') {
        section = start.substr(1, e);
        prev_name.clear();
      } else if (!error_) {
        error_ = lineno;
      }
    } else {
      const size_t e = find_chars_or_comment(start, "=:");
      if (e != std::string::npos && (start[e] == '=' || start[e] == ':')) {
        const std::string name = rstrip(start.substr(0, e));
        std::string value = lskip(start.substr(e + 1));
        const size_t c = find_chars_or_comment(value, nullptr);
        if (c != std::string::npos) value = value.substr(0, c);
        value = rstrip(value);
        prev_name = name;
        handle(name, value);
      } else if (!error_) {
        error_ = lineno;
      }
    }
  }
}

bool IniFile::has_section(const std::string &section) const {
  const std::string k = key(section, "");
  auto it = values_.lower_bound(k);
  return it != values_.end() && it->first.compare(0, k.size(), k) == 0;
}

bool IniFile::has_value(const std::string &section, const std::string &name) const {
  return values_.count(key(section, name)) != 0;
}

const std::string *IniFile::find(const std::string &section, const std::string &name) const {
  auto it = values_.find(key(section, name));
  return it == values_.end() ? nullptr : &it->second;
}

// ------------------------------------------------------------------ ParamReader
void ParamReader::record(std::string s, std::string n, const std::string &text) {
  const bool from_file = ini_.has_section(s) && ini_.has_value(s, n);
  s = lower(s);
  n = lower(n);
  if (values_.count(s) && values_.at(s).count(n)) throw std::runtime_error("parameter already set : " + n);
  Value &v = values_[s][n];
  v.text = text;
  v.from_file = from_file;
}

bool ParamReader::get_bool(const std::string &s, const std::string &n, bool def) {
  bool res = def;
  if (const std::string *v = ini_.find(s, n)) {
    const std::string l = lower(*v);
    if (l == "true" || l == "yes" || l == "on" || l == "1")
      res = true;
    else if (l == "false" || l == "no" || l == "off" || l == "0")
      res = false;
  }
  record(s, n, res ? "true" : "false");
  return res;
}

int ParamReader::get_int(const std::string &s, const std::string &n, int def) {
  long res = def;
  if (const std::string *v = ini_.find(s, n)) {
    const char *c = v->c_str();
    char *end;
    const long x = std::strtol(c, &end, 0);
    if (end > c) res = x;
  }
  record(s, n, std::to_string((int)res));
  return (int)res;
}

double ParamReader::get_float(const std::string &s, const std::string &n, double def) {
  float res = (float)def;  // the default is converted to float too
  if (const std::string *v = ini_.find(s, n)) {
    const char *c = v->c_str();
    char *end;
    const float x = std::strtof(c, &end);
    if (end > c) res = x;
  }
  std::ostringstream os;
  os << std::scientific << std::setprecision(12) << (double)res;
  record(s, n, os.str());
  return (double)res;
}

std::string ParamReader::get(const std::string &s, const std::string &n, const std::string &def) {
  const std::string *v = ini_.find(s, n);
  const std::string res = v ? *v : def;
  record(s, n, res);
  return res;
}

void ParamReader::write_echo(std::ostream &o) const {
  constexpr size_t name_width = 26, value_width = 20;
  std::string problem;
  auto ph = values_.find("physics");
  if (ph != values_.end()) {
    auto pv = ph->second.find("problem");
    if (pv != ph->second.end()) problem = pv->second.text;
  }
  const auto flags = o.flags();
  o << "; Parameters used for the problem: " << problem << std::endl;
  o << std::left;
  for (const auto &sec : values_) {
    if (!ini_.has_section(sec.first)) continue;
    o << "\n[" << sec.first << "]" << std::endl;
    for (const auto &var : sec.second) {
      o << std::setw((int)std::max(var.first.length(), name_width)) << var.first << " = "
        << std::setw((int)std::max(var.second.text.length(), value_width)) << var.second.text
        << (var.second.from_file ? "" : " ; default ") << std::endl;
    }
  }
  o.flags(flags);
}

void ParamReader::check_validity(std::ostream &warn) const {
  for (const auto &s : ini_.sections()) {
    auto it = values_.find(s);
    if (it == values_.end()) {
      warn << "WARNING: section [" << s << "] is unknown." << std::endl;
      continue;
    }
    const std::string prefix = s + "=";
    for (const auto &kv : ini_.values()) {
      if (kv.first.compare(0, prefix.size(), prefix) == 0) {
        const std::string name = kv.first.substr(prefix.size());
        if (!it->second.count(name))
          warn << "WARNING: parameter `" << name << "` in section [" << s << "] is unknown." << std::endl;
      }
    }
  }
}

// ------------------------------------------------------------------ readInifile
int problem_id(const std::string &name) {
  static const std::map<std::string, int> m{
      {"sod_x", FV2D_PB_SOD_X},
      {"sod_y", FV2D_PB_SOD_Y},
      {"blast", FV2D_PB_BLAST},
      {"rayleigh-taylor", FV2D_PB_RAYLEIGH_TAYLOR},
      {"diffusion", FV2D_PB_DIFFUSION},
      {"H84", FV2D_PB_H84},
      {"C91", FV2D_PB_C91},
      {"kelvin_helmholtz", FV2D_PB_KELVIN_HELMHOLTZ},
      {"gresho_vortex", FV2D_PB_GRESHO_VORTEX},
      {"sedov", FV2D_PB_SEDOV},
      {"kh_step", FV2D_PB_KH_STEP},
      {"rt_hydrostatic", FV2D_PB_RT_HYDROSTATIC},
  };
  auto it = m.find(name);
  return it == m.end() ? -1 : it->second;
}

void read_ini(ParamReader &r, fv2d_params *p, RunConfig *run) {
  params_default(p);
  // readInifile (SimInfo.h:535-551)
  p->tend = r.get_float("run", "tend", 1.0);
  run->multiple_outputs = r.get_bool("run", "multiple_outputs", false);
  run->restart_file = r.get("run", "restart_file", "");
  p->save_freq = r.get_float("run", "save_freq", 1.0e-1);
  run->filename_out = r.get("run", "output_filename", "run");
  run->output_path = r.get("run", "output_path", "./");
  p->time_stepping = r.get_map<int>({{"euler", FV2D_TS_EULER}, {"RK2", FV2D_TS_RK2}}, "solvers", "time_stepping",
                                    "euler");
  run->problem = r.get("physics", "problem", "blast");
  p->seed = r.get_int("misc", "seed", 12345);
  p->log_frequency = r.get_int("misc", "log_frequency", 10);
  p->epsilon_reset_negative = r.get_float("misc", "epsilon_reset_negative", 1.0e-8);
  // DeviceParams::init_from_inifile (SimInfo.h:359-458)
  p->Nx = r.get_int("mesh", "Nx", 32);
  p->Ny = r.get_int("mesh", "Ny", 32);
  p->Nghosts = r.get_int("mesh", "Nghosts", 2);
  p->xmin = r.get_float("mesh", "xmin", 0.0);
  p->xmax = r.get_float("mesh", "xmax", 1.0);
  p->ymin = r.get_float("mesh", "ymin", 0.0);
  p->ymax = r.get_float("mesh", "ymax", 1.0);
  p->CFL = r.get_float("solvers", "CFL", 0.8);
  const std::map<std::string, int> bc{{"reflecting", FV2D_BC_REFLECTING},
                                      {"absorbing", FV2D_BC_ABSORBING},
                                      {"periodic", FV2D_BC_PERIODIC}};
  p->boundary_x = r.get_map(bc, "run", "boundaries_x", "reflecting");
  p->boundary_y = r.get_map(bc, "run", "boundaries_y", "reflecting");
  p->reconstruction = r.get_map<int>({{"pcm", FV2D_PCM}, {"pcm_wb", FV2D_PCM_WB}, {"plm", FV2D_PLM},
                                      {"muscl_hancock", FV2D_MUSCL_HANCOCK}},
                                     "solvers", "reconstruction", "pcm");
  p->riemann_solver = r.get_map<int>({{"hll", FV2D_HLL}, {"hllc", FV2D_HLLC}, {"fslp", FV2D_FSLP}}, "solvers",
                                     "riemann_solver", "hllc");
  p->epsilon = r.get_float("misc", "epsilon", 1.0e-6);
  p->gamma0 = r.get_float("physics", "gamma0", 5.0 / 3.0);
  p->m1 = r.get_float("polytrope", "m1", 1.0);
  p->theta1 = r.get_float("polytrope", "theta1", 10.0);
  p->m2 = r.get_float("polytrope", "m2", 1.0);
  p->theta2 = r.get_float("polytrope", "theta2", 10.0);
  p->well_balanced_flux_at_y_bc = r.get_bool("physics", "well_balanced_flux_at_y_bc", false);
  p->fslp_K = r.get_float("physics", "fslp_K", 1.1);
  p->gravity_mode = r.get_map<int>({{"none", FV2D_GRAV_NONE}, {"constant", FV2D_GRAV_CONSTANT},
                                    {"analytical", FV2D_GRAV_ANALYTICAL}},
                                   "gravity", "mode", "none");
  p->gx = r.get_float("gravity", "gx", 0.0);
  p->gy = r.get_float("gravity", "gy", 0.0);
  p->analytical_gravity_mode = r.get_map<int>({{"hot_bubble", FV2D_AGM_HOT_BUBBLE}}, "gravity", "analytical_mode",
                                              "hot_bubble");
  p->thermal_conductivity_active = r.get_bool("thermal_conduction", "active", false);
  p->thermal_conductivity_mode = r.get_map<int>({{"constant", FV2D_TCM_CONSTANT}, {"B02", FV2D_TCM_B02}},
                                                "thermal_conduction", "conductivity_mode", "constant");
  p->kappa = r.get_float("thermal_conduction", "kappa", 0.0);
  const std::map<std::string, int> bctc{{"none", FV2D_BCTC_NONE},
                                        {"fixed_temperature", FV2D_BCTC_FIXED_TEMPERATURE},
                                        {"fixed_gradient", FV2D_BCTC_FIXED_GRADIENT}};
  p->bctc_ymin = r.get_map(bctc, "thermal_conduction", "bc_ymin", "none");
  p->bctc_ymax = r.get_map(bctc, "thermal_conduction", "bc_ymax", "none");
  p->bctc_ymin_value = r.get_float("thermal_conduction", "bc_ymin_value", 1.0);
  p->bctc_ymax_value = r.get_float("thermal_conduction", "bc_ymax_value", 1.0);
  p->viscosity_active = r.get_bool("viscosity", "active", false);
  p->viscosity_mode = r.get_map<int>({{"constant", FV2D_VSC_CONSTANT}}, "viscosity", "viscosity_mode", "constant");
  p->mu = r.get_float("viscosity", "mu", 0.0);
  p->h84_pert = r.get_float("H84", "perturbation", 1.0e-4);
  p->c91_pert = r.get_float("C91", "perturbation", 1.0e-3);
  p->hot_bubble_g0 = r.get_float("hot_bubble", "g0", 0.0);
  p->kh_a = r.get_float("kelvin_helmholtz", "a", 0.05);
  p->kh_amp = r.get_float("kelvin_helmholtz", "amp", 0.01);
  p->kh_P0 = r.get_float("kelvin_helmholtz", "P0", 1.0);
  p->kh_rho_fac = r.get_float("kelvin_helmholtz", "rho_fac", 0.0);
  p->kh_sigma = r.get_float("kelvin_helmholtz", "sigma", 0.2);
  p->kh_uflow = r.get_float("kelvin_helmholts", "uflow", 1.0);  // the reference's section name (SimInfo.h:452)
  p->kh_y1 = r.get_float("kelvin_helmholts", "y1", 0.5);
  p->kh_y2 = r.get_float("kelvin_helmholts", "y2", 1.5);
  p->gresho_density = r.get_float("gresho_vortex", "density", 1.0);
  p->gresho_Mach = r.get_float("gresho_vortex", "Mach", 0.1);
  // extension problems and the B02 constants, only when their section exists
  // (so the echo of a reference .ini is unchanged)
  const IniFile &ini = r.ini();
  if (ini.has_section("B02")) {
    p->b02_ymid = r.get_float("B02", "ymid", 0.0);
    p->b02_kappa1 = r.get_float("B02", "kappa1", 0.0);
    p->b02_kappa2 = r.get_float("B02", "kappa2", 0.0);
    p->b02_thickness = r.get_float("B02", "thickness", 1.0);
  }
  if (ini.has_section("sod")) {
    p->sod_rho_left = r.get_float("sod", "rho_left", 1.0);
    p->sod_p_left = r.get_float("sod", "p_left", 1.0);
    p->sod_rho_right = r.get_float("sod", "rho_right", 0.125);
    p->sod_p_right = r.get_float("sod", "p_right", 0.1);
  }
  if (ini.has_section("sedov")) {
    p->sedov_E0 = r.get_float("sedov", "E0", 1.0);
    p->sedov_r0 = r.get_float("sedov", "r0", 0.02);
    p->sedov_p_ambient = r.get_float("sedov", "p_ambient", 1.0e-5);
    p->sedov_rho = r.get_float("sedov", "rho", 1.0);
  }
  if (ini.has_section("kh_step")) {
    p->khs_rho_in = r.get_float("kh_step", "rho_in", 2.0);
    p->khs_rho_out = r.get_float("kh_step", "rho_out", 1.0);
    p->khs_u = r.get_float("kh_step", "u", 0.5);
    p->khs_p0 = r.get_float("kh_step", "p0", 2.5);
    p->khs_amp = r.get_float("kh_step", "amp", 0.01);
    p->khs_noise = r.get_float("kh_step", "noise", 1.0e-3);
  }
  if (ini.has_section("rt_hydrostatic")) {
    p->rt_rho_top = r.get_float("rt_hydrostatic", "rho_top", 2.0);
    p->rt_rho_bottom = r.get_float("rt_hydrostatic", "rho_bottom", 1.0);
    p->rt_p_interface = r.get_float("rt_hydrostatic", "p_interface", 2.5);
    p->rt_y_interface = r.get_float("rt_hydrostatic", "y_interface", 0.75);
    p->rt_amp = r.get_float("rt_hydrostatic", "amp", 0.01);
  }
}

}  // namespace fv2d
