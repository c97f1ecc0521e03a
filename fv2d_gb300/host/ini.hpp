// ini.hpp -- the reference's .ini parameter reading, restated for the GB300
// driver: inih's line format (jtilly/inih, an empty submodule in the
// reference, version unpinned) and the reference's Reader registry
// (SimInfo.h:99-263), readInifile (SimInfo.h:529-568) and
// DeviceParams::init_from_inifile (SimInfo.h:356-459).
#pragma once

#include <map>
#include <ostream>
#include <set>
#include <stdexcept>
#include <string>

#include "../../include/fv2d_types.h"

namespace fv2d {

// inih-format file: "[section]", "name = value" / "name : value", ';' or '#'
// full-line comments, " ;" inline comments, indented continuation lines,
// surrounding whitespace stripped.  Keys are stored lower-cased as
// "section=name"; a repeated key appends "\n" + value.  Section names are kept
// as written.
class IniFile {
 public:
  IniFile() = default;
  explicit IniFile(const std::string &path);
  static IniFile from_string(const std::string &text);
  int error() const { return error_; }  // 0, -1 (cannot open) or the first bad line
  bool has_section(const std::string &section) const;
  bool has_value(const std::string &section, const std::string &name) const;
  const std::string *find(const std::string &section, const std::string &name) const;
  const std::map<std::string, std::string> &values() const { return values_; }
  const std::set<std::string> &sections() const { return sections_; }
  static std::string key(const std::string &section, const std::string &name);

 private:
  void parse(std::istream &in);
  std::map<std::string, std::string> values_;
  std::set<std::string> sections_;
  int error_ = 0;
};

// The reference's Reader: every lookup is recorded with its value as text and
// whether it came from the file, for the parameter echo (last.ini).  Real
// values go through float, exactly like INIReader::GetFloat + strtof.
class ParamReader {
 public:
  explicit ParamReader(IniFile ini) : ini_(std::move(ini)) {}
  bool get_bool(const std::string &s, const std::string &n, bool def);
  int get_int(const std::string &s, const std::string &n, int def);
  double get_float(const std::string &s, const std::string &n, double def);
  std::string get(const std::string &s, const std::string &n, const std::string &def);
  template <class T>
  T get_map(const std::map<std::string, T> &m, const std::string &s, const std::string &n, const std::string &def) {
    std::string v = get(s, n, def);
    auto it = m.find(v);
    if (it == m.end()) {
      std::string allowed = "\nallowed values: ";
      for (auto &e : m) allowed += e.first + ", ";
      throw std::runtime_error("bad parameter for " + n + ": " + allowed);
    }
    return it->second;
  }
  // SimInfo.h:224-262: "; Parameters used for the problem: ..." then every
  // recorded section that appears in the file, keys left-aligned.
  void write_echo(std::ostream &o) const;
  // SimInfo.h:501-527: warnings for unknown sections and keys.
  void check_validity(std::ostream &warn) const;
  const IniFile &ini() const { return ini_; }

 private:
  struct Value {
    std::string text;
    bool from_file = false;
  };
  void record(std::string s, std::string n, const std::string &text);
  IniFile ini_;
  std::map<std::string, std::map<std::string, Value>> values_;
};

// Run-level settings of Params that are not in fv2d_params (SimInfo.h:463-492).
struct RunConfig {
  std::string problem = "blast";
  std::string filename_out = "run";
  std::string output_path = "./";
  std::string restart_file;
  bool multiple_outputs = false;
};

// readInifile (SimInfo.h:529-568): fills p (starting from the reference
// defaults) and run; throws std::runtime_error like the reference on bad
// map-valued parameters.  Problem names map through Init.h:293-301 plus the
// extension problems ("sedov", "kh_step", "rt_hydrostatic").
void read_ini(ParamReader &reader, fv2d_params *p, RunConfig *run);
int problem_id(const std::string &name);  // -1 if unknown

}  // namespace fv2d
