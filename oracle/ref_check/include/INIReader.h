// INIReader.h -- TEST INFRASTRUCTURE.  Stand-in, written for this repository,
// for the jtilly/inih header (an empty submodule in the reference,
// .gitmodules:1-3, version unpinned).  It restates the published behaviour of
// inih's line parser and of that header's accessors that SimInfo.h relies on:
//   - '[section]' lines, 'name = value' or 'name : value' pairs, full-line
//     comments starting with ';' or '#', inline comments ' ;', surrounding
//     whitespace stripped, indented lines continuing the previous value;
//   - keys stored lower-cased as "section=name"; repeated keys joined by '\n';
//     section names stored as written;
//   - GetInteger: strtol(base 0), GetReal: strtod, GetFloat: strtof returning
//     float, GetBoolean: true/yes/on/1 and false/no/off/0 (any case);
//     the default is returned when nothing was parsed.
#pragma once
#include <algorithm>
#include <cctype>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <map>
#include <set>
#include <string>

class INIReader {
 public:
  INIReader() {}
  explicit INIReader(const std::string &filename) { _error = Parse(filename); }
  int ParseError() const { return _error; }
  const std::set<std::string> &Sections() const { return _sections; }

  std::string Get(const std::string &section, const std::string &name, const std::string &default_value) const {
    std::string key = MakeKey(section, name);
    auto it = _values.find(key);
    return it != _values.end() ? it->second : default_value;
  }
  long GetInteger(const std::string &section, const std::string &name, long default_value) const {
    std::string valstr = Get(section, name, "");
    const char *value = valstr.c_str();
    char *end;
    long n = std::strtol(value, &end, 0);
    return end > value ? n : default_value;
  }
  double GetReal(const std::string &section, const std::string &name, double default_value) const {
    std::string valstr = Get(section, name, "");
    const char *value = valstr.c_str();
    char *end;
    double n = std::strtod(value, &end);
    return end > value ? n : default_value;
  }
  float GetFloat(const std::string &section, const std::string &name, float default_value) const {
    std::string valstr = Get(section, name, "");
    const char *value = valstr.c_str();
    char *end;
    float n = std::strtof(value, &end);
    return end > value ? n : default_value;
  }
  bool GetBoolean(const std::string &section, const std::string &name, bool default_value) const {
    std::string valstr = Get(section, name, "");
    std::transform(valstr.begin(), valstr.end(), valstr.begin(), ::tolower);
    if (valstr == "true" || valstr == "yes" || valstr == "on" || valstr == "1") return true;
    if (valstr == "false" || valstr == "no" || valstr == "off" || valstr == "0") return false;
    return default_value;
  }

 protected:
  int _error = 0;
  std::map<std::string, std::string> _values;
  std::set<std::string> _sections;

  static std::string MakeKey(const std::string &section, const std::string &name) {
    std::string key = section + "=" + name;
    std::transform(key.begin(), key.end(), key.begin(), ::tolower);
    return key;
  }

 private:
  static std::string rstrip(const std::string &s) {
    size_t e = s.size();
    while (e > 0 && std::isspace((unsigned char)s[e - 1])) --e;
    return s.substr(0, e);
  }
  static std::string lskip(const std::string &s) {
    size_t b = 0;
    while (b < s.size() && std::isspace((unsigned char)s[b])) ++b;
    return s.substr(b);
  }
  // First of `chars` (or an inline ';' preceded by whitespace) in s.
  static size_t find_chars_or_comment(const std::string &s, const char *chars) {
    bool was_space = false;
    for (size_t k = 0; k < s.size(); ++k) {
      char c = s[k];
      if (chars && std::strchr(chars, c)) return k;
      if (was_space && c == ';') return k;
      was_space = std::isspace((unsigned char)c) != 0;
    }
    return std::string::npos;
  }
  void handle(const std::string &section, const std::string &name, const std::string &value) {
    std::string key = MakeKey(section, name);
    if (!_values[key].empty()) _values[key] += "\n";
    _values[key] += value;
    _sections.insert(section);
  }
  int Parse(const std::string &filename) {
    std::ifstream f(filename);
    if (!f) return -1;
    std::string line, section, prev_name;
    int lineno = 0, error = 0;
    while (std::getline(f, line)) {
      ++lineno;
      if (lineno == 1 && line.size() >= 3 && (unsigned char)line[0] == 0xEF && (unsigned char)line[1] == 0xBB &&
          (unsigned char)line[2] == 0xBF)
        line = line.substr(3);
      std::string start = lskip(rstrip(line));
      bool indented = !line.empty() && std::isspace((unsigned char)line[0]);
      if (start.empty() || start[0] == ';' || start[0] == '#') continue;
      if (!prev_name.empty() && indented) {
        handle(section, prev_name, start);
      } else if (start[0] == '[') {
        size_t e = find_chars_or_comment(start.substr(1), "]");
        if (e != std::string::npos && start[1 + e] == ']') {
          section = start.substr(1, e);
          prev_name.clear();
        } else if (!error) {
          error = lineno;
        }
      } else {
        size_t e = find_chars_or_comment(start, "=:");
        if (e != std::string::npos && (start[e] == '=' || start[e] == ':')) {
          std::string name = rstrip(start.substr(0, e));
          std::string value = lskip(start.substr(e + 1));
          size_t c = find_chars_or_comment(value, nullptr);
          if (c != std::string::npos) value = value.substr(0, c);
          value = rstrip(value);
          prev_name = name;
          handle(section, name, value);
        } else if (!error) {
          error = lineno;
        }
      }
    }
    return error;
  }
};
