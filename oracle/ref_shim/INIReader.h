// Stand-in for the inih INIReader that the psvWave reference reads its
// configuration with (src/fdModel.cpp:475-518). inih is an un-vendored
// submodule of the reference (.gitmodules:4-6) and is absent here.
//
// Behaviour restated from inih's documented rules, as far as the reference's
// configuration files exercise them:
//  * "[section]" lines open a section; text after ']' is ignored;
//  * "name = value" or "name: value" lines; names are case-insensitive;
//  * whole-line comments start with ';' or '#';
//  * an inline comment starts at a ';' that follows whitespace, so
//    "8000;   int" keeps its ';' while "{90, 180} ;" loses the comment;
//  * GetInteger/GetReal parse the longest numeric prefix (strtol base 0 /
//    strtod) and fall back to the default when nothing parses;
//  * ParseError() is 0 on success, -1 when the file cannot be opened, or the
//    first line number that is neither a section, a pair nor a comment.
//
// Test infrastructure only: compiled solely into oracle/_ref.
#ifndef PSV_REF_SHIM_INIREADER_H
#define PSV_REF_SHIM_INIREADER_H

#include <cctype>
#include <cstdlib>
#include <fstream>
#include <map>
#include <sstream>
#include <string>

class INIReader {
 public:
  explicit INIReader(const std::string &filename) : error_(0) {
    std::ifstream in(filename.c_str());
    if (!in.good()) {
      error_ = -1;
      return;
    }
    std::string line, section;
    int lineno = 0;
    while (std::getline(in, line)) {
      ++lineno;
      if (!line.empty() && line[line.size() - 1] == '\r') line.erase(line.size() - 1);
      std::string s = trim(line);
      if (s.empty() || s[0] == ';' || s[0] == '#') continue;
      if (s[0] == '[') {
        std::size_t end = scan(s, 1, "]");
        if (end < s.size() && s[end] == ']') {
          section = trim(s.substr(1, end - 1));
        } else if (!error_) {
          error_ = lineno;
        }
        continue;
      }
      std::size_t sep = scan(s, 0, "=:");
      if (sep < s.size() && (s[sep] == '=' || s[sep] == ':')) {
        std::string name = trim(s.substr(0, sep));
        std::string value = trim(s.substr(sep + 1));
        std::size_t cut = scan(value, 0, "");
        value = trim(value.substr(0, cut));
        std::string key = lower(section) + "=" + lower(name);
        std::map<std::string, std::string>::iterator it = values_.find(key);
        if (it == values_.end())
          values_[key] = value;
        else
          it->second += "\n" + value;
      } else if (!error_) {
        error_ = lineno;
      }
    }
  }

  int ParseError() const { return error_; }

  std::string Get(const std::string &section, const std::string &name,
                  const std::string &default_value = "") const {
    std::map<std::string, std::string>::const_iterator it =
        values_.find(lower(section) + "=" + lower(name));
    return it == values_.end() ? default_value : it->second;
  }

  long GetInteger(const std::string &section, const std::string &name,
                  long default_value = 0) const {
    std::string v = Get(section, name, "");
    const char *p = v.c_str();
    char *end = 0;
    long n = std::strtol(p, &end, 0);
    return end > p ? n : default_value;
  }

  double GetReal(const std::string &section, const std::string &name,
                 double default_value = 0.0) const {
    std::string v = Get(section, name, "");
    const char *p = v.c_str();
    char *end = 0;
    double n = std::strtod(p, &end);
    return end > p ? n : default_value;
  }

 private:
  static std::string trim(const std::string &s) {
    std::size_t a = 0, b = s.size();
    while (a < b && std::isspace(static_cast<unsigned char>(s[a]))) ++a;
    while (b > a && std::isspace(static_cast<unsigned char>(s[b - 1]))) --b;
    return s.substr(a, b - a);
  }
  static std::string lower(std::string s) {
    for (std::size_t i = 0; i < s.size(); ++i)
      s[i] = static_cast<char>(std::tolower(static_cast<unsigned char>(s[i])));
    return s;
  }
  // First position holding one of `stops`, or an inline ';' comment (a ';'
  // right after whitespace), or s.size().
  static std::size_t scan(const std::string &s, std::size_t from, const char *stops) {
    bool was_space = false;
    for (std::size_t i = from; i < s.size(); ++i) {
      char c = s[i];
      for (const char *q = stops; *q; ++q)
        if (c == *q) return i;
      if (was_space && c == ';') return i;
      was_space = std::isspace(static_cast<unsigned char>(c)) != 0;
    }
    return s.size();
  }

  int error_;
  std::map<std::string, std::string> values_;
};

#endif
