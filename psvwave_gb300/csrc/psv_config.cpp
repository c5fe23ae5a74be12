// INI reading and validation of a P-SV model configuration.
#include "psv_config.hpp"

#include <algorithm>
#include <cctype>
#include <cmath>
#include <cstdlib>
#include <fstream>
#include <map>

#include "../../include/psvwave.h"

namespace psv {
namespace {

std::string trim(const std::string &s) {
  size_t a = 0, b = s.size();
  while (a < b && std::isspace(static_cast<unsigned char>(s[a]))) ++a;
  while (b > a && std::isspace(static_cast<unsigned char>(s[b - 1]))) --b;
  return s.substr(a, b - a);
}

std::string lower(std::string s) {
  for (auto &ch : s) ch = static_cast<char>(std::tolower(static_cast<unsigned char>(ch)));
  return s;
}

// Position of the first character of `stops`, or of a ';' that follows
// whitespace (an inline comment), or npos.
size_t find_stop(const std::string &s, const char *stops) {
  bool after_space = false;
  for (size_t i = 0; i < s.size(); ++i) {
    const char ch = s[i];
    for (const char *q = stops; *q; ++q)
      if (ch == *q) return i;
    if (after_space && ch == ';') return i;
    after_space = std::isspace(static_cast<unsigned char>(ch)) != 0;
  }
  return std::string::npos;
}

class Ini {
 public:
  explicit Ini(const std::string &path) {
    std::ifstream in(path);
    if (!in.good()) throw Error(PSV_ERR_INVALID_ARGUMENT, "Can't load .ini file.");
    std::string line, section;
    while (std::getline(in, line)) {
      std::string s = trim(line);
      if (s.empty() || s[0] == ';' || s[0] == '#') continue;
      if (s[0] == '[') {
        size_t e = find_stop(s.substr(1), "]");
        if (e != std::string::npos && s[1 + e] == ']') section = trim(s.substr(1, e));
        continue;
      }
      size_t e = find_stop(s, "=:");
      if (e == std::string::npos || (s[e] != '=' && s[e] != ':')) continue;
      std::string name = trim(s.substr(0, e));
      std::string value = trim(s.substr(e + 1));
      size_t cut = find_stop(value, "");
      if (cut != std::string::npos) value = trim(value.substr(0, cut));
      std::string key = lower(section) + "=" + lower(name);
      auto it = kv_.find(key);
      if (it == kv_.end())
        kv_[key] = value;
      else
        it->second += "\n" + value;
    }
  }
  std::string str(const char *sec, const char *name) const {
    auto it = kv_.find(lower(sec) + "=" + lower(name));
    return it == kv_.end() ? std::string() : it->second;
  }
  // Longest integer prefix (base prefixes as strtol with base 0); 0 if none.
  long integer(const char *sec, const char *name) const {
    std::string v = str(sec, name);
    char *end = nullptr;
    long x = std::strtol(v.c_str(), &end, 0);
    return end > v.c_str() ? x : 0;
  }
  double real(const char *sec, const char *name) const {
    std::string v = str(sec, name);
    char *end = nullptr;
    double x = std::strtod(v.c_str(), &end);
    return end > v.c_str() ? x : 0.0;
  }

 private:
  std::map<std::string, std::string> kv_;
};

std::string without_space(const std::string &s) {
  std::string out;
  for (char ch : s)
    if (!std::isspace(static_cast<unsigned char>(ch))) out += ch;
  return out;
}

// "{a, b, c}" -> numbers: everything between the first character and the
// first '}' split on ',' and read as doubles (src/fdModel.cpp:1574-1599).
std::vector<double> parse_list(const std::string &raw) {
  std::string s = without_space(raw);
  size_t close = s.find('}');
  if (close != std::string::npos) s.erase(close);
  if (!s.empty()) s.erase(0, 1);
  std::vector<double> out;
  size_t start = 0;
  for (;;) {
    size_t comma = s.find(',', start);
    out.push_back(std::atof(s.substr(start, comma - start).c_str()));
    if (comma == std::string::npos) break;
    start = comma + 1;
  }
  return out;
}

// "{{a, b}, {c}}" -> groups (src/fdModel.cpp:1601-1659).
std::vector<std::vector<int>> parse_groups(const std::string &raw) {
  std::string s = without_space(raw);
  s.erase(0, std::min<size_t>(2, s.size()));
  std::vector<std::vector<int>> groups;
  size_t start = 0;
  for (;;) {
    size_t sep = s.find("},{", start);
    size_t end = sep;
    if (sep == std::string::npos) end = s.find("}};", start);
    std::string body = s.substr(start, end == std::string::npos ? std::string::npos : end - start);
    std::vector<int> g;
    size_t p = 0;
    for (;;) {
      size_t comma = body.find(',', p);
      g.push_back(static_cast<int>(std::atof(body.substr(p, comma - p).c_str())));
      if (comma == std::string::npos) break;
      p = comma + 1;
    }
    groups.push_back(g);
    if (sep == std::string::npos) break;
    start = sep + 3;
  }
  return groups;
}

std::vector<int> to_int(const std::vector<double> &v) {
  std::vector<int> out;
  for (double x : v) out.push_back(static_cast<int>(x));
  return out;
}

}  // namespace

Config read_ini(const std::string &path) {
  Ini ini(path);
  Config c;
  c.nt = static_cast<int>(ini.integer("domain", "nt"));
  c.nx_inner = static_cast<int>(ini.integer("domain", "nx_inner"));
  c.nz_inner = static_cast<int>(ini.integer("domain", "nz_inner"));
  c.nx_inner_boundary = static_cast<int>(ini.integer("domain", "nx_inner_boundary"));
  c.nz_inner_boundary = static_cast<int>(ini.integer("domain", "nz_inner_boundary"));
  c.dx = ini.real("domain", "dx");
  c.dz = ini.real("domain", "dz");
  c.dt = ini.real("domain", "dt");
  c.np_boundary = static_cast<int>(ini.integer("boundary", "np_boundary"));
  c.np_factor = ini.real("boundary", "np_factor");
  c.scalar_rho = ini.real("medium", "scalar_rho");
  c.scalar_vp = ini.real("medium", "scalar_vp");
  c.scalar_vs = ini.real("medium", "scalar_vs");
  c.npx = static_cast<int>(ini.integer("basis", "npx"));
  c.npz = static_cast<int>(ini.integer("basis", "npz"));
  c.peak_frequency = ini.real("sources", "peak_frequency");
  c.source_timeshift = ini.real("sources", "source_timeshift");
  c.delay_cycles_per_shot = ini.real("sources", "delay_cycles_per_shot");
  c.n_sources = static_cast<int>(ini.integer("sources", "n_sources"));
  c.n_shots = static_cast<int>(ini.integer("sources", "n_shots"));
  c.ix_sources = to_int(parse_list(ini.str("sources", "ix_sources")));
  c.iz_sources = to_int(parse_list(ini.str("sources", "iz_sources")));
  c.moment_angles = parse_list(ini.str("sources", "moment_angles"));
  c.shots = parse_groups(ini.str("sources", "which_source_to_fire_in_which_shot"));
  c.nr = static_cast<int>(ini.integer("receivers", "nr"));
  c.ix_receivers = to_int(parse_list(ini.str("receivers", "ix_receivers")));
  c.iz_receivers = to_int(parse_list(ini.str("receivers", "iz_receivers")));
  c.snapshot_interval = static_cast<int>(ini.integer("inversion", "snapshot_interval"));
  c.observed_data_folder = ini.str("output", "observed_data_folder");
  c.stf_folder = ini.str("output", "stf_folder");
  return c;
}

Geometry validate(const Config &c) {
  auto bad = [](int code, const std::string &m) { throw Error(code, m); };
  if (c.nt <= 0) bad(PSV_ERR_INVALID_ARGUMENT, "nt must be positive");
  if (c.nx_inner <= 0 || c.nz_inner <= 0)
    bad(PSV_ERR_INVALID_ARGUMENT, "nx_inner and nz_inner must be positive");
  if (c.np_boundary < 0) bad(PSV_ERR_INVALID_ARGUMENT, "np_boundary must not be negative");
  if (c.nx_inner_boundary < 0 || c.nz_inner_boundary < 0)
    bad(PSV_ERR_INVALID_ARGUMENT, "inner boundaries must not be negative");
  if (!(c.dx > 0) || !(c.dz > 0) || !(c.dt > 0))
    bad(PSV_ERR_INVALID_ARGUMENT, "dx, dz and dt must be positive");
  if (!(c.peak_frequency > 0)) bad(PSV_ERR_INVALID_ARGUMENT, "peak_frequency must be positive");
  if (c.snapshot_interval <= 0) bad(PSV_ERR_INVALID_ARGUMENT, "snapshot_interval must be positive");
  if (c.npx <= 0 || c.npz <= 0) bad(PSV_ERR_INVALID_ARGUMENT, "npx and npz must be positive");
  if (c.n_sources < 0 || c.nr < 0 || c.n_shots < 0)
    bad(PSV_ERR_INVALID_ARGUMENT, "n_sources, n_shots and nr must not be negative");

  Geometry g;
  g.nx = c.nx_inner + 2 * c.np_boundary;
  g.nz = c.nz_inner + 2 * c.np_boundary;
  if (static_cast<long long>(g.nx) * g.nz > (1LL << 31) - 1)
    bad(PSV_ERR_INVALID_ARGUMENT, "grid larger than 2^31 points");
  g.nx_free = c.nx_inner - 2 * c.nx_inner_boundary;
  g.nz_free = c.nz_inner - 2 * c.nz_inner_boundary;
  if (g.nx_free < 0 || g.nz_free < 0)
    bad(PSV_ERR_INVALID_ARGUMENT, "inner boundaries leave a negative free region");
  // The reference asserts divisibility of the free region by the basis
  // (src/fdModel.cpp:404-405); here it is a recoverable error.
  if (g.nx_free % c.npx != 0 || g.nz_free % c.npz != 0)
    bad(PSV_ERR_INVALID_ARGUMENT, "free-parameter region is not divisible by the basis (npx, npz)");
  g.free_parameters = 3 * g.nx_free * g.nz_free / (c.npx * c.npz);

  if (static_cast<int>(c.ix_sources.size()) != c.n_sources ||
      static_cast<int>(c.iz_sources.size()) != c.n_sources ||
      static_cast<int>(c.moment_angles.size()) != c.n_sources)
    bad(PSV_ERR_INVALID_ARGUMENT,
        "Dimension mismatch between n_sources and sources.ix_sources, sources.iz_sources or "
        "sources.moment_angles");
  if (static_cast<int>(c.shots.size()) != c.n_shots)
    bad(PSV_ERR_INVALID_ARGUMENT,
        "Mismatch between n_shots and sources.which_source_to_fire_in_which_shot");
  int total = 0;
  for (const auto &s : c.shots) total += static_cast<int>(s.size());
  if (total != c.n_sources)
    bad(PSV_ERR_INVALID_ARGUMENT,
        "Mismatch between n_sources and sources.which_source_to_fire_in_which_shot.");
  for (const auto &s : c.shots)
    for (int id : s)
      if (id < 0 || id >= c.n_sources)
        bad(PSV_ERR_INVALID_ARGUMENT, "which_source_to_fire_in_which_shot names an unknown source");
  if (static_cast<int>(c.ix_receivers.size()) != c.nr ||
      static_cast<int>(c.iz_receivers.size()) != c.nr)
    bad(PSV_ERR_INVALID_ARGUMENT,
        "Mismatch between nr and receivers.ix_receivers or receivers.iz_receivers");

  // Bounds: every source writes a 3x3 neighbourhood, every receiver reads
  // one point. The reference does not check these; out-of-grid positions
  // would address memory outside the fields.
  for (int i = 0; i < c.n_sources; ++i) {
    int x = c.ix_sources[i] + c.np_boundary, z = c.iz_sources[i] + c.np_boundary;
    if (x < 1 || x > g.nx - 2 || z < 1 || z > g.nz - 2)
      bad(PSV_ERR_INVALID_ARGUMENT, "source " + std::to_string(i) + " lies outside the grid");
  }
  for (int i = 0; i < c.nr; ++i) {
    int x = c.ix_receivers[i] + c.np_boundary, z = c.iz_receivers[i] + c.np_boundary;
    if (x < 0 || x >= g.nx || z < 0 || z >= g.nz)
      bad(PSV_ERR_INVALID_ARGUMENT, "receiver " + std::to_string(i) + " lies outside the grid");
  }

  g.alpha = 1.0 / c.peak_frequency;
  g.snapshots = c.nt / c.snapshot_interval;
  if (c.nt % c.snapshot_interval != 0)
    bad(PSV_ERR_LENGTH, "Snapshot interval and size of accumulator don't match!");
  g.fx0 = c.np_boundary + c.nx_inner_boundary;
  g.fx1 = c.np_boundary + c.nx_inner - c.nx_inner_boundary;
  g.fz0 = c.np_boundary + c.nz_inner_boundary;
  g.fz1 = c.np_boundary + c.nz_inner - c.nz_inner_boundary;
  return g;
}

}  // namespace psv
