// Launch-shape cache of the autotuner: the winners of the timing runs at prepare, kept
// per GPU and per system structure in a text file that later runs read instead of timing
// again.
//
// File: $CUPSSGB_TUNE_CACHE if set (an empty value or "off" disables the cache), else
// $XDG_CACHE_HOME/cupss_gb300/tune_v1.txt, else $HOME/.cache/cupss_gb300/tune_v1.txt.
// One entry per line, three fields separated by tabs:
//   cupssgb-tune-v1 <key> <value>
// where the key names the GPU, the grid, the batch span and the phase's generated
// update program (see Solver::tune_key) and the value is "name=number" pairs separated by
// spaces.  Lines are only ever appended (one write per line); a later line for the same
// key replaces an earlier one; lines that do not parse are ignored.
#include "tune_cache.h"

#include <fcntl.h>
#include <sys/stat.h>
#include <unistd.h>

#include <cerrno>
#include <cstdlib>
#include <fstream>
#include <mutex>
#include <sstream>

namespace cupssgb {

namespace {
constexpr const char* kTag = "cupssgb-tune-v1";
std::mutex g_mu;

bool make_dirs(const std::string& path) {
  // creates every directory of path's parent
  size_t pos = 0;
  while ((pos = path.find('/', pos + 1)) != std::string::npos) {
    const std::string d = path.substr(0, pos);
    if (mkdir(d.c_str(), 0755) != 0 && errno != EEXIST) return false;
  }
  return true;
}
}  // namespace

std::string tune_cache_path() {
  if (const char* p = std::getenv("CUPSSGB_TUNE_CACHE")) {
    const std::string s(p);
    return (s.empty() || s == "off") ? std::string() : s;
  }
  if (const char* x = std::getenv("XDG_CACHE_HOME"))
    if (*x) return std::string(x) + "/cupss_gb300/tune_v1.txt";
  if (const char* h = std::getenv("HOME"))
    if (*h) return std::string(h) + "/.cache/cupss_gb300/tune_v1.txt";
  return std::string();
}

bool tune_cache_lookup(const std::string& key, std::string* value) {
  const std::string path = tune_cache_path();
  if (path.empty()) return false;
  std::lock_guard<std::mutex> lk(g_mu);
  std::ifstream in(path);
  if (!in) return false;
  std::string line;
  bool found = false;
  while (std::getline(in, line)) {
    const size_t a = line.find('\t');
    if (a == std::string::npos || line.compare(0, a, kTag) != 0) continue;
    const size_t b = line.find('\t', a + 1);
    if (b == std::string::npos) continue;
    if (line.compare(a + 1, b - a - 1, key) != 0) continue;
    *value = line.substr(b + 1);
    found = true;   // keep reading: the last entry wins
  }
  return found;
}

bool tune_cache_store(const std::string& key, const std::string& value) {
  const std::string path = tune_cache_path();
  if (path.empty()) return false;
  if (key.find_first_of("\t\n") != std::string::npos || value.find_first_of("\t\n") != std::string::npos)
    return false;
  std::lock_guard<std::mutex> lk(g_mu);
  if (!make_dirs(path)) return false;
  const std::string line = std::string(kTag) + "\t" + key + "\t" + value + "\n";
  const int fd = open(path.c_str(), O_WRONLY | O_CREAT | O_APPEND, 0644);
  if (fd < 0) return false;
  const ssize_t n = write(fd, line.data(), line.size());
  close(fd);
  return n == (ssize_t)line.size();
}

bool tune_value_get(const std::string& value, const std::string& name, double* out) {
  std::istringstream is(value);
  std::string tok;
  while (is >> tok) {
    const size_t eq = tok.find('=');
    if (eq == std::string::npos || tok.compare(0, eq, name) != 0 || eq != name.size()) continue;
    char* end = nullptr;
    const std::string num = tok.substr(eq + 1);
    const double v = std::strtod(num.c_str(), &end);
    if (end == num.c_str() || *end != '\0') return false;
    *out = v;
    return true;
  }
  return false;
}

uint64_t fnv1a64(const std::string& s) {
  uint64_t h = 0xcbf29ce484222325ull;
  for (unsigned char c : s) {
    h ^= c;
    h *= 0x100000001b3ull;
  }
  return h;
}

}  // namespace cupssgb
