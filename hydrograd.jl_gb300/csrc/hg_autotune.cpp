// Persistent cache of the stage-kernel autotuner's choices.
//
// The file is a small JSON object written by this code only:
//   {
//    "hydrograd_gb_autotune": 1,
//    "entries": {
//     "<key>": {"kernel": 3, "variant": 0, "ms": 0.0743},
//     ...
//    }
//   }
// one entry per line, keyed by GPU, mesh signature, precision and kernel
// family (hg_capi.cpp, autotune_key), so that a later context on the same
// mesh and GPU reuses the choice without timing the candidates again.
#include "hg_autotune.hpp"

#include <cerrno>
#include <cstdio>
#include <cstdlib>
#include <map>
#include <sys/stat.h>
#include <unistd.h>

namespace hg {

namespace {

struct Entry {
  TuneChoice c;
  double ms = 0.0;
};

// Parses one entry line: "<key>": {"kernel": K, "variant": V, "ms": T}
bool parse_line(const std::string& line, std::string& key, Entry& e) {
  const size_t q0 = line.find('"');
  if (q0 == std::string::npos) return false;
  const size_t q1 = line.find('"', q0 + 1);
  if (q1 == std::string::npos) return false;
  key = line.substr(q0 + 1, q1 - q0 - 1);
  const size_t k = line.find("\"kernel\":", q1);
  const size_t v = line.find("\"variant\":", q1);
  if (k == std::string::npos || v == std::string::npos) return false;
  e.c.kernel = std::atoi(line.c_str() + k + 9);
  e.c.variant = std::atoi(line.c_str() + v + 10);
  const size_t t = line.find("\"ms\":", q1);
  e.ms = t == std::string::npos ? 0.0 : std::atof(line.c_str() + t + 5);
  return e.c.kernel >= 0;
}

std::map<std::string, Entry> read_all(const std::string& path) {
  std::map<std::string, Entry> out;
  FILE* f = std::fopen(path.c_str(), "r");
  if (!f) return out;
  char buf[1024];
  while (std::fgets(buf, sizeof(buf), f)) {
    std::string key;
    Entry e;
    const std::string line(buf);
    if (line.find("\"kernel\":") != std::string::npos && parse_line(line, key, e)) out[key] = e;
  }
  std::fclose(f);
  return out;
}

// mkdir -p of the file's directory.
void make_dirs(const std::string& path) {
  for (size_t i = 1; i < path.size(); ++i)
    if (path[i] == '/') {
      const std::string d = path.substr(0, i);
      if (::mkdir(d.c_str(), 0755) != 0 && errno != EEXIST) return;
    }
}

}  // namespace

std::string autotune_cache_path() {
  if (const char* e = std::getenv("HG_AUTOTUNE_CACHE")) return std::string(e);
  if (const char* x = std::getenv("XDG_CACHE_HOME"))
    if (*x) return std::string(x) + "/hydrograd_gb/autotune.json";
  if (const char* h = std::getenv("HOME"))
    if (*h) return std::string(h) + "/.cache/hydrograd_gb/autotune.json";
  return std::string();
}

bool autotune_cache_load(const std::string& path, const std::string& key, TuneChoice& out) {
  if (path.empty()) return false;
  const auto all = read_all(path);
  const auto it = all.find(key);
  if (it == all.end()) return false;
  out = it->second.c;
  return true;
}

bool autotune_cache_store(const std::string& path, const std::string& key, const TuneChoice& c, double ms) {
  if (path.empty()) return false;
  auto all = read_all(path);
  all[key] = Entry{c, ms};
  make_dirs(path);
  const std::string tmp = path + ".tmp." + std::to_string((long)::getpid());
  FILE* f = std::fopen(tmp.c_str(), "w");
  if (!f) return false;
  std::fprintf(f, "{\n \"hydrograd_gb_autotune\": 1,\n \"entries\": {\n");
  size_t i = 0;
  for (const auto& kv : all) {
    std::fprintf(f, "  \"%s\": {\"kernel\": %d, \"variant\": %d, \"ms\": %.6f}%s\n", kv.first.c_str(),
                 kv.second.c.kernel, kv.second.c.variant, kv.second.ms, ++i < all.size() ? "," : "");
  }
  std::fprintf(f, " }\n}\n");
  const bool ok = std::fclose(f) == 0;
  if (!ok || std::rename(tmp.c_str(), path.c_str()) != 0) {
    std::remove(tmp.c_str());
    return false;
  }
  return true;
}

uint64_t fnv1a(const void* data, size_t n, uint64_t h) {
  const unsigned char* p = static_cast<const unsigned char*>(data);
  for (size_t i = 0; i < n; ++i) {
    h ^= p[i];
    h *= 1099511628211ull;
  }
  return h;
}

}  // namespace hg
