// Persistent cache of the stage-kernel autotuner's choices (hg_autotune).
#pragma once
#include <cstddef>
#include <cstdint>
#include <string>

namespace hg {

// A stage kernel (StageKernel) and its shape (DevMesh::stageVariant).
struct TuneChoice {
  int kernel = -1;
  int variant = 0;
};

// The cache file: HG_AUTOTUNE_CACHE when set (empty: no cache), else
// $XDG_CACHE_HOME/hydrograd_gb/autotune.json, else
// $HOME/.cache/hydrograd_gb/autotune.json; "" when there is none.
std::string autotune_cache_path();
// The choice stored under key, if any.
bool autotune_cache_load(const std::string& path, const std::string& key, TuneChoice& out);
// Stores (replaces) the choice under key; the file is rewritten whole and
// renamed into place, so a reader never sees half a file.
bool autotune_cache_store(const std::string& path, const std::string& key, const TuneChoice& c, double ms);
// FNV-1a over n bytes, continuing from h.
uint64_t fnv1a(const void* data, size_t n, uint64_t h = 1469598103934665603ull);

}  // namespace hg
