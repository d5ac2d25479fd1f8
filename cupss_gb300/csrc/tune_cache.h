// Launch-shape cache of the autotuner (tune_cache.cpp describes the file).
#pragma once
#include <cstdint>
#include <string>

namespace cupssgb {

// The cache file, or "" when the cache is off.
std::string tune_cache_path();
// The value of the last entry for key; false when there is none (or no cache).
bool tune_cache_lookup(const std::string& key, std::string* value);
// Appends an entry; false when the cache is off or the file cannot be written.
bool tune_cache_store(const std::string& key, const std::string& value);
// Reads "name=number" from a value string.
bool tune_value_get(const std::string& value, const std::string& name, double* out);
uint64_t fnv1a64(const std::string& s);

}  // namespace cupssgb
