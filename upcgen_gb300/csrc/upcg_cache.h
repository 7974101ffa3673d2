// Luminosity cache files (upcg_cache.cpp): host code only.
#pragma once

#include <string>
#include <vector>

namespace upcg {

// "upcg_lumi_<FNV-1a 64 of key, 16 hex digits>.bin"
std::string lumi_cache_file_name(const std::string& key);
// 1 and the payload [ntab][nm][ny] in out when path holds a complete file for
// exactly this key and shape, else 0
int lumi_cache_read(const std::string& path, const std::string& key, int ntab, int nm, int ny,
                    std::vector<double>& out);
// 0 on success; written to a temporary file and renamed over path
int lumi_cache_write(const std::string& path, const std::string& key, int ntab, int nm, int ny,
                     const double* data);
// 1 when this process holds the lock file ("<host> <pid>"), 0 when it could
// not be had within timeout_s (or the directory refuses it); a lock of this
// host whose owner process is gone is taken over, one of another host waited for
int lumi_lock_acquire(const std::string& lock, double timeout_s);
// removes the lock file if it still names this process
void lumi_lock_release(const std::string& lock);

}  // namespace upcg
