// Luminosity cache: the table of prepareTwoPhotonLumi (src/UpcCrossSection.cpp:463-592)
// kept on disk between processes.
//
// The reference stores twoPhotonLumi.root (twoPhotonLumiPol.root when
// polarized) in the luminosity directory and reuses whatever file is there,
// whatever the nucleus, energy or grid it was made for (:481-491); a lock
// file created with O_CREAT | O_EXCL keeps concurrent generators from
// computing it twice (:466-478), and a generator waits for the lock without a
// limit.  Here the file name carries a 64-bit FNV-1a hash of a key text that
// spells out every input of the table (exact hex-float values), the file
// repeats the full key and a checksum of the payload, and the lock wait is
// bounded: a lock whose process is gone is removed, and a lock still held at
// the limit lets this generator compute without writing.
//
// File layout (host byte order, every field 8-byte aligned):
//   char  magic[8]   = "UPCGLUM1"
//   u32   version    = 1
//   u32   ntab       (1, or 2 for the scalar and pseudoscalar tables)
//   u32   nm, ny
//   u64   key_len    then key_len bytes of key text, zero-padded to 8
//   u64   checksum   FNV-1a 64 over the payload bytes
//   f64   payload[ntab][nm][ny]  (L dm dy, the table of the handle)
#include <errno.h>
#include <fcntl.h>
#include <signal.h>
#include <sys/stat.h>
#include <time.h>
#include <unistd.h>

#include <cstdint>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "upcg_cache.h"

namespace upcg {

namespace {

constexpr char kMagic[8] = {'U', 'P', 'C', 'G', 'L', 'U', 'M', '1'};
constexpr uint32_t kVersion = 1;

uint64_t fnv1a(const void* data, size_t n, uint64_t h = 0xcbf29ce484222325ull) {
  const unsigned char* p = static_cast<const unsigned char*>(data);
  for (size_t i = 0; i < n; ++i) {
    h ^= p[i];
    h *= 0x100000001b3ull;
  }
  return h;
}

bool read_all(FILE* f, void* dst, size_t n) { return fread(dst, 1, n, f) == n; }
bool write_all(FILE* f, const void* src, size_t n) { return fwrite(src, 1, n, f) == n; }

void sleep_ms(int ms) {
  timespec ts{ms / 1000, (long)(ms % 1000) * 1000000L};
  nanosleep(&ts, nullptr);
}

double now_s() {
  timespec ts{};
  clock_gettime(CLOCK_MONOTONIC, &ts);
  return ts.tv_sec + 1e-9 * ts.tv_nsec;
}

// a lock file holds the decimal pid of its owner; false if that process is gone
bool lock_owner_alive(const std::string& lock) {
  FILE* f = fopen(lock.c_str(), "r");
  if (!f) return true;  // vanished or unreadable: let the caller retry
  long pid = 0;
  const int got = fscanf(f, "%ld", &pid);
  fclose(f);
  if (got != 1 || pid <= 0) {
    // no pid yet: being written, unless its owner died between create and write
    struct stat st{};
    return stat(lock.c_str(), &st) != 0 || time(nullptr) - st.st_mtime < 10;
  }
  return !(kill((pid_t)pid, 0) != 0 && errno == ESRCH);
}

}  // namespace

std::string lumi_cache_file_name(const std::string& key) {
  char name[64];
  snprintf(name, sizeof name, "upcg_lumi_%016llx.bin", (unsigned long long)fnv1a(key.data(), key.size()));
  return name;
}

int lumi_cache_read(const std::string& path, const std::string& key, int ntab, int nm, int ny,
                    std::vector<double>& out) {
  FILE* f = fopen(path.c_str(), "rb");
  if (!f) return 0;
  bool ok = true;
  char magic[8];
  uint32_t hdr[4];
  uint64_t klen = 0, sum = 0;
  ok = ok && read_all(f, magic, 8) && std::memcmp(magic, kMagic, 8) == 0;
  ok = ok && read_all(f, hdr, sizeof hdr);
  ok = ok && hdr[0] == kVersion && hdr[1] == (uint32_t)ntab && hdr[2] == (uint32_t)nm &&
       hdr[3] == (uint32_t)ny;
  ok = ok && read_all(f, &klen, 8) && klen == key.size();
  if (ok) {
    std::string k((klen + 7) / 8 * 8, '\0');
    ok = read_all(f, &k[0], k.size()) && std::memcmp(k.data(), key.data(), klen) == 0;
  }
  ok = ok && read_all(f, &sum, 8);
  const size_t n = (size_t)ntab * nm * ny;
  if (ok) {
    out.resize(n);
    ok = read_all(f, out.data(), n * sizeof(double)) && fnv1a(out.data(), n * sizeof(double)) == sum;
    char extra;
    ok = ok && fread(&extra, 1, 1, f) == 0;  // nothing after the payload
  }
  fclose(f);
  return ok ? 1 : 0;
}

int lumi_cache_write(const std::string& path, const std::string& key, int ntab, int nm, int ny,
                     const double* data) {
  // write a private temporary file, then rename it over the target: readers
  // see either the old file or the complete new one
  const std::string tmp = path + ".tmp." + std::to_string((long)getpid());
  FILE* f = fopen(tmp.c_str(), "wb");
  if (!f) return -1;
  const size_t n = (size_t)ntab * nm * ny;
  const uint32_t hdr[4] = {kVersion, (uint32_t)ntab, (uint32_t)nm, (uint32_t)ny};
  const uint64_t klen = key.size();
  std::string kp = key;
  kp.resize((klen + 7) / 8 * 8, '\0');
  const uint64_t sum = fnv1a(data, n * sizeof(double));
  bool ok = write_all(f, kMagic, 8) && write_all(f, hdr, sizeof hdr) && write_all(f, &klen, 8) &&
            write_all(f, kp.data(), kp.size()) && write_all(f, &sum, 8) &&
            write_all(f, data, n * sizeof(double));
  ok = (fflush(f) == 0) && ok;
  ok = (fclose(f) == 0) && ok;
  if (ok) ok = rename(tmp.c_str(), path.c_str()) == 0;
  if (!ok) unlink(tmp.c_str());
  return ok ? 0 : -1;
}

int lumi_lock_acquire(const std::string& lock, double timeout_s) {
  const double t0 = now_s();
  for (;;) {
    const int fd = open(lock.c_str(), O_CREAT | O_EXCL | O_WRONLY, 0644);
    if (fd >= 0) {
      const std::string pid = std::to_string((long)getpid()) + "\n";
      const ssize_t w = write(fd, pid.data(), pid.size());
      (void)w;
      close(fd);
      return 1;
    }
    if (errno != EEXIST) return 0;  // directory not writable: run without a lock
    if (!lock_owner_alive(lock)) {
      unlink(lock.c_str());  // its owner died while holding it
      continue;
    }
    if (now_s() - t0 > timeout_s) return 0;
    sleep_ms(20);
  }
}

void lumi_lock_release(const std::string& lock) { unlink(lock.c_str()); }

}  // namespace upcg
