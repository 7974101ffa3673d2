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
// bounded.  A lock names its owner as "<host> <pid>": a lock of this host
// whose process is gone is taken over (renamed away, never unlinked blind), a
// lock of another host is waited for, a lock still held at the limit lets
// this generator compute without writing, and a generator removes the lock
// only while it still names it.  Temporary files carry the host and pid too.
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
#include <cstdlib>
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

// This process as a lock owner: "<host> <pid>" (host name reduced to
// [A-Za-z0-9.-], so that it is one token).
std::string owner_id() {
  char host[256] = {0};
  if (gethostname(host, sizeof host - 1) != 0) host[0] = 0;
  std::string h;
  for (const char* c = host; *c; ++c)
    h += ((*c >= 'a' && *c <= 'z') || (*c >= 'A' && *c <= 'Z') || (*c >= '0' && *c <= '9') ||
          *c == '.' || *c == '-')
             ? *c
             : '_';
  if (h.empty()) h = "unknown-host";
  return h + " " + std::to_string((long)getpid());
}

std::string host_of(const std::string& id) { return id.substr(0, id.find(' ')); }

bool read_text(const std::string& path, std::string& out) {
  FILE* f = fopen(path.c_str(), "r");
  if (!f) return false;
  char buf[512];
  const size_t n = fread(buf, 1, sizeof buf - 1, f);
  fclose(f);
  out.assign(buf, n);
  while (!out.empty() && (out.back() == '\n' || out.back() == '\r')) out.pop_back();
  return true;
}

// A lock file holds "<host> <pid>" of its owner (a bare "<pid>" is read as a
// lock of this host).  False only when the owner is known to be gone: a lock
// of this host whose process no longer exists, or one left without an owner
// for more than 10 s.  A lock of another host (a shared luminosity
// directory) counts as alive: its process cannot be checked from here, so
// the waiter's time limit decides.  *content gets the text judged.
bool lock_owner_alive(const std::string& lock, std::string* content) {
  std::string txt;
  if (!read_text(lock, txt)) return true;  // vanished or unreadable: let the caller retry
  *content = txt;
  std::string host = host_of(owner_id()), pid_s = txt;
  const size_t sp = txt.find(' ');
  if (sp != std::string::npos) {
    host = txt.substr(0, sp);
    pid_s = txt.substr(sp + 1);
  }
  char* end = nullptr;
  const long pid = pid_s.empty() ? 0 : strtol(pid_s.c_str(), &end, 10);
  if (pid <= 0 || (end && *end)) {
    // no owner yet: being written, unless its owner died between create and write
    struct stat st{};
    return stat(lock.c_str(), &st) != 0 || time(nullptr) - st.st_mtime < 10;
  }
  if (host != host_of(owner_id())) return true;
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
  std::string id = owner_id();
  id[id.find(' ')] = '.';
  const std::string tmp = path + ".tmp." + id;
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
  const std::string me = owner_id();
  for (;;) {
    const int fd = open(lock.c_str(), O_CREAT | O_EXCL | O_WRONLY, 0644);
    if (fd >= 0) {
      const std::string line = me + "\n";
      const ssize_t w = write(fd, line.data(), line.size());
      (void)w;
      close(fd);
      return 1;
    }
    if (errno != EEXIST) return 0;  // directory not writable: run without a lock
    std::string dead;
    if (!lock_owner_alive(lock, &dead)) {
      // Take the dead lock out of the way by renaming it to a name of our own
      // (of two waiters only one rename finds it).  If what was moved is not
      // the text judged dead, a new owner took the lock meanwhile: put it
      // back (link fails if yet another lock is there) and drop the copy.
      std::string grave_id = me;
      grave_id[grave_id.find(' ')] = '.';
      const std::string grave = lock + ".stale." + grave_id;
      if (rename(lock.c_str(), grave.c_str()) == 0) {
        std::string moved;
        if (read_text(grave, moved) && moved != dead) {
          const int rl = link(grave.c_str(), lock.c_str());
          (void)rl;
        }
        unlink(grave.c_str());
      }
      continue;
    }
    if (now_s() - t0 > timeout_s) return 0;
    sleep_ms(20);
  }
}

// Removes the lock only while it still names this process.
void lumi_lock_release(const std::string& lock) {
  std::string txt;
  if (read_text(lock, txt) && txt == owner_id()) unlink(lock.c_str());
}

}  // namespace upcg
