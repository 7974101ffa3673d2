// ROOT macro: a luminosity cache file of upcgen_gb300 -> the reference's
// twoPhotonLumi.root layout (src/UpcCrossSection.cpp:496-503, 556-585):
// TH2D "hD2LDMDY" (or "hD2LDMDY_s" and "hD2LDMDY_p" for a polarized table)
// with nm bins over [mmin, mmax] and ny bins over [ymin, ymax], bin
// (im + 1, iy + 1) = L dm dy of cell (im, iy).
//
//   root -b -q 'lumi_cache_to_root.C("upcg_lumi_0123456789abcdef.bin", "twoPhotonLumi.root")'
//
// The file layout is documented in upcgen_gb300/lumi_cache.py.
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <string>
#include <vector>

#include "TFile.h"
#include "TH2D.h"

namespace {
// "; <ax> [<hex lo>, <hex hi>] bins <n>" in the key text
bool lumi_cache_axis(const std::string& key, const char* ax, double& lo, double& hi, int& n) {
  const std::string tag = std::string("; ") + ax + " [";
  const size_t p = key.find(tag);
  if (p == std::string::npos) return false;
  const char* s = key.c_str() + p + tag.size();
  char* e = nullptr;
  lo = std::strtod(s, &e);
  if (e == s || std::strncmp(e, ", ", 2) != 0) return false;
  s = e + 2;
  hi = std::strtod(s, &e);
  if (e == s || std::strncmp(e, "] bins ", 7) != 0) return false;
  n = std::atoi(e + 7);
  return n > 0;
}
}  // namespace

int lumi_cache_to_root(const char* cache, const char* out = "twoPhotonLumi.root") {
  std::ifstream in(cache, std::ios::binary);
  char magic[8];
  uint32_t hdr[4];
  uint64_t klen = 0, sum = 0;
  if (!in.read(magic, 8) || std::memcmp(magic, "UPCGLUM1", 8) != 0) {
    std::printf("%s: not a luminosity cache file\n", cache);
    return 1;
  }
  if (!in.read(reinterpret_cast<char*>(hdr), sizeof hdr) || hdr[0] != 1) {
    std::printf("%s: unsupported cache version\n", cache);
    return 1;
  }
  const int ntab = (int)hdr[1], nm = (int)hdr[2], ny = (int)hdr[3];
  in.read(reinterpret_cast<char*>(&klen), 8);
  std::string key((klen + 7) / 8 * 8, '\0');
  in.read(&key[0], (std::streamsize)key.size());
  key.resize(klen);
  in.read(reinterpret_cast<char*>(&sum), 8);
  std::vector<double> v((size_t)ntab * nm * ny);
  if (!in.read(reinterpret_cast<char*>(v.data()), (std::streamsize)(v.size() * sizeof(double)))) {
    std::printf("%s: truncated\n", cache);
    return 1;
  }
  uint64_t h = 0xcbf29ce484222325ull;  // FNV-1a 64 of the payload
  const unsigned char* b = reinterpret_cast<const unsigned char*>(v.data());
  for (size_t i = 0; i < v.size() * sizeof(double); ++i) h = (h ^ b[i]) * 0x100000001b3ull;
  double mlo, mhi, ylo, yhi;
  int nmk, nyk;
  if (h != sum || !lumi_cache_axis(key, "m", mlo, mhi, nmk) ||
      !lumi_cache_axis(key, "y", ylo, yhi, nyk) || nmk != nm || nyk != ny) {
    std::printf("%s: corrupted\n", cache);
    return 1;
  }
  TFile f(out, "recreate");
  const char* names[2] = {ntab == 1 ? "hD2LDMDY" : "hD2LDMDY_s", "hD2LDMDY_p"};
  for (int t = 0; t < ntab; ++t) {
    TH2D hist(names[t], "", nm, mlo, mhi, ny, ylo, yhi);
    for (int im = 0; im < nm; ++im)
      for (int iy = 0; iy < ny; ++iy)
        hist.SetBinContent(im + 1, iy + 1, v[((size_t)t * nm + im) * ny + iy]);
    hist.Write();
  }
  f.Close();
  return 0;
}
