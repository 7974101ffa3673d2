// CPU oracle -- the random engines, histogram samplers and vector algebra of
// the event loop (TEST INFRASTRUCTURE ONLY).
//
// Shared by the oracle's event loop (oracle_gen.cpp) and by the GSL / ROOT
// stand-ins of refshim/ that the reference's own src/UpcGenerator.cpp is
// compiled against for the generator pin, so that pin checks the reference's
// code around these calls (draw order, cuts, boosts, bins) against the
// oracle's restatement of it.  Each piece restates the published algorithm
// of the library the reference calls:
//   * GSL's mt19937 (gsl_rng_default; gsl_rng_set: seed 0 -> 4357, the
//     standard 32-bit initialisation; gsl_rng_uniform = x / 2^32);
//   * ROOT's TRandomMT64 (the 64-bit Mersenne twister, seeded directly;
//     Rndm = x / 2^64, a zero word redrawn; Uniform(a, b) = a + (b - a) Rndm);
//   * gsl_histogram_pdf_init / gsl_histogram2d_pdf_init (running mean, then
//     the cumulative sum of (bin / mean) / n) and their bin search;
//   * TH1::ComputeIntegral / TH1::GetRandom on uniform bins;
//   * TLorentzVector::Boost, SetVectM, Mag; TVector3::RotateUz, Unit,
//     PseudoRapidity.
#pragma once

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <random>
#include <vector>

namespace uo {

struct GslUniform {  // gsl_rng_default (mt19937) + gsl_rng_uniform
  std::mt19937 e;
  explicit GslUniform(unsigned long s = 0) : e((uint32_t)(s == 0 ? 4357 : s)) {}
  double operator()() { return e() / 4294967296.0; }
};

struct RootMT64 {  // TRandomMT64::Rndm / Uniform
  std::mt19937_64 e;
  explicit RootMT64(uint64_t s = 0) : e(s) {}
  double rndm() {
    for (;;) {
      uint64_t x = e();
      if (x != 0) return x * (1.0 / 18446744073709551616.0);
    }
  }
  double uniform(double lo, double hi) { return lo + (hi - lo) * rndm(); }
};

// gsl_histogram_pdf_init: running mean, then cumulative (bin/mean)/n.
inline std::vector<double> gsl_cdf(const double* bins, size_t n) {
  std::vector<double> sum(n + 1);
  double mean = 0;
  for (size_t i = 0; i < n; i++) mean += (bins[i] - mean) / ((double)(i + 1));
  double s = 0;
  sum[0] = 0;
  for (size_t i = 0; i < n; i++) {
    s += (bins[i] / mean) / n;
    sum[i + 1] = s;
  }
  return sum;
}

// find(): i with sum[i] <= r < sum[i+1]; -1 when r is outside [sum[0], sum[n]).
inline long gsl_find(const std::vector<double>& sum, double r) {
  const size_t n = sum.size() - 1;
  if (r < sum[0] || r >= sum[n]) return -1;
  size_t lo = 0, hi = n;
  while (hi - lo > 1) {
    size_t mid = (hi + lo) / 2;
    if (r >= sum[mid]) lo = mid; else hi = mid;
  }
  return (long)lo;
}

struct Vec4 { double x, y, z, t; };

inline void boost(Vec4& p, double bx, double by, double bz) {  // TLorentzVector::Boost
  double b2 = bx * bx + by * by + bz * bz;
  double gamma = 1.0 / std::sqrt(1.0 - b2);
  double bp = bx * p.x + by * p.y + bz * p.z;
  double gamma2 = b2 > 0 ? (gamma - 1.0) / b2 : 0.0;
  double x = p.x + gamma2 * bp * bx + gamma * bx * p.t;
  double y = p.y + gamma2 * bp * by + gamma * by * p.t;
  double z = p.z + gamma2 * bp * bz + gamma * bz * p.t;
  p.t = gamma * (p.t + bp);
  p.x = x; p.y = y; p.z = z;
}

inline void rotate_uz(Vec4& p, double u1, double u2, double u3) {  // TVector3::RotateUz
  double up = u1 * u1 + u2 * u2;
  if (up) {
    up = std::sqrt(up);
    double px = p.x, py = p.y, pz = p.z;
    p.x = (u1 * u3 * px - u2 * py + u1 * up * pz) / up;
    p.y = (u2 * u3 * px + u1 * py + u2 * up * pz) / up;
    p.z = (u3 * u3 * px - px + u3 * up * pz) / up;
  } else if (u3 < 0.) {
    p.x = -p.x;
    p.z = -p.z;
  }
}

// TVector3::Unit: the components times 1 / |v| (v itself when |v| = 0)
inline void unit3(double x, double y, double z, double u[3]) {
  const double tot2 = x * x + y * y + z * z;
  const double tot = tot2 > 0 ? 1.0 / std::sqrt(tot2) : 1.0;
  u[0] = x * tot;
  u[1] = y * tot;
  u[2] = z * tot;
}

inline double pt_of(const Vec4& p) { return std::sqrt(p.x * p.x + p.y * p.y); }

inline double eta_of(const Vec4& p) {  // TVector3::PseudoRapidity
  double mag = std::sqrt(p.x * p.x + p.y * p.y + p.z * p.z);
  double ct = mag == 0.0 ? 1.0 : p.z / mag;
  if (ct * ct < 1) return -0.5 * std::log((1.0 - ct) / (1.0 + ct));
  if (p.z == 0) return 0;
  return p.z > 0 ? 10e10 : -10e10;
}

inline Vec4 set_vect_m(double x, double y, double z, double m) {  // TLorentzVector::SetVectM
  if (m >= 0) return Vec4{x, y, z, std::sqrt(x * x + y * y + z * z + m * m)};
  return Vec4{x, y, z, std::sqrt(std::max(x * x + y * y + z * z - m * m, 0.))};
}

inline double mag2_of(const Vec4& p) { return p.t * p.t - (p.x * p.x + p.y * p.y + p.z * p.z); }

inline double mag_of(const Vec4& p) {  // TLorentzVector::Mag (negative for space-like)
  const double mm = mag2_of(p);
  return mm < 0.0 ? -std::sqrt(-mm) : std::sqrt(mm);
}

// TH1::ComputeIntegral of bins 1..n: I[0] = 0, I[b] = sum of the first b
// contents, then divided by the total.
inline std::vector<double> th1_integral(const double* content, int n) {
  std::vector<double> I(n + 1, 0.0);
  for (int b = 1; b <= n; ++b) I[b] = I[b - 1] + content[b - 1];
  const double tot = I[n];
  for (int b = 1; b <= n; ++b) I[b] /= tot;
  return I;
}

// TH1::GetRandom on n uniform bins over [xmin, xmax) with integral I and the
// uniform r1: TMath::BinarySearch, then linear inside the bin.
inline double th1_sample(const std::vector<double>& I, int n, double xmin, double xmax,
                         double r1) {
  long ib = (long)(std::lower_bound(I.begin(), I.begin() + n, r1) - I.begin());
  if (!(ib != n && I[ib] == r1)) ib -= 1;
  const double w = (xmax - xmin) / n;
  double x = xmin + ib * w;
  if (r1 > I[ib]) x += w * (r1 - I[ib]) / (I[ib + 1] - I[ib]);
  return x;
}

}  // namespace uo
